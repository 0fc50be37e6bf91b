"""The synthetic-input layer on the CPU: the .egr, batch-file and MIS-file
formats (the reference's own file formats: README "File formats",
core/FlashGraph.h:108-169 for .egr, core/cli_setup.h:66-82 for batch lines),
the graph families' invariants, and the toggle streams' contracts (deletes of
current edges, inserts of non-adjacent pairs, the requested split)."""
import os

import numpy as np
import pytest

from misfit_gb300 import workloads as W


def _edge_set(n, nindex, nlist):
    lo, hi = W.undirected_pairs(n, nindex, nlist)
    return set((lo * n + hi).tolist())


def _check_csr(n, nindex, nlist):
    """Symmetric, rows sorted ascending, no self-loops, no duplicates."""
    nindex = np.asarray(nindex, np.int64)
    nlist = np.asarray(nlist, np.int64)
    assert nindex.size == n + 1 and nindex[0] == 0 and nindex[-1] == nlist.size
    assert np.all(np.diff(nindex) >= 0)
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(nindex))
    assert np.all((nlist >= 0) & (nlist < n))
    assert not np.any(src == nlist)
    key = src * n + nlist
    assert np.all(key[1:] > key[:-1])                    # sorted rows, no duplicates
    rev = np.sort(nlist * n + src)
    assert np.array_equal(rev, key)                      # every (a, b) has its (b, a)


@pytest.mark.parametrize("wide", [False, True])
def test_egr_round_trip(tmp_path, wide):
    nindex, nlist = W.er_graph(300, 6.0, 5)
    p = str(tmp_path / "g.egr")
    W.write_egr(p, 300, nindex, nlist, wide=wide)
    n, ni, nl, w = W.read_egr(p)
    assert (n, w) == (300, wide)
    assert np.array_equal(ni, nindex) and np.array_equal(nl, nlist)
    # header layout: n, then the entry count or the -1 sentinel and a 64-bit count
    head = np.fromfile(p, dtype="<i4", count=2)
    assert head[0] == 300 and head[1] == (-1 if wide else nlist.size)
    size = os.path.getsize(p)
    assert size == (16 + 8 * 301 if wide else 8 + 4 * 301) + 4 * nlist.size


def test_egr_truncated_file_is_refused(tmp_path):
    nindex, nlist = W.er_graph(50, 4.0, 6)
    p = str(tmp_path / "g.egr")
    W.write_egr(p, 50, nindex, nlist)
    data = open(p, "rb").read()
    with open(p, "wb") as f:
        f.write(data[:-4])
    with pytest.raises(ValueError):
        W.read_egr(p)


def test_csr_from_pairs_drops_loops_and_duplicates():
    u = np.array([0, 1, 1, 2, 3, 3, 0])
    v = np.array([1, 0, 1, 3, 2, 0, 3])
    nindex, nlist = W.csr_from_pairs(4, u, v)
    _check_csr(4, nindex, nlist)
    assert _edge_set(4, nindex, nlist) == {0 * 4 + 1, 2 * 4 + 3, 0 * 4 + 3}


@pytest.mark.parametrize("family", ["er", "rmat", "rgg"])
def test_graph_families_are_symmetric_sorted_simple(family):
    if family == "er":
        n = 2000
        nindex, nlist = W.er_graph(n, 8.0, 1)
        assert nlist.size == 2 * 8000                    # exactly m = n*avg/2 undirected edges
    elif family == "rmat":
        n, (nindex, nlist) = W.rmat_graph(11, 8, 2)
    else:
        n = 3000
        nindex, nlist = W.rgg_graph(n, 10.0, 3)
        assert 7.0 < nlist.size / n < 13.0               # mean degree near the request
    _check_csr(n, nindex, nlist)


def test_graph_families_are_seeded():
    a = W.er_graph(500, 5.0, 9)
    b = W.er_graph(500, 5.0, 9)
    c = W.er_graph(500, 5.0, 10)
    assert np.array_equal(a[1], b[1]) and not np.array_equal(a[1], c[1])
    _, (x0, x1) = W.rmat_graph(9, 4, 4)
    _, (y0, y1) = W.rmat_graph(9, 4, 4)
    assert np.array_equal(x0, y0) and np.array_equal(x1, y1)


def test_rmat_is_skewed():
    n, (nindex, nlist) = W.rmat_graph(12, 8, 7)
    deg = np.diff(nindex)
    assert deg.max() > 20 * max(1.0, deg.mean())       # hubs, as a=.57 gives
    assert deg[: n // 16].sum() > deg[-(n // 16):].sum()  # low ids carry the mass


def test_torch_generators_on_cpu_give_valid_graphs():
    torch = pytest.importorskip("torch")
    n, (nindex, nlist) = W.rmat_graph_torch(10, 8, 3, device="cpu")
    _check_csr(n, nindex, nlist)
    n2, (m0, m1) = W.rmat_graph_torch(10, 8, 3, device="cpu")
    assert np.array_equal(nindex, m0) and np.array_equal(nlist, m1)
    ri, rl = W.rgg_graph_torch(2000, 12.0, 5, device="cpu")
    _check_csr(2000, ri, rl)
    assert 8.0 < rl.size / 2000 < 16.0
    del torch


@pytest.mark.parametrize("endpoints", ["uniform", "preferential", "low_degree"])
def test_toggle_stream_tracks_the_nominal_graph(endpoints):
    """Every delete is an edge of the graph as it stands after the earlier
    batches, every insert a non-adjacent pair; the split is as requested;
    no pair repeats within a batch."""
    n = 400
    nindex, nlist = W.er_graph(n, 10.0, 11)
    ts = W.ToggleStream(n, nindex, nlist, 12)
    edges = _edge_set(n, nindex, nlist)
    for b in range(6):
        u, v, ins = ts.next_batch(300, delete_frac=0.4, endpoints=endpoints, with_flags=True)
        assert u.size == 300 and int((ins == 0).sum()) == 120
        assert not np.any(u == v)
        key = np.minimum(u, v).astype(np.int64) * n + np.maximum(u, v)
        assert np.unique(key).size == key.size
        for k, f in zip(key.tolist(), ins.tolist()):
            if f:
                assert k not in edges
                edges.add(k)
            else:
                assert k in edges
                edges.remove(k)
        assert ts.num_edges == len(edges)
    if endpoints == "preferential":
        deg = np.diff(nindex)
        u, v, ins = ts.next_batch(2000, delete_frac=0.0, endpoints=endpoints, with_flags=True)
        assert deg[np.concatenate([u, v])].mean() > deg.mean()


@pytest.mark.parametrize("endpoints", ["uniform", "preferential", "low_degree"])
def test_device_toggles_on_cpu(endpoints):
    """DeviceToggles (run here with torch on the CPU): deletes are distinct
    base edges, inserts distinct non-adjacent pairs, the split as asked."""
    pytest.importorskip("torch")
    n, (nindex, nlist) = W.rmat_graph(10, 8, 21)
    edges = _edge_set(n, nindex, nlist)
    dt = W.DeviceToggles(nindex, nlist, 22, device="cpu")
    u, v, ins = dt.next_batch(500, delete_frac=0.5, endpoints=endpoints)
    assert u.dtype == np.int32 and v.dtype == np.int32 and ins.dtype == np.uint8
    assert u.size == 500 and int((ins == 0).sum()) == 250
    assert not np.any(u == v)
    key = np.minimum(u, v).astype(np.int64) * n + np.maximum(u, v)
    assert np.unique(key).size == key.size
    for k, f in zip(key.tolist(), ins.tolist()):
        assert (k in edges) == (f == 0)
    if endpoints == "preferential":
        deg = np.diff(nindex)
        assert deg[np.concatenate([u[ins == 1], v[ins == 1]])].mean() > 2 * deg.mean()


def test_batch_and_mis_files_round_trip(tmp_path):
    u = np.array([0, 5, 9], np.int64)
    v = np.array([3, 2, 0], np.int64)
    folder = str(tmp_path / "batches")
    W.write_batch_folder(folder, [(u, v), (v, u)])
    assert sorted(os.listdir(folder)) == ["1.mtx", "2.mtx"]
    assert open(os.path.join(folder, "1.mtx")).read() == "1 4\n6 3\n10 1\n"   # 1-indexed
    ru, rv = W.read_batch_file(os.path.join(folder, "2.mtx"))
    assert np.array_equal(ru, v) and np.array_equal(rv, u)
    # comment lines and lines without two integers are skipped
    p = str(tmp_path / "c.mtx")
    with open(p, "w") as f:
        f.write("%%MatrixMarket matrix coordinate pattern symmetric\n% comment\n\n7\n2 8\n")
    ru, rv = W.read_batch_file(p)
    assert list(ru) == [1] and list(rv) == [7]
    mis = np.zeros(12, np.uint8)
    mis[[0, 4, 11]] = 1
    q = str(tmp_path / "mis.txt")
    W.write_mis_file(q, mis)
    assert open(q).read() == "1\n5\n12\n"
    assert np.array_equal(W.read_mis_file(q, 12), mis)
    empty = str(tmp_path / "empty.mtx")
    W.write_batch_file(empty, [], [])
    ru, rv = W.read_batch_file(empty)
    assert ru.size == 0 and rv.size == 0
