"""GPU path (libmisfit_gb through its C-ABI) against the oracle and the
golden vectors.  Integer work: every comparison is bit-exact."""
import hashlib

import numpy as np
import pytest

import oracle as O
from misfit_gb300 import native
from misfit_gb300 import workloads as W
from tests import _golden as G

pytestmark = pytest.mark.gpu


def _assert_same_trace(gpu_recs, orc_recs, n):
    assert len(gpu_recs) == len(orc_recs)
    for k, (a, b) in enumerate(zip(gpu_recs, orc_recs)):
        ha, hb = a[0], b[0]
        # p, q, seeds, candidates, max_after, clusters, processed, rows, estimate
        for f in (0, 1, 2, 3, 5, 6, 7, 8, 9):
            assert ha[f] == hb[f], ("header", k, f, ha.tolist(), hb.tolist())
        if ha[4] >= 0:
            assert ha[4] == hb[4], ("packed", k)
            assert np.array_equal(a[6], b[6]), ("row lengths", k)
        for f, what in ((1, "seeds"), (2, "candidates"), (3, "cluster ids"), (4, "order"), (5, "membership")):
            assert np.array_equal(a[f], b[f]), (what, k)


@pytest.mark.parametrize("name", G.NAMES)
def test_golden_streams(name, gpu_lib, tmp_path):
    g = G.load(name)
    gr = native.Graph.from_csr(g["nindex"], g["nlist"])
    assert gr.max_csr == int(g["initial_max_csr"])
    if "max_csr" in g:
        gr.max_csr = int(g["max_csr"])
    gr.set_mis(g["mis0"])
    assert np.array_equal(gr.greedy_mis(), g["mis0"])
    bs = G.batches(g)
    for u, v, ins in bs:
        assert np.array_equal(gr.flag_updates(u, v), ins)
    for i, (u, v, ins) in enumerate(bs):
        gr.trace(True)
        gr.apply_batch(u, v, ins)
        want = G.rows(g, i)
        for x in range(gr.n):
            assert np.array_equal(gr.row(x), want[x]), (i, x)
        assert np.array_equal(gr.degrees(), g["b%d_deg" % i])
        assert np.array_equal(gr.get_mis(), g["b%d_mis_oracle" % i]), i
        hdr = np.stack([r[0] for r in gr.trace_records()])
        ref_hdr = g["b%d_trace_hdr" % i]
        assert hdr.shape == ref_hdr.shape
        cols = [0, 1, 2, 3, 5, 6, 7, 8, 9]
        assert np.array_equal(hdr[:, cols], ref_hdr[:, cols]), i
        known = hdr[:, 4] >= 0
        assert np.array_equal(hdr[known, 4], ref_hdr[known, 4])
    out = str(tmp_path / "c.egr")
    gr.compact(out)
    data = open(out, "rb").read()
    assert len(data) == int(g["compact_len"])
    assert hashlib.sha256(data).digest() == bytes(g["compact_sha256"])
    gr.close()


@pytest.mark.parametrize("name", G.REF_NAMES)
def test_reference_engine_golden(name, gpu_lib):
    """The library against the reference's own sync engine (src/misfit/misfit.cu
    run on the CPU with its kernels emulated thread by thread, clustering
    under the bulk-synchronous schedule), after every batch: the membership,
    every cluster id (stale ones included), each sub-batch's edges, rows and
    cluster count, and MAX_CSR_ELEMENTS."""
    g = G.load(name)
    gr = native.Graph.from_csr(g["nindex"], g["nlist"])
    assert gr.max_csr == int(g["initial_max_csr"])
    gr.max_csr = G.initial_max_csr(g)
    gr.set_mis(G.mis0(g))
    for i, (u, v, ins) in enumerate(G.batches(g)):
        gr.trace(True)
        gr.apply_batch(u, v, ins)
        assert np.array_equal(gr.get_mis(), G.mis_ref(g, i)), i
        assert G.cid_sha(gr.cluster_ids()) == bytes(g["b%d_cid_ref_sha" % i]), i
        hdr = np.stack([r[0] for r in gr.trace_records()])
        got = np.stack([hdr[:, 1] - hdr[:, 0], hdr[:, 8], hdr[:, 6]], axis=1)
        assert np.array_equal(got, g["b%d_sb_ref" % i]), i
        assert gr.max_csr == int(g["b%d_maxcsr_ref" % i]), i
    gr.close()


def test_pipelined_engine(gpu_lib):
    """mf_apply_batch_async / mf_collect in the loop of the reference's
    misfit_async (batch i+1 launched before batch i is collected): the same
    memberships as the plain engine, batch by batch; the queue's rules."""
    g = G.load("er1500")
    bs = G.batches(g)
    plain = native.Graph.from_csr(g["nindex"], g["nlist"])
    piped = native.Graph.from_csr(g["nindex"], g["nlist"])
    plain.set_mis(g["mis0"])
    piped.set_mis(g["mis0"])
    want = []
    for u, v, ins in bs:
        plain.apply_batch(u, v, ins)
        want.append((plain.get_mis(), plain.stats()))
    piped.apply_batch_async(*bs[0])
    for i in range(len(bs)):
        if i + 1 < len(bs):
            piped.apply_batch_async(*bs[i + 1])
        st = piped.collect()
        assert st["updates"] == bs[i][0].size
        assert st["sub_batches"] == want[i][1]["sub_batches"] and st["clusters"] == want[i][1]["clusters"]
    assert np.array_equal(piped.get_mis(), want[-1][0])
    assert np.array_equal(piped.get_mis(), g["b%d_mis_oracle" % (len(bs) - 1)])
    # nothing left to collect
    with pytest.raises(native.MisfitError) as e:
        piped.collect()
    assert e.value.status == -1
    # the plain entry point refuses a context with uncollected batches
    u, v, ins = bs[0]
    piped.apply_batch_async(u, v, ins)
    with pytest.raises(native.MisfitError) as e:
        piped.apply_batch(u, v, ins)
    assert e.value.status == -1
    piped.sync()
    # a bad batch fails when collected; the batch queued after it still runs
    ref = native.Graph.from_csr(g["nindex"], g["nlist"])
    ref.set_mis(piped.get_mis())
    bad = (np.array([0, 5], np.int32), np.array([1, 5], np.int32), np.zeros(2, np.uint8))
    piped.apply_batch_async(*bad)
    piped.apply_batch_async(*bs[1])
    with pytest.raises(native.MisfitError) as e:
        piped.collect()
    assert e.value.status == -1
    piped.collect()
    for u, v, ins in (bs[0], bs[1]):
        ref.apply_batch(u, v, ins)
    assert np.array_equal(piped.get_mis(), ref.get_mis())
    for gr in (plain, piped, ref):
        gr.close()


def _stream(kind, seed, batches, size, endpoints="uniform"):
    if kind == "er":
        n = 3000
        ni, nl = W.er_graph(n, 8, seed)
    else:
        n, (ni, nl) = W.rmat_graph(11, 8, seed)
    ts = W.ToggleStream(n, ni, nl, seed + 1)
    return n, ni, nl, [ts.next_batch(size, endpoints=endpoints) for _ in range(batches)]


@pytest.mark.parametrize("kind,seed,max_csr,pull", [("er", 11, None, 1), ("rmat", 12, None, 1), ("rmat", 13, 3000, 1),
                                                    ("rmat", 14, 40000, 1), ("er", 15, 3000, 2), ("rmat", 13, 3000, 2),
                                                    ("rmat", 14, 40000, 0)])
def test_stage_parity_live(kind, seed, max_csr, pull, gpu_lib):
    """Every sub-batch's header, seeds, candidates, exact row lengths (when
    the size bound reaches the limit), cluster ids, order and membership
    against the oracle; pull = tuning pull_sizes (exact 2-hop sizes by the
    push form, the cost model, or row passes for every seed)."""
    n, ni, nl, bs = _stream(kind, seed, 4, 500)
    orc = O.Oracle.from_csr(ni, nl)
    gr = native.Graph.from_csr(ni, nl)
    gr.set_tuning(pull_sizes=pull)
    if max_csr:
        orc.max_csr = max_csr
        gr.max_csr = max_csr
    mis = O.greedy_mis(ni, nl)
    orc.set_mis(mis)
    gr.set_mis(mis)
    flags = [orc.flag_updates(u, v) for u, v in bs]
    for (u, v), ins in zip(bs, flags):
        assert np.array_equal(gr.flag_updates(u, v), ins)
    for (u, v), ins in zip(bs, flags):
        orc.trace(True)
        gr.trace(True)
        orc.apply_batch(u, v, ins)
        gr.apply_batch(u, v, ins)
        _assert_same_trace(gr.trace_records(), orc.trace_records(), n)
        assert np.array_equal(gr.get_mis(), orc.get_mis())
        assert np.array_equal(gr.cluster_ids(), orc.cluster_ids())
        assert np.array_equal(gr.degrees(), orc.degrees())
        assert gr.max_csr == orc.max_csr
        assert gr.check_mis() == orc.check_mis()


@pytest.mark.parametrize("caps", ["3,0", "0,4096", "2,4096"])
def test_exact_sizes_push_form_retries(caps, gpu_lib, monkeypatch):
    """The push form of the exact 2-hop sizes with its per-pass capacities
    lowered (dense seeds, light pairs), so that seeds are turned away and
    retried in later passes, as at R-MAT scale 26 where 128 dense bitmaps
    fill a pass: row lengths, growths and results equal the oracle's."""
    monkeypatch.setenv("MISFIT_GB_EXACT_CAPS", caps)
    n, ni, nl, bs = _stream("rmat", 16, 3, 500, endpoints="preferential")
    orc = O.Oracle.from_csr(ni, nl)
    gr = native.Graph.from_csr(ni, nl)
    gr.set_tuning(pull_sizes=0)
    orc.max_csr = 3000
    gr.max_csr = 3000
    mis = O.greedy_mis(ni, nl)
    orc.set_mis(mis)
    gr.set_mis(mis)
    exact = 0
    for u, v in bs:
        ins = orc.flag_updates(u, v)
        orc.trace(True)
        gr.trace(True)
        orc.apply_batch(u, v, ins)
        gr.apply_batch(u, v, ins)
        _assert_same_trace(gr.trace_records(), orc.trace_records(), n)
        exact += gr.stats()["exact_sizes"]
        assert np.array_equal(gr.get_mis(), orc.get_mis())
        assert gr.max_csr == orc.max_csr
    assert exact > 0
    gr.close()


def _with_hubs(n, ni, nl, hubs, seed):
    """The symmetric graph (ni, nl) plus, for each (hub, degree) of hubs,
    edges from the hub to `degree` random vertices; sorted, de-duplicated."""
    rng = np.random.default_rng(seed)
    src = [np.repeat(np.arange(n, dtype=np.int64), np.diff(ni))]
    dst = [nl.astype(np.int64)]
    for h, d in hubs:
        x = rng.choice(n, size=d, replace=False).astype(np.int64)
        x = x[x != h]
        src += [np.full(x.size, h, np.int64), x]
        dst += [x, np.full(x.size, h, np.int64)]
    key = np.unique(np.concatenate(src) * n + np.concatenate(dst))
    s, d = key // n, key % n
    out = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(s, minlength=n), out=out[1:])
    return out, d.astype(np.int32)


@pytest.mark.parametrize("pull", [0, 2])
def test_exact_sizes_with_huge_rows(pull, gpu_lib):
    """Hubs of 20,000 and 17,000 neighbours on a sparse random graph: every
    seed's 2-hop list is large, so under a small limit the exact sizes decide
    each growth.  The row passes split the hubs' rows (more than 16,384
    positions) into chunks over many warps; sizes, growths and results
    equal the oracle's, and those of the push form."""
    n = 40000
    ni, nl = W.er_graph(n, 4, 51)
    ni, nl = _with_hubs(n, ni, nl, [(7, 20000), (12345, 17000)], 52)
    ts = W.ToggleStream(n, ni, nl, 53)
    bs = [ts.next_batch(300) for _ in range(3)]
    orc = O.Oracle.from_csr(ni, nl)
    gr = native.Graph.from_csr(ni, nl)
    gr.set_tuning(pull_sizes=pull)
    orc.max_csr = 50000
    gr.max_csr = 50000
    mis = O.greedy_mis(ni, nl)
    orc.set_mis(mis)
    gr.set_mis(mis)
    exact = 0
    for u, v in bs:
        ins = orc.flag_updates(u, v)
        orc.trace(True)
        gr.trace(True)
        orc.apply_batch(u, v, ins)
        gr.apply_batch(u, v, ins)
        _assert_same_trace(gr.trace_records(), orc.trace_records(), n)
        exact += gr.stats()["exact_sizes"]
        assert np.array_equal(gr.get_mis(), orc.get_mis())
        assert gr.max_csr == orc.max_csr
    assert exact > 0
    gr.close()


def test_config1_er10k_ten_batches(gpu_lib, tmp_path):
    """ER G(10000, avg 8), int32 .egr, seed 42; 10 batches of 2000 toggles
    (1000 deletes of existing edges, 1000 inserts of non-adjacent pairs);
    MIS after every batch identical to the oracle."""
    n = 10000
    ni, nl = W.er_graph(n, 8, 42)
    p = str(tmp_path / "er10k.egr")
    W.write_egr(p, n, ni, nl)
    ts = W.ToggleStream(n, ni, nl, 42)
    bs = [ts.next_batch(2000) for _ in range(10)]
    gr = native.Graph.open_egr(p)
    orc = O.Oracle.open_egr(p)
    mis = gr.greedy_mis()
    assert np.array_equal(mis, O.greedy_mis(ni, nl))
    gr.set_mis(mis)
    orc.set_mis(mis)
    flags = [gr.flag_updates(u, v) for u, v in bs]
    for (u, v), ins in zip(bs, flags):
        assert np.array_equal(ins, orc.flag_updates(u, v))
    for (u, v), ins in zip(bs, flags):
        gr.apply_batch(u, v, ins)
        orc.apply_batch(u, v, ins)
        assert np.array_equal(gr.get_mis(), orc.get_mis())
    assert gr.check_mis() == orc.check_mis()


@pytest.mark.parametrize("wide", [False, True])
def test_open_egr_layouts(wide, gpu_lib, tmp_path):
    g = G.load("er1500")
    p = str(tmp_path / "g.egr")
    W.write_egr(p, int(g["n"]), g["nindex"], g["nlist"], wide=wide)
    gr = native.Graph.open_egr(p)
    gr.set_mis(g["mis0"])
    for i, (u, v, ins) in enumerate(G.batches(g)):
        gr.apply_batch(u, v, ins)
        assert np.array_equal(gr.get_mis(), g["b%d_mis_oracle" % i])


def test_free_flags_all_overlay_transitions(gpu_lib):
    """Flags chosen at random instead of from the base graph: inserts of base
    edges, deletes of absent pairs, un-tombstones and forgets all occur,
    repeatedly on the same pairs within one batch."""
    n = 80
    ni, nl = W.er_graph(n, 5, 3)
    orc = O.Oracle.from_csr(ni, nl)
    gr = native.Graph.from_csr(ni, nl)
    mis = O.greedy_mis(ni, nl)
    orc.set_mis(mis)
    gr.set_mis(mis)
    rng = np.random.default_rng(5)
    for _ in range(8):
        m = 300
        u = rng.integers(0, n, m).astype(np.int32)
        v = rng.integers(0, n, m).astype(np.int32)
        keep = u != v
        u, v = u[keep], v[keep]
        ins = rng.integers(0, 2, u.size).astype(np.uint8)
        orc.apply_batch(u, v, ins)
        gr.apply_batch(u, v, ins)
        for x in range(n):
            assert np.array_equal(gr.row(x), orc.row(x)), x
        assert np.array_equal(gr.degrees(), orc.degrees())
        assert np.array_equal(gr.get_mis(), orc.get_mis())


def test_empty_and_invalid_batches(gpu_lib):
    g = G.load("er1500")
    gr = native.Graph.from_csr(g["nindex"], g["nlist"])
    gr.set_mis(g["mis0"])
    gr.apply_batch(np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0, np.uint8))
    assert np.array_equal(gr.get_mis(), g["mis0"])
    assert gr.stats()["sub_batches"] == 0
    for u, v in (([0], [0]), ([0], [1500]), ([-1], [3])):
        with pytest.raises(native.MisfitError) as e:
            gr.apply_batch(np.array(u, np.int32), np.array(v, np.int32), np.zeros(1, np.uint8))
        assert e.value.status == -1
    # the context stays usable after a rejected call
    u, v, ins = G.batches(g)[0]
    gr.apply_batch(u, v, ins)
    assert np.array_equal(gr.get_mis(), g["b0_mis_oracle"])


def test_bad_egr_files(gpu_lib, tmp_path):
    p = tmp_path / "t.egr"
    p.write_bytes(b"\x05\x00\x00\x00")
    with pytest.raises(native.MisfitError) as e:
        native.Graph.open_egr(str(p))
    assert e.value.status == -3
    g = G.load("er1500")
    W.write_egr(str(p), int(g["n"]), g["nindex"], g["nlist"])
    data = p.read_bytes()
    p.write_bytes(data[:-40])
    with pytest.raises(native.MisfitError) as e:
        native.Graph.open_egr(str(p))
    assert e.value.status == -3
    with pytest.raises(native.MisfitError) as e:
        native.Graph.open_egr(str(tmp_path / "missing.egr"))
    assert e.value.status == -2


_SEQ_SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import oracle as O
from misfit_gb300 import native, workloads as W
n, (ni, nl) = W.rmat_graph(11, 8, 21)
ts = W.ToggleStream(n, ni, nl, 22)
bs = [ts.next_batch(600) for _ in range(3)]
orc = O.Oracle.from_csr(ni, nl); gr = native.Graph.from_csr(ni, nl)
mis = O.greedy_mis(ni, nl); orc.set_mis(mis); gr.set_mis(mis)
seq = sys.argv[2] == "sequential"
for u, v in bs:
    ins = orc.flag_updates(u, v)
    orc.apply_batch(u, v, ins); gr.apply_batch(u, v, ins)
    assert np.array_equal(gr.get_mis(), orc.get_mis())
    assert (gr.stats()["repair_rounds"] == 0) == seq
# free flags: tombstones in base rows and added entries at row ends
n2 = 300
ni2, nl2 = W.er_graph(n2, 6, 4)
orc = O.Oracle.from_csr(ni2, nl2); gr = native.Graph.from_csr(ni2, nl2)
mis = O.greedy_mis(ni2, nl2); orc.set_mis(mis); gr.set_mis(mis)
rng = np.random.default_rng(9)
for _ in range(12):
    u = rng.integers(0, n2, 900).astype(np.int32); v = rng.integers(0, n2, 900).astype(np.int32)
    keep = u != v; u, v = u[keep], v[keep]
    ins = rng.integers(0, 2, u.size).astype(np.uint8)
    orc.apply_batch(u, v, ins); gr.apply_batch(u, v, ins)
    assert np.array_equal(gr.get_mis(), orc.get_mis())
print("ok")
"""


@pytest.mark.parametrize("mode,env", [("sequential", {"MISFIT_GB_REPAIR": "sequential"}),
                                      ("grid", {"MISFIT_GB_BIG_THRESHOLD": "0"}),
                                      ("host_rounds", {"MISFIT_GB_REPAIR": "rounds"}),
                                      ("host_rounds_grid", {"MISFIT_GB_REPAIR": "rounds",
                                                            "MISFIT_GB_BIG_THRESHOLD": "0"})])
def test_repair_variants_match(mode, env, gpu_lib, tmp_path):
    """The single-CTA sequential repair (the fallback after the round limit),
    the grid-wide hop-2 search (forced for every long search by a tiny
    threshold) and the host-driven rounds (each read back before the next is
    queued, where every other test queues two per read-back) all give the
    oracle's results on a whole stream."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    script = tmp_path / "variant.py"
    script.write_text(_SEQ_SCRIPT)
    out = subprocess.run([sys.executable, str(script), root, mode], env=dict(os.environ, **env),
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip().endswith("ok")


@pytest.mark.parametrize("layout", ["unsorted_rows", "asymmetric"])
def test_general_graphs_use_push_form(layout, gpu_lib):
    """Graphs that are not symmetric with sorted rows take the push form of
    the clustering write; results still equal the oracle's."""
    n, (ni, nl) = W.rmat_graph(10, 8, 31)
    nl = nl.copy()
    rng = np.random.default_rng(2)
    if layout == "unsorted_rows":
        for x in range(n):
            seg = nl[ni[x]:ni[x + 1]]
            nl[ni[x]:ni[x + 1]] = seg[rng.permutation(seg.size)]
    else:
        # drop one direction of some entries: rebuild CSR without them
        deg = np.diff(ni)
        src = np.repeat(np.arange(n), deg)
        keep = ~((src < nl) & (rng.random(nl.size) < 0.1))
        src, dst = src[keep], nl[keep]
        ni = np.zeros(n + 1, np.int64)
        np.cumsum(np.bincount(src, minlength=n), out=ni[1:])
        nl = dst.astype(np.int32)
    orc = O.Oracle.from_csr(ni, nl)
    gr = native.Graph.from_csr(ni, nl)
    mis = O.greedy_mis(ni, nl)
    orc.set_mis(mis)
    gr.set_mis(mis)
    u = rng.integers(0, n, 1500).astype(np.int32)
    v = rng.integers(0, n, 1500).astype(np.int32)
    keep = u != v
    u, v = u[keep], v[keep]
    for k in range(3):
        sl = slice(k * 400, (k + 1) * 400)
        ins = orc.flag_updates(u[sl], v[sl])
        assert np.array_equal(gr.flag_updates(u[sl], v[sl]), ins)
        orc.trace(True)
        gr.trace(True)
        orc.apply_batch(u[sl], v[sl], ins)
        gr.apply_batch(u[sl], v[sl], ins)
        _assert_same_trace(gr.trace_records(), orc.trace_records(), n)
        assert np.array_equal(gr.get_mis(), orc.get_mis())


@pytest.mark.parametrize("kind", ["er", "rmat"])
def test_exact_mode_matches_oracle(gpu_lib, kind):
    """Exact-MIS mode: the membership after every batch equals the oracle's
    exact mode bit for bit, and it is independent and maximal."""
    if kind == "er":
        nindex, nlist = W.er_graph(4000, 8, 31)
    else:
        _, (nindex, nlist) = W.rmat_graph(12, 8, 31)
    n = nindex.size - 1
    gr = native.Graph.from_csr(nindex, nlist)
    orc = O.Oracle.from_csr(nindex, nlist)
    try:
        mis0 = O.greedy_mis(nindex, nlist)
        gr.set_mis(mis0)
        orc.set_mis(mis0)
        gr.set_exact(True)
        orc.set_exact(True)
        ts = W.ToggleStream(n, nindex, nlist, 32)
        for b in range(4):
            u, v, ins = ts.next_batch(1500, with_flags=True)
            gr.apply_batch(u, v, ins)
            orc.apply_batch(u, v, ins)
            assert np.array_equal(gr.get_mis(), orc.get_mis()), b
            assert gr.check_mis() == (0, 0), b
    finally:
        gr.close()
        orc.close()


def test_tuning_settings_change_no_result(gpu_lib):
    """mf_set_tuning moves work between kernels, never a result: an R-MAT
    stream with cut sub-batches gives the same memberships and cluster ids
    under extreme settings as under the defaults; bad settings are refused."""
    from misfit_gb300 import autotune
    n, ni, nl, bs = _stream("rmat", 21, 3, 600, endpoints="preferential")
    mis0 = O.greedy_mis(ni, nl)
    orc = O.Oracle.from_csr(ni, nl)
    flags = [orc.flag_updates(u, v) for u, v in bs]
    results = []
    for tune in ({}, {"pull_long": 32, "heavy_min": 64, "big_threshold": 0, "first_bound": 8, "cand_push": 1,
                      "pull_sizes": 2},
                 {"pull_long": 1 << 20, "heavy_min": 1 << 30, "big_threshold": 1 << 40, "first_bound": 1 << 20,
                  "cand_push": 2, "pull_sizes": 0}):
        g = native.Graph.from_csr(ni, nl)
        if not tune:
            assert g.tuning() == autotune.DEFAULT_TUNING
        g.max_csr = 30000
        g.set_tuning(**tune)
        g.set_mis(mis0)
        out = []
        for (u, v), ins in zip(bs, flags):
            g.apply_batch(u, v, ins)
            out.append((g.get_mis(), g.cluster_ids()))
        results.append(out)
        for bad in ({"pull_long": 1}, {"first_bound": 4}, {"big_threshold": -1}, {"cand_push": 3},
                    {"pull_sizes": 3}):
            with pytest.raises(native.MisfitError):
                g.set_tuning(**bad)
        g.close()
    for other in results[1:]:
        for (m0, c0), (m1, c1) in zip(results[0], other):
            assert np.array_equal(m0, m1) and np.array_equal(c0, c1)
