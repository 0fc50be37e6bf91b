"""The batched form's one-CTA engine (misfit_gb300/csrc/mf_cta.cuh), run on
the CPU by an emulated CTA, against the oracle batch by batch: membership,
cluster ids, overlay rows, degrees, MAX_CSR_ELEMENTS and sub-batch counts.
The same source is the persistent kernel on the GPU
(tests/test_gpu_batched.py holds that one against the plain path)."""
import numpy as np
import pytest

import oracle as O
from misfit_gb300 import workloads as W
from tests import _golden as G
from tests.cta_emul import EmulGraph


def _compare(orc, eg, ctx, rows=True):
    assert np.array_equal(eg.get_mis(), orc.get_mis()), ctx
    assert np.array_equal(eg.cluster_ids(), orc.cluster_ids()), ctx
    assert np.array_equal(eg.degrees(), orc.degrees()), ctx
    assert eg.max_csr == orc.max_csr, ctx
    if rows:
        for x in range(orc.n):
            assert np.array_equal(eg.row(x), orc.row(x)), (ctx, x)


def _run(nindex, nlist, batches, threads, mis=None, max_csr=None, rows=True):
    orc = O.Oracle.from_csr(nindex, nlist)
    eg = EmulGraph(nindex, nlist)
    assert eg.max_csr == orc.max_csr
    if max_csr is not None:
        orc.max_csr = max_csr
        eg.max_csr = max_csr
    if mis is None:
        mis = O.greedy_mis(nindex, nlist)
    orc.set_mis(mis)
    eg.set_mis(mis)
    for i, (u, v, ins) in enumerate(batches):
        ns_o = orc.apply_batch(u, v, ins)
        ns_e = eg.apply_batch(u, v, ins, threads=threads)
        assert ns_o == ns_e, (i, ns_o, ns_e)
        _compare(orc, eg, i, rows)
    return orc, eg


@pytest.mark.parametrize("name", G.NAMES)
def test_engine_golden_streams(name):
    g = G.load(name)
    max_csr = int(g["max_csr"]) if "max_csr" in g else None
    _run(g["nindex"], g["nlist"], G.batches(g), threads=7, mis=g["mis0"], max_csr=max_csr)


@pytest.mark.parametrize("threads", [1, 32, 64])
def test_engine_er_insert_delete(threads):
    n = 600
    nindex, nlist = W.er_graph(n, 6, 3)
    st = W.ToggleStream(n, nindex, nlist, 5)
    orc = O.Oracle.from_csr(nindex, nlist)
    batches = []
    for _ in range(4):
        u, v = st.next_batch(150)
        batches.append((u, v, orc.flag_updates(u, v)))
    _run(nindex, nlist, batches, threads)


def test_engine_forced_growth_and_cuts():
    """A small MAX_CSR_ELEMENTS: many sub-batches, exact sizes and growth."""
    n, (nindex, nlist) = W.rmat_graph(9, 8, 4)
    st = W.ToggleStream(n, nindex, nlist, 9)
    orc = O.Oracle.from_csr(nindex, nlist)
    batches = []
    for _ in range(3):
        u, v = st.next_batch(300)
        batches.append((u, v, orc.flag_updates(u, v)))
    orc, eg = _run(nindex, nlist, batches, threads=33, max_csr=3000)
    assert eg.max_csr > 3000           # the limit grew
    assert eg.last()[8] > 0            # sub-batches that needed exact sizes
    assert eg.last()[3] > 1            # several sub-batches


def test_engine_free_flags_and_repeats():
    """Random flags that disagree with adjacency, pairs repeated inside a
    batch and across batches: every overlay transition (append, kill,
    tombstone, un-tombstone, re-append)."""
    rng = np.random.default_rng(12)
    n = 120
    nindex, nlist = W.er_graph(n, 5, 8)
    batches = []
    pool_u = rng.integers(0, n, 60)
    pool_v = rng.integers(0, n, 60)
    keep = pool_u != pool_v
    pool_u, pool_v = pool_u[keep], pool_v[keep]
    ui, vi = W.undirected_pairs(n, nindex, nlist)
    for b in range(5):
        k = 200
        pick = rng.integers(0, pool_u.size, k // 2)
        e = rng.integers(0, ui.size, k // 2)
        u = np.concatenate([pool_u[pick], ui[e]]).astype(np.int32)
        v = np.concatenate([pool_v[pick], vi[e]]).astype(np.int32)
        sw = rng.random(u.size) < 0.5
        u[sw], v[sw] = v[sw], u[sw].copy()
        perm = rng.permutation(u.size)
        u, v = u[perm], v[perm]
        ins = (rng.random(u.size) < 0.5).astype(np.uint8)
        batches.append((u, v, ins))
    _run(nindex, nlist, batches, threads=16)


def test_engine_rgg_stream():
    nindex, nlist = W.rgg_graph(800, 12, 21)
    n = nindex.size - 1
    st = W.ToggleStream(n, nindex, nlist, 22)
    orc = O.Oracle.from_csr(nindex, nlist)
    batches = []
    for mode in ("uniform", "low-degree"):
        u, v = st.next_batch(400, endpoints=mode.replace("-", "_"))
        batches.append((u, v, orc.flag_updates(u, v)))
    _run(nindex, nlist, batches, threads=32, rows=False)


def test_engine_full_block_width():
    """512 threads, a block size the kernel launches with: every chunked
    scan and window at full width, and the radix sort (2,200 endpoint slots,
    above the rank-sort limit)."""
    n = 800
    nindex, nlist = W.er_graph(n, 6, 31)
    st = W.ToggleStream(n, nindex, nlist, 32)
    orc = O.Oracle.from_csr(nindex, nlist)
    u, v = st.next_batch(1100)
    _run(nindex, nlist, [(u, v, orc.flag_updates(u, v))], 512, rows=False)


def test_engine_random_cases():
    """Seeded random cases: ER, RGG, R-MAT and general graphs (asymmetric,
    unsorted rows, repeated entries), initial sets that may not be
    independent, random flags, small MAX_CSR_ELEMENTS, thread counts from 1
    to 33."""
    rng = np.random.default_rng(77)
    for case in range(14):
        kind = case % 4
        n = int(rng.integers(20, 500))
        if kind == 0:
            ni, nl = W.er_graph(n, float(rng.uniform(1, 10)), int(rng.integers(1 << 30)))
        elif kind == 1:
            ni, nl = W.rgg_graph(n, float(rng.uniform(2, 14)), int(rng.integers(1 << 30)))
        elif kind == 2:
            _, (ni, nl) = W.rmat_graph(int(rng.integers(5, 9)), 6, int(rng.integers(1 << 30)))
        else:
            m0 = int(rng.integers(n, 6 * n))
            src, dst = rng.integers(0, n, m0), rng.integers(0, n, m0)
            keep = src != dst
            src, dst = src[keep], dst[keep]
            order = np.argsort(src, kind="stable")
            src, dst = src[order], dst[order]
            ni = np.zeros(n + 1, np.int64)
            np.add.at(ni, src + 1, 1)
            ni, nl = np.cumsum(ni), dst.astype(np.int32)
        n = ni.size - 1
        orc = O.Oracle.from_csr(ni, nl)
        batches = []
        for _ in range(2):
            m = int(rng.integers(1, 300))
            u, v = rng.integers(0, n, m).astype(np.int32), rng.integers(0, n, m).astype(np.int32)
            ok = u != v
            u, v = u[ok], v[ok]
            if u.size == 0:
                continue
            ins = orc.flag_updates(u, v) if rng.random() < 0.5 else (rng.random(u.size) < 0.5).astype(np.uint8)
            batches.append((u, v, ins))
        mis = (rng.random(n) < 0.2).astype(np.uint8) if case % 2 else None
        max_csr = int(rng.integers(50, 5000)) if case % 3 == 0 else None
        _run(ni, nl, batches, int(rng.choice([1, 5, 33])), mis=mis, max_csr=max_csr)


def test_engine_config1_stream():
    """The plain-method small configuration: ER G(10000, avg 8), seed 42,
    10 batches of 2000 toggles (half deletes of existing edges, half inserts
    of non-adjacent pairs), flags against the base graph; membership,
    cluster ids and degrees equal to the oracle after every batch."""
    n = 10000
    ni, nl = W.er_graph(n, 8, 42)
    ts = W.ToggleStream(n, ni, nl, 42)
    bs = [ts.next_batch(2000) for _ in range(10)]
    base = O.Oracle.from_csr(ni, nl)
    batches = [(u, v, base.flag_updates(u, v)) for u, v in bs]
    _run(ni, nl, batches, 16, rows=False)
