"""Batched form (mf_apply_batches) through the C-ABI: every graph's state
after each step -- membership, cluster ids, degrees, rows, MAX_CSR_ELEMENTS
-- must equal what the plain per-graph loop (mf_apply_batch on a dedicated
context) gives on the same batches.  Batches that fit one CTA run in the
persistent kernel, the others through the multi-launch path in the same
call; a graph's batches may alternate between the two.  All values are
integers or bytes: comparisons are exact."""
import numpy as np
import pytest

import oracle as O
from misfit_gb300 import native
from misfit_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _graphs(seed):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(14):
        n = int(rng.integers(150, 12000))
        kind = k % 3
        if kind == 0:
            nindex, nlist = W.er_graph(n, float(rng.uniform(3, 12)), seed + k)
        elif kind == 1:
            nindex, nlist = W.rgg_graph(n, float(rng.uniform(4, 20)), seed + k)
        else:
            _, (nindex, nlist) = W.rmat_graph(int(rng.integers(8, 13)), 8, seed + k)
        out.append((nindex, nlist))
    return out


def _state(g, rows):
    return (g.get_mis(), g.cluster_ids(), g.degrees(), g.max_csr, [g.row(int(x)) for x in rows])


def _same(a, b, ctx):
    assert np.array_equal(a[0], b[0]), ("membership", ctx)
    assert np.array_equal(a[1], b[1]), ("cluster ids", ctx)
    assert np.array_equal(a[2], b[2]), ("degrees", ctx)
    assert a[3] == b[3], ("MAX_CSR_ELEMENTS", ctx)
    for ra, rb in zip(a[4], b[4]):
        assert np.array_equal(ra, rb), ("rows", ctx)


def _run(seed, steps, opts, small_limit=None):
    graphs = _graphs(seed)
    rng = np.random.default_rng(seed + 1)
    plain, batched, streams, probe = [], [], [], []
    try:
        for k, (nindex, nlist) in enumerate(graphs):
            a = native.Graph.from_csr(nindex, nlist)
            b = native.Graph.from_csr(nindex, nlist)
            plain.append(a)
            batched.append(b)
            if small_limit is not None and k % 4 == 1:
                a.max_csr = small_limit
                b.max_csr = small_limit
            mis = a.greedy_mis()
            a.set_mis(mis)
            b.set_mis(mis)
            n = nindex.size - 1
            streams.append(W.ToggleStream(n, nindex, nlist, seed + 31 * k))
            probe.append(rng.integers(0, n, 64))
        kinds = {"kernel_items": 0, "path_items": 0}
        for step in range(steps):
            batches = []
            for k, (a, st) in enumerate(zip(plain, streams)):
                size = int(np.exp(rng.uniform(np.log(5), np.log(3000))))
                if step == 1 and k % 5 == 0:
                    size = 12000          # above the kernel's default limit: the multi-launch path
                mode = ("uniform", "preferential", "low_degree")[(k + step) % 3]
                u, v = st.next_batch(size, endpoints=mode)
                batches.append((u, v, a.flag_updates(u, v)))
            for a, (u, v, ins) in zip(plain, batches):
                a.apply_batch(u, v, ins)
            stats = native.apply_batches(batched, batches, opts)
            for key in kinds:
                kinds[key] += stats[key]
            for k, (a, b) in enumerate(zip(plain, batched)):
                _same(_state(b, probe[k]), _state(a, probe[k]), (seed, step, k))
                assert b.stats()["sub_batches"] == a.stats()["sub_batches"], (seed, step, k)
        return kinds
    finally:
        for g in plain + batched:
            g.close()


def test_batched_equals_plain_loop():
    kinds = _run(5, 3, None)
    assert kinds["kernel_items"] > 0 and kinds["path_items"] > 0


def test_batched_plain_launches_and_block_sizes():
    _run(6, 2, native.batched_opts(use_graph=0, block=256, ctas_per_sm=1))
    _run(7, 2, native.batched_opts(block=1024, ctas_per_sm=1))


def test_batched_growth_and_cuts():
    """A small MAX_CSR_ELEMENTS on some graphs: many sub-batches, exact
    sizes and growth of the limit inside the kernel."""
    _run(8, 2, None, small_limit=4000)


def test_batched_matches_oracle():
    nindex, nlist = W.rgg_graph(3000, 10, 44)
    n = nindex.size - 1
    orc = O.Oracle.from_csr(nindex, nlist)
    g = native.Graph.from_csr(nindex, nlist)
    try:
        mis = O.greedy_mis(nindex, nlist)
        orc.set_mis(mis)
        g.set_mis(mis)
        st = W.ToggleStream(n, nindex, nlist, 45)
        for _ in range(4):
            u, v = st.next_batch(700)
            ins = orc.flag_updates(u, v)
            orc.apply_batch(u, v, ins)
            s = native.apply_batches([g], [(u, v, ins)])
            assert s["kernel_items"] == 1
            assert np.array_equal(g.get_mis(), orc.get_mis())
            assert np.array_equal(g.cluster_ids(), orc.cluster_ids())
            assert np.array_equal(g.degrees(), orc.degrees())
    finally:
        g.close()


def test_batched_rejects_bad_batch_before_running():
    nindex, nlist = W.er_graph(500, 6, 3)
    a = native.Graph.from_csr(nindex, nlist)
    b = native.Graph.from_csr(nindex, nlist)
    try:
        mis = a.greedy_mis()
        a.set_mis(mis)
        b.set_mis(mis)
        st = W.ToggleStream(500, nindex, nlist, 4)
        u, v = st.next_batch(50)
        good = (u, v, a.flag_updates(u, v))
        bad = (np.array([1, 2], np.int32), np.array([2, 500], np.int32), np.array([1, 1], np.uint8))
        with pytest.raises(native.MisfitError):
            native.apply_batches([a, b], [good, bad])
        assert np.array_equal(a.get_mis(), mis)     # nothing ran
        with pytest.raises(native.MisfitError):
            native.apply_batches([a, a], [good, good])   # the same context twice
    finally:
        a.close()
        b.close()
