"""Serving pool (mf_pool_*) through the C-ABI: every graph's membership after
its batches must equal the one a dedicated context gives ("alone"), while the
pool runs the graphs' batches concurrently under an HBM budget that forces
evictions to pinned host memory and restores ("in the mix").  Membership is
bytes: comparisons are exact."""
import numpy as np
import pytest

from misfit_gb300 import native
from misfit_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _graphs(count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(rng.integers(2000, 20000))
        if k % 2 == 0:
            nindex, nlist = W.er_graph(n, float(rng.uniform(4, 12)), seed + k)
        else:
            nindex, nlist = W.rgg_graph(n, float(rng.uniform(4, 16)), seed + k)
        out.append((nindex, nlist))
    return out


def _streams(graphs, nbatches, seed):
    """Per graph: initial MIS, its batches with flags, the membership a
    dedicated context has after each batch."""
    plans = []
    for k, (nindex, nlist) in enumerate(graphs):
        n = nindex.size - 1
        g = native.Graph.from_csr(nindex, nlist)
        try:
            mis0 = g.greedy_mis()
            g.set_mis(mis0)
            ts = W.ToggleStream(n, nindex, nlist, seed + 17 * k)
            batches, after = [], []
            for b in range(nbatches):
                u, v = ts.next_batch(int(np.random.default_rng(seed + k + b).integers(10, 3000)))
                ins = g.flag_updates(u, v)
                g.apply_batch(u, v, ins)
                batches.append((u, v, ins))
                after.append(g.get_mis())
        finally:
            g.close()
        plans.append((mis0, batches, after))
    return plans


def test_pool_matches_dedicated_contexts_under_eviction(gpu_lib):
    graphs = _graphs(12, 5)
    plans = _streams(graphs, 3, 100)
    # a budget that holds only a few of the graphs at once (a graph's device
    # footprint is ~100-200 B per vertex plus ~8 B per entry)
    budget = int(3 * max((ni.size - 1) * 200 + nl.size * 8 for ni, nl in graphs))
    with native.Pool(budget, workers=4) as pool:
        gids = [pool.add_graph(ni, nl, plans[k][0]) for k, (ni, nl) in enumerate(graphs)]
        rids = []
        for b in range(3):                       # interleaved: batch b of every graph
            for k, gid in enumerate(gids):
                u, v, ins = plans[k][1][b]
                rids.append(pool.submit(gid, u, v, ins))
        lat = [pool.wait(r) for r in rids]
        assert all(x >= 0 for x in lat)
        for k, gid in enumerate(gids):
            assert np.array_equal(pool.get_mis(gid), plans[k][2][-1]), k
        st = pool.stats()
    assert st["completed"] == 3 * len(graphs)
    assert st["errors"] == 0
    assert st["evictions"] > 0 and st["restores"] > 0


def test_pool_one_graph_batch_by_batch(gpu_lib):
    """Waiting for each batch before the next: the membership after every
    batch equals the dedicated context's."""
    graphs = _graphs(3, 9)
    plans = _streams(graphs, 4, 300)
    with native.Pool(1 << 34, workers=2) as pool:
        gids = [pool.add_graph(ni, nl, plans[k][0]) for k, (ni, nl) in enumerate(graphs)]
        for b in range(4):
            for k, gid in enumerate(gids):
                u, v, ins = plans[k][1][b]
                pool.wait(pool.submit(gid, u, v, ins))
                assert np.array_equal(pool.get_mis(gid), plans[k][2][b]), (k, b)


def test_pool_errors(gpu_lib):
    with native.Pool(1 << 30, workers=1) as pool:
        ni, nl = W.er_graph(500, 4, 3)
        gid = pool.add_graph(ni, nl, np.zeros(500, np.uint8))
        with pytest.raises(native.MisfitError):
            pool.submit(gid + 5, np.array([0], np.int32), np.array([1], np.int32), np.array([1], np.uint8))
        # a bad batch fails on its own request; the pool keeps serving
        bad = pool.submit(gid, np.array([0, 3], np.int32), np.array([0, 4], np.int32), np.array([1, 1], np.uint8))
        with pytest.raises(native.MisfitError):
            pool.wait(bad)
        ok = pool.submit(gid, np.array([0], np.int32), np.array([1], np.int32), np.array([1], np.uint8))
        pool.wait(ok)
        assert pool.stats()["errors"] == 1


def test_pool_batched_dispatch_matches_dedicated_contexts(gpu_lib):
    """Continuous batching (mf_pool_set_batching): small requests are applied
    in mf_apply_batches steps by the dispatcher, large ones by the workers,
    under a budget that forces evictions; every graph's membership equals the
    dedicated context's, and a bad request fails alone."""
    graphs = _graphs(12, 15)
    plans = _streams(graphs, 3, 700)
    budget = int(3 * max((ni.size - 1) * 200 + nl.size * 8 for ni, nl in graphs))
    with native.Pool(budget, workers=3) as pool:
        pool.set_batching(native.batched_opts(max_cta_updates=1500, pool_idle_first=0))
        gids = [pool.add_graph(ni, nl, plans[k][0]) for k, (ni, nl) in enumerate(graphs)]
        rids = []
        for b in range(3):
            for k, gid in enumerate(gids):
                u, v, ins = plans[k][1][b]
                rids.append(pool.submit(gid, u, v, ins))
        bad = pool.submit(gids[0], np.array([0, 3], np.int32), np.array([0, 4], np.int32), np.array([1, 1], np.uint8))
        lat = [pool.wait(r) for r in rids]
        assert all(x >= 0 for x in lat)
        with pytest.raises(native.MisfitError):
            pool.wait(bad)
        for k, gid in enumerate(gids):
            assert np.array_equal(pool.get_mis(gid), plans[k][2][-1]), k
        st = pool.stats()
    assert st["completed"] == 3 * len(graphs) + 1
    assert st["errors"] == 1
    assert st["batched_steps"] > 0 and 0 < st["batched_requests"] < 3 * len(graphs)
    assert st["evictions"] > 0


@pytest.mark.timeout(240, method="thread")
def test_pool_drain_wakes_after_eviction(gpu_lib):
    """A request's completion can push the pool over its budget, so the
    worker evicts an idle graph right after it reports the request done.
    mf_pool_drain and mf_pool_get_mis wait for every graph to be idle; they
    must wake when that eviction ends, not only when a request completes.
    Many submit-then-drain cycles at a budget that evicts on every
    completion; the timeout turns a lost wake-up into a failure."""
    graphs = _graphs(4, 41)
    plans = _streams(graphs, 2, 400)
    budget = int(1.2 * max((ni.size - 1) * 200 + nl.size * 8 for ni, nl in graphs))
    with native.Pool(budget, workers=2) as pool:
        gids = [pool.add_graph(ni, nl, plans[k][0]) for k, (ni, nl) in enumerate(graphs)]
        for b in range(2):
            for k, gid in enumerate(gids):
                u, v, ins = plans[k][1][b]
                rid = pool.submit(gid, u, v, ins)
                pool.drain()
                assert pool.wait(rid) >= 0
                assert np.array_equal(pool.get_mis(gid), plans[k][2][b]), (b, k)
        st = pool.stats()
    assert st["errors"] == 0 and st["evictions"] > 0


def test_pool_batched_dispatch_leaves_dense_graphs_to_workers(gpu_lib):
    """Continuous batching gives the dispatcher a request only while one CTA's
    walk of its 2-hop neighbourhoods stays small: lines * (1 + mean degree)^2
    within max_cta_updates * 33^2.  On a dense graph (mean degree ~95) the
    200-line requests go to the workers and the 20-line ones to the
    dispatcher; memberships equal the dedicated context's either way.  With
    pool_idle_first (the default) a lone small request meets idle workers and
    goes to them: no batched step at all."""
    n = 120
    ni, nl = W.er_graph(n, 95.0, 77)
    g = native.Graph.from_csr(ni, nl)
    mis0 = g.greedy_mis()
    g.set_mis(mis0)
    ts = W.ToggleStream(n, ni, nl, 78)
    reqs, after = [], []
    for size in (200, 20, 200, 20, 200, 20):
        u, v = ts.next_batch(size)
        ins = g.flag_updates(u, v)
        g.apply_batch(u, v, ins)
        reqs.append((u, v, ins))
        after.append(g.get_mis())
    g.close()
    for idle_first, batched, handed in ((0, 3, 0), (1, 0, 3)):
        with native.Pool(1 << 30, workers=2) as pool:
            pool.set_batching(native.batched_opts(max_cta_updates=512, pool_idle_first=idle_first))
            gid = pool.add_graph(ni, nl, mis0)
            for k, (u, v, ins) in enumerate(reqs):
                assert pool.wait(pool.submit(gid, u, v, ins)) >= 0
                assert np.array_equal(pool.get_mis(gid), after[k]), (idle_first, k)
            st = pool.stats()
        assert st["completed"] == len(reqs)
        assert (st["batched_requests"], st["handed_to_workers"]) == (batched, handed), idle_first
