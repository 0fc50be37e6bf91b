"""mf_flag_updates_noalloc (fixed device scratch, no allocation) against
mf_flag_updates, both through the C-ABI.  Collected last, so that it runs
both after the other GPU tests and, with `pytest tests/test_zz_no_alloc.py`,
alone in a fresh process.  Flags are bytes: comparisons are exact."""
import numpy as np
import pytest

from misfit_gb300 import native
from misfit_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MAXM = native.NOALLOC_MAX_UPDATES


def _queries(nindex, nlist, m, seed):
    """m pairs: half existing edges of the base graph, half random pairs."""
    rng = np.random.default_rng(seed)
    n = nindex.size - 1
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(nindex))
    pick = rng.integers(0, nlist.size, size=m // 2)
    eu, ev = src[pick], nlist[pick].astype(np.int64)
    ru = rng.integers(0, n, size=m - m // 2)
    rv = (ru + rng.integers(1, n, size=ru.size)) % n  # never equal to ru
    u = np.concatenate([eu, ru]).astype(np.int32)
    v = np.concatenate([ev, rv]).astype(np.int32)
    perm = rng.permutation(m)
    return u[perm], v[perm]


def _graph(shuffle_rows, seed):
    nindex, nlist = W.er_graph(20000, 8, seed)
    nlist = nlist.copy()
    if shuffle_rows:  # unsorted rows: the flag kernel takes its linear-scan branch
        rng = np.random.default_rng(seed + 1)
        for x in range(0, nindex.size - 1, 7):
            seg = nlist[nindex[x]:nindex[x + 1]]
            rng.shuffle(seg)
    return nindex, nlist


@pytest.mark.parametrize("shuffle_rows", [False, True])
def test_noalloc_flags_match_two_calls_in_a_row(gpu_lib, shuffle_rows):
    nindex, nlist = _graph(shuffle_rows, 11)
    g = native.Graph.from_csr(nindex, nlist)
    try:
        # give the overlay added entries and tombstones first
        bu, bv = _queries(nindex, nlist, 30000, 5)
        g.apply_batch(bu, bv, g.flag_updates(bu, bv))

        q1 = _queries(nindex, nlist, MAXM, 21)  # the largest accepted call
        q2 = (np.concatenate([bu[:500], q1[0][:700]]), np.concatenate([bv[:500], q1[1][:700]]))
        want1 = g.flag_updates(*q1)
        want2 = g.flag_updates(*q2)
        # two calls in a row; the second is shorter than the first, so the
        # scratch still holds the first call's entries beyond its length
        got1 = g.flag_updates_noalloc(*q1)
        got2 = g.flag_updates_noalloc(*q2)
        assert np.array_equal(got1, want1)
        assert np.array_equal(got2, want2)
        assert 0 < int(got1.sum()) < MAXM  # both flag values occur
        # and once more after the other entry point ran in between
        assert np.array_equal(g.flag_updates(*q2), g.flag_updates_noalloc(*q2))
    finally:
        g.close()


def test_noalloc_first_call_on_a_fresh_context_allocates_nothing(gpu_lib):
    """The first call on a new context, at the largest size, before any
    other entry point has grown the context's staging buffers: the
    library's allocation counter does not move, and a second call after it
    still matches mf_flag_updates."""
    nindex, nlist = _graph(False, 13)
    g = native.Graph.from_csr(nindex, nlist)
    try:
        q = _queries(nindex, nlist, MAXM, 31)
        before = native.allocations()
        got = g.flag_updates_noalloc(*q)
        again = g.flag_updates_noalloc(q[0][:1000], q[1][:1000])
        assert native.allocations() == before
        assert np.array_equal(got, g.flag_updates(*q))
        assert np.array_equal(again, got[:1000])
        assert native.allocations() > before   # mf_flag_updates grew the staging buffers
    finally:
        g.close()


def test_noalloc_limits_and_errors(gpu_lib):
    nindex, nlist = _graph(False, 12)
    g = native.Graph.from_csr(nindex, nlist)
    try:
        assert g.flag_updates_noalloc(np.zeros(0, np.int32), np.zeros(0, np.int32)).size == 0
        big = np.zeros(MAXM + 1, np.int32)
        with pytest.raises(native.MisfitError) as e:
            g.flag_updates_noalloc(big, big + 1)
        assert e.value.status == -7  # MF_ELIMIT
        n = nindex.size - 1
        for bad_u, bad_v in ((3, 3), (n, 1), (-1, 2)):
            u = np.array([0, bad_u, 5], np.int32)
            v = np.array([1, bad_v, 6], np.int32)
            with pytest.raises(native.MisfitError) as e:
                g.flag_updates_noalloc(u, v)
            assert e.value.status == -1  # MF_EINVAL
        # a valid call after the failures still agrees
        q = _queries(nindex, nlist, 4096, 3)
        assert np.array_equal(g.flag_updates_noalloc(*q), g.flag_updates(*q))
    finally:
        g.close()


def test_noalloc_two_contexts_one_device(gpu_lib):
    """Two contexts on one device share the scratch; calls made one after
    the other each see their own graph."""
    a_ni, a_nl = _graph(False, 13)
    b_ni, b_nl = _graph(False, 14)
    ga = native.Graph.from_csr(a_ni, a_nl)
    gb = native.Graph.from_csr(b_ni, b_nl)
    try:
        qa = _queries(a_ni, a_nl, 8192, 7)
        qb = _queries(b_ni, b_nl, 8192, 8)
        ra = ga.flag_updates_noalloc(*qa)
        rb = gb.flag_updates_noalloc(*qb)
        assert np.array_equal(ra, ga.flag_updates(*qa))
        assert np.array_equal(rb, gb.flag_updates(*qb))
    finally:
        ga.close()
        gb.close()
