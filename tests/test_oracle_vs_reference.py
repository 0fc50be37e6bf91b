"""The oracle and the library's file helpers against the reference's own
host code (oracle/_ref), on fresh seeded inputs.  Skipped where the
reference tree is not present."""
import hashlib
import os

import numpy as np
import pytest

import oracle as O
from misfit_gb300 import workloads as W

pytestmark = pytest.mark.skipif(O.ref_lib() is None, reason="reference harness unavailable")


def _graph(kind, seed):
    if kind == "er":
        n = 800
        ni, nl = W.er_graph(n, 6, seed)
    else:
        n, (ni, nl) = W.rmat_graph(9, 6, seed)
    return n, ni, nl


@pytest.mark.parametrize("kind,seed,wide", [("er", 1, False), ("er", 2, True), ("rmat", 3, False)])
def test_overlay_bfs_flags_compaction(kind, seed, wide, tmp_path):
    n, ni, nl = _graph(kind, seed)
    p = str(tmp_path / "g.egr")
    W.write_egr(p, n, ni, nl, wide=wide)
    ts = W.ToggleStream(n, ni, nl, seed + 10)
    W.write_batch_folder(str(tmp_path / "b"), [ts.next_batch(150) for _ in range(4)])
    ref = O.Reference(p)
    orc = O.Oracle.open_egr(p)
    orc.set_mis(O.greedy_mis(ni, nl))
    from misfit_gb300 import build, native
    build.build()
    files = O.ref_list_batch_files(str(tmp_path / "b"))
    assert files == native.list_batch_files(str(tmp_path / "b"))
    parsed = []
    for f in files:
        u, v, ins = ref.parse_batch_file(str(tmp_path / "b" / f))
        lu, lv = native.read_batch_file(str(tmp_path / "b" / f), n)
        assert np.array_equal(lu, u) and np.array_equal(lv, v)
        assert np.array_equal(orc.flag_updates(u, v), ins)
        parsed.append((u, v, ins))
    for u, v, ins in parsed:
        ref.apply_updates(u, v, ins)
        orc.apply_batch(u, v, ins)
        for x in range(n):
            assert np.array_equal(ref.row(x), orc.row(x))
            assert ref.degree(x) == orc.degree(x)
        for s in np.unique(np.concatenate([u, v]))[:60]:
            a, _ = ref.two_hop(int(s))
            assert np.array_equal(a, orc.two_hop(int(s)))
        for a, b in zip(u[:50], v[:50]):
            assert ref.is_adjacent(int(a), int(b)) == orc.is_adjacent(int(a), int(b))
    ref.compact(str(tmp_path / "r.egr"))
    orc.compact(str(tmp_path / "o.egr"))
    assert open(str(tmp_path / "r.egr"), "rb").read() == open(str(tmp_path / "o.egr"), "rb").read()


def test_overlay_general_semantics_on_asymmetric_toggles(tmp_path):
    """Flags chosen freely (not from the base graph) drive every overlay
    transition: un-tombstone, forget of an added edge, re-insert order."""
    n = 60
    ni, nl = W.er_graph(n, 4, 7)
    p = str(tmp_path / "g.egr")
    W.write_egr(p, n, ni, nl)
    ref = O.Reference(p)
    orc = O.Oracle.open_egr(p)
    rng = np.random.default_rng(0)
    for _ in range(6):
        m = 120
        u = rng.integers(0, n, m).astype(np.int32)
        v = rng.integers(0, n, m).astype(np.int32)
        keep = u != v
        u, v = u[keep], v[keep]
        ins = rng.integers(0, 2, u.size).astype(np.uint8)
        ref.apply_updates(u, v, ins)
        orc.apply_batch(u, v, ins)
        for x in range(n):
            assert np.array_equal(ref.row(x), orc.row(x))
            assert ref.degree(x) == orc.degree(x)
