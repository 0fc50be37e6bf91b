"""The oracle against the reference's whole sync engine, run on the CPU.

oracle/_ref/libref_sync_emul.so is src/misfit/misfit.cu compiled with g++
against the host-only CUDA stand-in in oracle/ref_emul/ (kernels emulated
thread by thread; oracle/build.py, build_ref_emul).  These tests drive it on
fresh seeded streams -- insert-heavy ones, forced sub-batch cuts, growth of
MAX_CSR_ELEMENTS, both .egr layouts, flags chosen freely -- and compare,
after every batch, the membership, every cluster id, each sub-batch's edges,
rows and cluster count, and MAX_CSR_ELEMENTS with the oracle, under both
clustering schedules.  The last tests run the engines' own main()
(bin/misfit, bin/misfit_async) end to end.  Skipped where the emulation is
not built (it needs the reference tree: MISFIT_REF_ROOT).
"""
import hashlib
import os

import numpy as np
import pytest

import oracle as O
from misfit_gb300 import workloads as W

pytestmark = pytest.mark.skipif(O.ref_emul_lib("sync") is None or O.ref_emul_lib("async") is None,
                                reason="reference engine emulation not built (set MISFIT_REF_ROOT)")


def _compare_stream(path, mis0, batches, max_csr, serial):
    orc = O.Oracle.open_egr(path)
    orc.max_csr = max_csr
    orc.set_serial_clustering(serial)
    ref = O.RefEngine(path, max_csr, O.SERIAL if serial else O.BULK_SYNCHRONOUS)
    orc.set_mis(mis0)
    ref.set_mis(mis0)
    total_sb = 0
    grew = False
    for i, (u, v, ins) in enumerate(batches):
        orc.trace(True)
        orc.apply_batch(u, v, ins)
        before = ref.max_csr
        recs = ref.apply_batch(u, v, ins)
        grew |= ref.max_csr != before
        hdr = np.stack([r[0] for r in orc.trace_records()])
        assert [tuple(r) for r in recs] == [(int(h[1] - h[0]), int(h[8]), int(h[6])) for h in hdr], i
        assert np.array_equal(orc.get_mis(), ref.get_mis()), i
        assert np.array_equal(orc.cluster_ids(), ref.cluster_ids()), i
        assert orc.max_csr == ref.max_csr, i
        total_sb += len(recs)
    ref.close()
    return total_sb, grew


@pytest.mark.parametrize("serial", [False, True], ids=["bulk_synchronous", "serial"])
@pytest.mark.parametrize("kind,seed,wide,delete_frac", [
    ("er", 1, False, 0.5), ("er", 2, True, 0.2), ("er", 3, False, 0.0), ("rmat", 4, False, 0.5),
    ("rgg", 5, True, 0.5)])
def test_engine_matches_oracle(kind, seed, wide, delete_frac, serial, tmp_path):
    if kind == "er":
        n = 1200
        ni, nl = W.er_graph(n, 7, seed)
    elif kind == "rmat":
        n, (ni, nl) = W.rmat_graph(10, 6, seed)
    else:
        n = 1500
        ni, nl = W.rgg_graph(n, 10, seed)
    p = str(tmp_path / "g.egr")
    W.write_egr(p, n, ni, nl, wide=wide)
    ts = W.ToggleStream(n, ni, nl, seed + 100)
    pairs = [ts.next_batch(400, delete_frac=delete_frac) for _ in range(4)]
    orc = O.Oracle.open_egr(p)
    flags = [orc.flag_updates(u, v) for u, v in pairs]
    batches = [(u, v, f) for (u, v), f in zip(pairs, flags)]
    _compare_stream(p, O.greedy_mis(ni, nl), batches, orc.max_csr, serial)


@pytest.mark.parametrize("max_csr", [3000, 40000])
def test_engine_cuts_and_growth(max_csr, tmp_path):
    """A small MAX_CSR_ELEMENTS: the split rule cuts many sub-batches
    (misfit.cu:494-523) and, at 3000, the packed rows overflow it so that it
    grows during packing (misfit.cu:565-583) and steers every later cut."""
    n, (ni, nl) = W.rmat_graph(10, 8, 11)
    p = str(tmp_path / "g.egr")
    W.write_egr(p, n, ni, nl)
    ts = W.ToggleStream(n, ni, nl, 12)
    pairs = [ts.next_batch(250, endpoints="preferential") for _ in range(3)]
    orc = O.Oracle.open_egr(p)
    batches = [(u, v, orc.flag_updates(u, v)) for u, v in pairs]
    nsb, grew = _compare_stream(p, O.greedy_mis(ni, nl), batches, max_csr, False)
    assert nsb > 3 * len(batches)
    if max_csr == 3000:
        assert grew


def test_engine_free_flags(tmp_path):
    """Flags drawn at random instead of from the base graph: inserts of present
    edges and deletes of absent pairs (no-ops for the overlay, still processed
    by the kernels), un-tombstones and forgets of added edges."""
    n = 300
    ni, nl = W.er_graph(n, 5, 21)
    p = str(tmp_path / "g.egr")
    W.write_egr(p, n, ni, nl)
    rng = np.random.default_rng(22)
    batches = []
    for _ in range(5):
        m = 400
        u = rng.integers(0, n, m).astype(np.int32)
        v = rng.integers(0, n, m).astype(np.int32)
        keep = u != v
        batches.append((u[keep], v[keep], rng.integers(0, 2, int(keep.sum())).astype(np.uint8)))
    orc = O.Oracle.open_egr(p)
    _compare_stream(p, O.greedy_mis(ni, nl), batches, orc.max_csr, False)


@pytest.mark.parametrize("engine", ["sync", "async"])
def test_reference_main_end_to_end(engine, tmp_path):
    """The engine's own main() -- 5-argument CLI, batch-folder parsing with
    flags against the base graph, final-MIS file, in-place compaction -- on a
    fresh insert/delete stream, against the oracle driven the same way."""
    n = 2000
    ni, nl = W.er_graph(n, 9, 31)
    W.write_egr(str(tmp_path / "er.egr"), n, ni, nl)
    ts = W.ToggleStream(n, ni, nl, 32)
    pairs = [ts.next_batch(500) for _ in range(6)]
    W.write_batch_folder(str(tmp_path / "b"), pairs)
    mis0 = O.greedy_mis(ni, nl)
    W.write_mis_file(str(tmp_path / "mis.txt"), mis0)
    orc = O.Oracle.from_csr(ni, nl)
    orc.set_mis(mis0)
    flags = [orc.flag_updates(u, v) for u, v in pairs]
    for (u, v), f in zip(pairs, flags):
        orc.apply_batch(u, v, f)
    rc, log = O.run_reference_main(engine, ["er.egr", "mis.txt", "b", 6, 0], str(tmp_path))
    assert rc == 0, log[-2000:]
    fm = W.read_mis_file(str(tmp_path / "datasets" / "Final_MISs" / "er_flash_final_mis.txt"), n)
    assert np.array_equal(fm, orc.get_mis())
    assert "Final MIS cardinality:   %d" % int(fm.sum()) in log
    orc.compact(str(tmp_path / "o.egr"))
    assert (hashlib.sha256((tmp_path / "er.egr").read_bytes()).digest()
            == hashlib.sha256((tmp_path / "o.egr").read_bytes()).digest())


def test_schedules_differ_on_inserts_but_not_on_deletes(tmp_path):
    """Why one clustering schedule must be pinned: on an insert-bearing stream
    the two legal schedules of the reference's clustering kernel give
    different memberships; on a delete-only stream they agree."""
    n = 3000
    ni, nl = W.er_graph(n, 8, 41)
    p = str(tmp_path / "g.egr")
    W.write_egr(p, n, ni, nl)
    mis0 = O.greedy_mis(ni, nl)
    orc = O.Oracle.open_egr(p)
    for delete_frac, differ in ((0.5, True), (1.0, False)):
        ts = W.ToggleStream(n, ni, nl, 42)
        pairs = [ts.next_batch(600, delete_frac=delete_frac) for _ in range(4)]
        engines = [O.RefEngine(p, orc.max_csr, s) for s in (O.BULK_SYNCHRONOUS, O.SERIAL)]
        for e in engines:
            e.set_mis(mis0)
        for u, v in pairs:
            f = orc.flag_updates(u, v)
            for e in engines:
                e.apply_batch(u, v, f)
        assert (not np.array_equal(engines[0].get_mis(), engines[1].get_mis())) == differ
        for e in engines:
            e.close()
