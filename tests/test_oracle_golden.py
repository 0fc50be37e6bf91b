"""The oracle against the golden vectors taken from the reference's own host
code (flags, overlay rows, degrees, 2-hop lists, compaction bytes, greedy
seed MIS) and against its own recorded per-batch results."""
import hashlib
import os

import numpy as np
import pytest

import oracle as O
from tests import _golden as G


@pytest.mark.parametrize("name", G.NAMES)
def test_oracle_matches_reference_golden(name, tmp_path):
    g = G.load(name)
    orc = O.Oracle.from_csr(g["nindex"], g["nlist"])
    assert orc.max_csr == int(g["initial_max_csr"])
    if "max_csr" in g:
        orc.max_csr = int(g["max_csr"])
    orc.set_mis(g["mis0"])
    bs = G.batches(g)
    for u, v, ins in bs:  # flags are evaluated before any batch is applied
        assert np.array_equal(orc.flag_updates(u, v), ins)
    for i, (u, v, ins) in enumerate(bs):
        orc.trace(True)
        orc.apply_batch(u, v, ins)
        want = G.rows(g, i)
        for x in range(orc.n):
            assert np.array_equal(orc.row(x), want[x]), (i, x)
        assert np.array_equal(orc.degrees(), g["b%d_deg" % i])
        for s, lst in G.twohop(g, i):
            assert np.array_equal(orc.two_hop(s), lst), (i, s)
        assert np.array_equal(orc.get_mis(), g["b%d_mis_oracle" % i])
        hdr = np.stack([r[0] for r in orc.trace_records()])
        assert np.array_equal(hdr, g["b%d_trace_hdr" % i])
    out = str(tmp_path / "c.egr")
    assert orc.compact(out) == 0
    data = open(out, "rb").read()
    assert len(data) == int(g["compact_len"])
    assert hashlib.sha256(data).digest() == bytes(g["compact_sha256"])


def test_sample_is_schedule_independent_golden():
    """The bundled stream is delete-only: the reference leaves the seed MIS
    unchanged whatever the schedule, so the final MIS is a pinned answer."""
    g = G.load("sample")
    assert int(g["mis0"].sum()) == 533
    assert all(int(g["b%d_ins" % i].sum()) == 0 for i in range(int(g["num_batches"])))
    assert np.array_equal(g["b4_mis_oracle"], g["mis0"])


@pytest.mark.parametrize("name", G.NAMES)
def test_greedy_seed_mis(name):
    g = G.load(name)
    mis = O.greedy_mis(g["nindex"], g["nlist"])
    assert np.array_equal(mis, g["mis0"])
    # the algorithm of tools/compute_initial_mis.py, restated in numpy-free Python
    n = int(g["n"])
    ni, nl = g["nindex"], g["nlist"]
    blocked = np.zeros(n, bool)
    want = np.zeros(n, np.uint8)
    for x in range(n):
        if blocked[x]:
            continue
        want[x] = 1
        blocked[nl[ni[x]:ni[x + 1]]] = True
    assert np.array_equal(mis, want)


def test_oracle_property_counts_sample():
    g = G.load("sample")
    orc = O.Oracle.from_csr(g["nindex"], g["nlist"])
    orc.set_mis(g["mis0"])
    for u, v, ins in G.batches(g):
        orc.apply_batch(u, v, ins)
    viol, uncovered = orc.check_mis()
    assert viol == 0
    assert uncovered == 19


def test_oracle_exact_mode_is_a_mis():
    """Exact-MIS mode of the oracle: independent and maximal after every batch."""
    from misfit_gb300 import workloads as W
    nindex, nlist = W.er_graph(2000, 6, 41)
    orc = O.Oracle.from_csr(nindex, nlist)
    try:
        orc.set_mis(O.greedy_mis(nindex, nlist))
        orc.set_exact(True)
        ts = W.ToggleStream(2000, nindex, nlist, 42)
        for _ in range(3):
            u, v, ins = ts.next_batch(600, with_flags=True)
            orc.apply_batch(u, v, ins)
            assert orc.check_mis() == (0, 0)
    finally:
        orc.close()


@pytest.mark.parametrize("serial", [False, True], ids=["bulk_synchronous", "serial"])
@pytest.mark.parametrize("name", G.REF_NAMES)
def test_oracle_matches_reference_engine_golden(name, serial):
    """The oracle against the reference's own sync engine (src/misfit/misfit.cu
    run on the CPU, kernels emulated thread by thread), batch after batch:
    membership, every cluster id (stale ones included), each sub-batch's
    edges, rows and cluster count, and MAX_CSR_ELEMENTS -- under the
    bulk-synchronous clustering schedule, and the membership under the serial
    one."""
    g = G.load(name)
    orc = O.Oracle.from_csr(g["nindex"], g["nlist"])
    orc.max_csr = G.initial_max_csr(g)
    orc.set_serial_clustering(serial)
    orc.set_mis(G.mis0(g))
    for i, (u, v, ins) in enumerate(G.batches(g)):
        orc.trace(True)
        orc.apply_batch(u, v, ins)
        assert np.array_equal(orc.get_mis(), G.mis_ref(g, i, serial)), i
        if serial:
            continue
        assert G.cid_sha(orc.cluster_ids()) == bytes(g["b%d_cid_ref_sha" % i]), i
        hdr = np.stack([r[0] for r in orc.trace_records()])
        got = np.stack([hdr[:, 1] - hdr[:, 0], hdr[:, 8], hdr[:, 6]], axis=1)
        assert np.array_equal(got, g["b%d_sb_ref" % i]), i
        assert orc.max_csr == int(g["b%d_maxcsr_ref" % i]), i


@pytest.mark.parametrize("name", ["sample", "er1500", "cfg1"])
def test_reference_mains_agree_with_their_engine(name):
    """bin/misfit and bin/misfit_async (the reference's own main(), run on the
    CPU) write the same final MIS as the engine stepped a batch at a time, and
    both compact to the bytes the reference's compactor writes."""
    g = G.load(name)
    nb = int(g["num_batches"])
    for engine in ("sync", "async"):
        assert np.array_equal(G.main_final_mis(g, engine), G.mis_ref(g, nb - 1)), engine
    if "compact_sha256" in g:
        assert bytes(g["main_sync_compact_sha256"]) == bytes(g["compact_sha256"])
        assert bytes(g["main_async_compact_sha256"]) == bytes(g["compact_sha256"])
