"""Generate the golden fixtures under tests/golden/ (run where the reference
tree is present; the output is committed and the tests read only the .npz).

Pins taken from the reference's own host code (oracle/_ref, built from the
reference sources by oracle/build.py):
  * parse-time flags of every batch line (core/cli_setup.h:66-82),
  * every overlay row and DeltaOverlay::degree after every batch
    (core/FlashGraph.h:172-311 driven by the batch-apply loop),
  * exact 2-hop lists and hop-1 sets of the seeds (get_h_hop_neighborhood),
  * the bytes of the compacted .egr (core/flash_compactor.h),
  * the greedy seed MIS of tools/compute_initial_mis.py (sample_mis.txt).
Taken from the reference's whole sync engine run on the CPU (src/misfit/misfit.cu
compiled against oracle/ref_emul, its kernels emulated thread by thread;
oracle/_ref/libref_sync_emul.so): after every batch the membership, the
cluster ids (sha256 of the int32 array), each sub-batch's edges, rows and
cluster count, and MAX_CSR_ELEMENTS -- under the bulk-synchronous
clustering schedule (the one the oracle and the library pin) and, for the
membership, under the serial one.  Taken from the reference engines' own
main() (bin/misfit and bin/misfit_async, run the same way): the final-MIS
file and the bytes of the in-place compaction.
Taken from the oracle (misfit_oracle.cpp, canonical schedule): the MIS after
every batch and the per-sub-batch trace headers.

cfg1.npz holds the config-1 stream (ER G(10000, 8), seed 42, 10 x 2000
toggles): its inputs and the reference engines' results only.

Usage: python tests/golden/make_golden.py <reference_root>
       (or with MISFIT_REF_ROOT set)
"""
import hashlib
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from misfit_gb300 import workloads as W  # noqa: E402


def rows_csr(get_row, n):
    rows = [get_row(x) for x in range(n)]
    indptr = np.zeros(n + 1, np.int64)
    indptr[1:] = np.cumsum([len(r) for r in rows])
    return indptr, (np.concatenate(rows).astype(np.int32) if indptr[-1] else np.zeros(0, np.int32))


def seeds_first_appearance(u, v):
    seen, out = set(), []
    for a, b in zip(u.tolist(), v.tolist()):
        for x in (a, b):
            if x not in seen:
                seen.add(x)
                out.append(x)
    return np.array(out, np.int32)


def sha(a):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), np.uint8)


def capture_reference_engine(out, egr_path, batches, mis0, max_csr):
    """The reference's sync engine (CPU emulation) one batch at a time, under
    both clustering schedules."""
    bsp = O.RefEngine(egr_path, max_csr, O.BULK_SYNCHRONOUS)
    ser = O.RefEngine(egr_path, max_csr, O.SERIAL)
    bsp.set_mis(mis0)
    ser.set_mis(mis0)
    for i, (u, v, ins) in enumerate(batches):
        recs = bsp.apply_batch(u, v, ins)
        ser.apply_batch(u, v, ins)
        out["b%d_mis_ref" % i] = np.packbits(bsp.get_mis())
        out["b%d_cid_ref_sha" % i] = sha(bsp.cluster_ids().astype("<i4"))
        out["b%d_sb_ref" % i] = np.array(recs, np.int64).reshape(-1, 3)
        out["b%d_maxcsr_ref" % i] = np.int64(bsp.max_csr)
        out["b%d_mis_ref_serial" % i] = np.packbits(ser.get_mis())
    bsp.close()
    ser.close()


def capture_reference_mains(out, egr_path, batch_paths, mis0):
    """bin/misfit and bin/misfit_async (the engines' own main(), CPU
    emulation) on a copy of the inputs: final-MIS file and compacted bytes."""
    n = mis0.size
    for engine in ("sync", "async"):
        run = tempfile.mkdtemp()
        try:
            stem = "g"
            shutil.copy(egr_path, os.path.join(run, stem + ".egr"))
            W.write_mis_file(os.path.join(run, "mis.txt"), mis0)
            os.makedirs(os.path.join(run, "b"))
            for k, bp in enumerate(batch_paths):
                shutil.copy(bp, os.path.join(run, "b", "%d.mtx" % (k + 1)))
            rc, log = O.run_reference_main(engine, [stem + ".egr", "mis.txt", "b", len(batch_paths), 0], run)
            if rc != 0:
                raise SystemExit("reference %s main failed:\n%s" % (engine, log[-2000:]))
            fm = W.read_mis_file(os.path.join(run, "datasets", "Final_MISs", stem + "_flash_final_mis.txt"), n)
            out["main_%s_final_mis" % engine] = np.packbits(fm)
            data = open(os.path.join(run, stem + ".egr"), "rb").read()
            out["main_%s_compact_sha256" % engine] = np.frombuffer(hashlib.sha256(data).digest(), np.uint8)
        finally:
            shutil.rmtree(run)


def capture(name, egr_path, batch_paths, mis0, max_csr=None, twohop_seeds=40):
    ref = O.Reference(egr_path)
    orc = O.Oracle.open_egr(egr_path)
    n = orc.n
    n_, nindex, nlist, wide = W.read_egr(egr_path)
    out = {"n": np.int64(n), "nindex": nindex, "nlist": nlist, "wide": np.int64(wide), "mis0": mis0}
    if max_csr is not None:
        orc.max_csr = max_csr
        out["max_csr"] = np.int64(max_csr)
    out["initial_max_csr"] = np.int64(O.Oracle.open_egr(egr_path).max_csr)
    parsed = [ref.parse_batch_file(p) for p in batch_paths]
    orc.set_mis(mis0)
    for i, (u, v, ins) in enumerate(parsed):
        out["b%d_u" % i], out["b%d_v" % i], out["b%d_ins" % i] = u, v, ins
    out["num_batches"] = np.int64(len(parsed))
    for i, (u, v, ins) in enumerate(parsed):
        ref.apply_updates(u, v, ins)
        orc.trace(True)
        orc.apply_batch(u, v, ins)
        ip, ix = rows_csr(ref.row, n)
        out["b%d_rows_ptr" % i], out["b%d_rows_idx" % i] = ip, ix
        out["b%d_deg" % i] = np.array([ref.degree(x) for x in range(n)], np.int32)
        seeds = seeds_first_appearance(u, v)[:twohop_seeds]
        lists, hop1 = [], []
        for s in seeds.tolist():
            a, h = ref.two_hop(s)
            lists.append(a)
            hop1.append(h)
        out["b%d_2hop_seeds" % i] = seeds
        out["b%d_2hop_ptr" % i] = np.concatenate([[0], np.cumsum([len(a) for a in lists])]).astype(np.int64)
        out["b%d_2hop_idx" % i] = np.concatenate(lists).astype(np.int32)
        out["b%d_hop1_ptr" % i] = np.concatenate([[0], np.cumsum([len(a) for a in hop1])]).astype(np.int64)
        out["b%d_hop1_idx" % i] = np.concatenate(hop1).astype(np.int32) if hop1 else np.zeros(0, np.int32)
        out["b%d_mis_oracle" % i] = orc.get_mis()
        recs = orc.trace_records()
        out["b%d_trace_hdr" % i] = np.stack([r[0] for r in recs])
    capture_reference_engine(out, egr_path, parsed, mis0,
                             max_csr if max_csr is not None else int(out["initial_max_csr"]))
    if max_csr is None:   # main() sizes MAX_CSR_ELEMENTS itself
        capture_reference_mains(out, egr_path, batch_paths, mis0)
    tmp = tempfile.mkdtemp()
    try:
        cpath = os.path.join(tmp, "c.egr")
        ref.compact(cpath)
        data = open(cpath, "rb").read()
        out["compact_sha256"] = np.frombuffer(hashlib.sha256(data).digest(), np.uint8)
        out["compact_len"] = np.int64(len(data))
    finally:
        shutil.rmtree(tmp)
    ref.close()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name, "batches", len(parsed))


def capture_cfg1(tmp):
    """Config 1: ER G(10000, avg 8), int32 .egr, seed 42; 10 batch files of
    2000 toggles (1000 deletes of existing edges, 1000 inserts of
    non-adjacent pairs)."""
    n = 10000
    ni, nl = W.er_graph(n, 8, 42)
    p = os.path.join(tmp, "er10k.egr")
    W.write_egr(p, n, ni, nl)
    ts = W.ToggleStream(n, ni, nl, 42)
    pairs = [ts.next_batch(2000) for _ in range(10)]
    W.write_batch_folder(os.path.join(tmp, "cfg1b"), pairs)
    paths = [os.path.join(tmp, "cfg1b", "%d.mtx" % (i + 1)) for i in range(10)]
    ref = O.Reference(p)
    parsed = [ref.parse_batch_file(q) for q in paths]
    ref.close()
    mis0 = O.greedy_mis(ni, nl)
    out = {"n": np.int64(n), "nindex": ni.astype(np.int32), "nlist": nl, "mis0": np.packbits(mis0),
           "num_batches": np.int64(len(parsed)),
           "initial_max_csr": np.int64(O.Oracle.open_egr(p).max_csr)}
    for i, (u, v, ins) in enumerate(parsed):
        out["b%d_u" % i], out["b%d_v" % i], out["b%d_ins" % i] = u, v, ins
    capture_reference_engine(out, p, parsed, mis0, int(out["initial_max_csr"]))
    capture_reference_mains(out, p, paths, mis0)
    np.savez_compressed(os.path.join(HERE, "cfg1.npz"), **out)
    print("wrote cfg1 batches", len(parsed))


def main():
    refroot = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MISFIT_REF_ROOT")
    if not refroot:
        raise SystemExit("usage: make_golden.py <reference_root>  (or set MISFIT_REF_ROOT)")
    os.environ["MISFIT_REF_ROOT"] = refroot
    from oracle import build as OB
    OB.build_ref(refroot)
    OB.build_ref_emul(refroot)
    if O.ref_lib() is None or O.ref_emul_lib("sync") is None or O.ref_emul_lib("async") is None:
        raise SystemExit("reference harness unavailable")
    tmp = tempfile.mkdtemp()
    try:
        # 1. the reference's bundled sample (int64-sentinel .egr, delete-only batches)
        sample = os.path.join(refroot, "datasets", "sample")
        shutil.copy(os.path.join(sample, "sample.egr"), os.path.join(tmp, "sample.egr"))
        n, ni, nl, _ = W.read_egr(os.path.join(tmp, "sample.egr"))
        mis0 = W.read_mis_file(os.path.join(sample, "sample_mis.txt"), n)
        assert np.array_equal(O.greedy_mis(ni, nl), mis0), "sample_mis.txt is not the greedy MIS"
        bdir = os.path.join(sample, "batches")
        files = O.ref_list_batch_files(bdir)
        capture("sample", os.path.join(tmp, "sample.egr"), [os.path.join(bdir, f) for f in files], mis0)

        # 2. ER(1500, 8) int32 .egr with insert/delete toggles
        n = 1500
        ni, nl = W.er_graph(n, 8, 42)
        W.write_egr(os.path.join(tmp, "er.egr"), n, ni, nl)
        ts = W.ToggleStream(n, ni, nl, 5)
        W.write_batch_folder(os.path.join(tmp, "erb"), [ts.next_batch(300) for _ in range(5)])
        capture("er1500", os.path.join(tmp, "er.egr"),
                [os.path.join(tmp, "erb", "%d.mtx" % (i + 1)) for i in range(5)], O.greedy_mis(ni, nl))

        # 3. small R-MAT with hubs, a small MAX_CSR_ELEMENTS so that the split
        #    rule cuts sub-batches and the limit grows
        n, (ni, nl) = W.rmat_graph(10, 8, 3)
        W.write_egr(os.path.join(tmp, "rmat.egr"), n, ni, nl, wide=True)
        ts = W.ToggleStream(n, ni, nl, 9)
        W.write_batch_folder(os.path.join(tmp, "rmb"), [ts.next_batch(200) for _ in range(4)])
        capture("rmat10", os.path.join(tmp, "rmat.egr"),
                [os.path.join(tmp, "rmb", "%d.mtx" % (i + 1)) for i in range(4)], O.greedy_mis(ni, nl),
                max_csr=60000)

        # 4. the same R-MAT with a limit below the packed 2-hop volume, so that
        #    MAX_CSR_ELEMENTS grows during packing (src/misfit/misfit.cu:565-583)
        capture("rmat10g", os.path.join(tmp, "rmat.egr"),
                [os.path.join(tmp, "rmb", "%d.mtx" % (i + 1)) for i in range(4)], O.greedy_mis(ni, nl),
                max_csr=2000)

        # 5. the config-1 stream
        capture_cfg1(tmp)
    finally:
        shutil.rmtree(tmp)


if __name__ == "__main__":
    main()
