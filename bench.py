"""Benchmark: MISFIT dynamic-MIS maintenance, plain per-batch loop.

Workload (the plain method at scale): R-MAT scale 22 (4,194,304 vertices,
16 undirected samples per vertex, a,b,c,d = .57/.19/.19/.05, symmetrised,
de-duplicated, self-loops removed), seed 7, int32 .egr layout; batches of
100,000 toggles, half deletes of uniformly sampled existing edges and half
inserts of uniformly sampled non-adjacent pairs, drawn against the nominal
graph as it evolves; parse-time flags against the base graph, as the
reference CLI computes them.  Seeded synthetic data; the graph is built on
the GPU with torch (input preparation only).

One step = one batch through libmisfit_gb (overlay apply, split rule,
neighbourhoods, clustering, repair).  `value` is updates/s with the batch
inputs resident in HBM (mf_apply_batch_device); `e2e` is the same through
the host-buffer C-ABI call (mf_apply_batch: host->device copy of the batch
inside the timed region) plus a device->host read of the membership vector
after every step.  Times come from CUDA events the library records on its
own stream around each batch.

--impl reference runs the oracle (the reference path restated on the CPU,
OpenMP over all host cores) on bounded samples of the same workload.

Multi-GPU: the path does not shard within one graph (replicas only); under
torchrun every rank runs its own replica and `value` sums the ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "edge updates/s and p50/p99 batch latency, served vs plain loop, 1 GB300, exact MIS"
# What the line's top-level value is; the served, batched and exact-MIS
# figures of the same metric are the sub-objects "served", "batched" and
# "exact_mode".
VALUE_IS = ("plain per-batch loop (the reference's method, compat mode) on the R-MAT scale-22 workload; "
            "served and batched forms in 'served' / 'batched', exact-MIS mode in 'exact_mode'")
UNIT = "updates/s"

# DRAM bytes (read + write) per pushed element of k_lb_push_hop, measured by
# ncu on this workload (R-MAT scale 22, the bench's first batch):
# dram__bytes_read.sum + dram__bytes_write.sum over the kernel's launches
# 200-202 (135,575,040 bytes) divided by their pushed elements (9,720,762,
# printed with MISFIT_GB_DEBUG=2).  ncu flushes the caches before each
# launch, so this is a cold-L2 figure; 12 bytes per element are algorithmic.
PUSH_HOP_DRAM_BYTES_PER_ELEMENT = 13.95
# DRAM bytes (read + write) per launch of k_pull_cand on this workload: ncu
# over the kernel's launches 100-102 of the bench's first batch (cold L2),
# 699,086,592 bytes in three launches.  Its launches read every vertex's row
# bounds, so their traffic hardly varies from one sub-batch to the next.
PULL_DRAM_BYTES_PER_LAUNCH = 233028864


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="misfit", choices=["misfit", "reference"])
    ap.add_argument("--scale", type=int, default=22)
    ap.add_argument("--edge-factor", type=int, default=16)
    ap.add_argument("--batch", type=int, default=100000)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="CPU-baseline sample budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-served", action="store_true", help="skip the served and batched legs")
    ap.add_argument("--no-exact", action="store_true", help="skip the exact-MIS leg")
    ap.add_argument("--batched-graphs", type=int, default=256, help="graphs of the batched form")
    ap.add_argument("--served-graphs", type=int, default=1000, help="resident graphs of the serving form")
    ap.add_argument("--graphs-nmax", type=int, default=1000000,
                    help="largest vertex count of the served/batched graph sets (log-uniform from 1,000)")
    ap.add_argument("--served-requests", type=int, default=1000, help="requests per arrival rate")
    ap.add_argument("--served-rates", default="2000,10000,50000", help="Poisson arrival rates per second")
    ap.add_argument("--served-workers", type=int, default=8)
    ap.add_argument("--served-budget", type=float, default=0.6, help="HBM budget as a fraction of the footprint")
    ap.add_argument("--served-cta-limit", type=int, default=512,
                    help="largest request the served form's continuous batching gives to the persistent kernel")
    ap.add_argument("--served-cta-vertices", type=int, default=65536,
                    help="largest graph whose requests the served form's continuous batching gives to the "
                         "persistent kernel (one CTA walks every vertex of its graph in some stages)")
    ap.add_argument("--no-large", action="store_true", help="skip the 64-bit-layout leg (R-MAT scale 26)")
    ap.add_argument("--large-only", action="store_true", help="run only the 64-bit-layout leg and print its JSON")
    ap.add_argument("--large-scale", type=int, default=26)
    ap.add_argument("--large-edge-factor", type=int, default=20)
    ap.add_argument("--large-batch", type=int, default=1000000, help="toggles per batch of the large leg")
    ap.add_argument("--large-seconds", type=float, default=60.0,
                    help="device-time budget of the large leg's timed sample")
    ap.add_argument("--large-dir", default=None, help="folder for the large .egr file (default: the system temp)")
    ap.add_argument("--large-max-csr", type=int, default=0,
                    help="MAX_CSR_ELEMENTS to start the large leg from (default: the reference's initial value)")
    ap.add_argument("--large-pull-sizes", type=int, default=-1, choices=[-1, 0, 1, 2],
                    help="tuning pull_sizes of the large leg (-1: the library default)")
    ap.add_argument("--served-only", action="store_true", help="run only the served leg and print its JSON")
    ap.add_argument("--batched-only", action="store_true",
                    help="run only the batched-form leg and print its JSON (profiling runs)")
    ap.add_argument("--no-autotune", action="store_true", help="batched leg with the library's default settings")
    ap.add_argument("--profile-step", action="store_true",
                    help="one batched step only (every batch in the persistent kernel, plain launch, batches "
                         "capped at 8192 lines, no plain-loop or pool legs): the command profiled by ncu")
    return ap.parse_args()


def workload_config(args):
    return {
        "workload": "R-MAT scale %d, %d samples/vertex, abcd .57/.19/.19/.05, seed %d; batches of %d toggles "
                    "(50/50 delete existing / insert non-adjacent, uniform)" % (
                        args.scale, args.edge_factor, args.seed, args.batch),
        "vertices": 1 << args.scale,
        "batch_updates": args.batch,
        "parallelism": "replicas" if args.gpus > 1 else "single GPU",
        "l2": "inputs larger than L2 (base CSR ~0.5 GB)",
        "flags": "parse-time, against the base graph",
    }


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def stop(self, window=None):
        """Stop sampling; summarise the samples read inside `window` (host
        perf_counter seconds, with one sampling period of slack), all samples
        when it is None."""
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for t, line in self.lines:
            if window is not None and not (window[0] <= t <= window[1] + 0.25):
                continue
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(args, device):
    from misfit_gb300 import workloads as W
    n, (nindex, nlist) = W.rmat_graph_torch(args.scale, args.edge_factor, args.seed, device=device)
    stream = W.ToggleStream(n, nindex, nlist, args.seed)
    return n, nindex, nlist, stream


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_sample(n, nindex, nlist, batch, ins, budget_s):
    """Oracle on the first lines of `batch`, from the initial state, in chunks
    that double until the budget is spent.  Returns (updates/s, lines, s)."""
    import oracle as O
    orc = O.Oracle.from_csr(nindex, nlist)
    orc.set_mis(O.greedy_mis(nindex, nlist))
    u, v = batch
    done, spent, chunk = 0, 0.0, 16
    while done < u.size and spent < budget_s:
        k = min(chunk, u.size - done)
        t = time.perf_counter()
        orc.apply_batch(u[done:done + k], v[done:done + k], ins[done:done + k])
        spent += time.perf_counter() - t
        done += k
        chunk *= 2
    orc.close()
    return done / spent, done, spent


def cpu_greedy(nindex, nlist, batches, flags):
    """The from-scratch alternative on the host cores: each batch applied to
    the overlay, then the greedy MIS of tools/compute_initial_mis.py
    recomputed over the whole current graph, single-threaded as that tool
    is.  It yields the exact greedy MIS after every batch, not the
    reference's repair result; it is a baseline, not a check."""
    import oracle as O
    orc = O.Oracle.from_csr(nindex, nlist)
    spent, lines = 0.0, 0
    for (u, v), ins in zip(batches, flags):
        t = time.perf_counter()
        orc.apply_overlay(u, v, ins)
        orc.greedy_current()
        spent += time.perf_counter() - t
        lines += int(u.size)
    orc.close()
    return {"value": lines / spent, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "%d batches (%d lines): overlay apply + greedy recompute over the whole graph, %.1f s"
                      % (len(batches), lines, spent)}


def run_reference(args, rank):
    """The reference arm: the reference path restated on the CPU (the oracle,
    OpenMP over all host cores) on the same batches, state carried from step
    to step.  One oracle holds the graph and the membership for the whole
    run.  Each step times the leading lines of its batch through the whole
    path (overlay apply, split, neighbourhoods, clustering, repair) in
    doubling chunks until the per-step budget is spent, then applies the
    batch's remaining lines to the overlay only (untimed), so that the next
    step starts from the graph the full batch leaves.  The membership evolves
    through the timed lines only.  `value` is the timed lines over the time
    spent on them; `ms_per_step` is that time per step (what the run really
    spent), and each step's timed lines are listed."""
    if rank != 0:
        return
    import torch
    device = "cuda:%d" % int(os.environ.get("LOCAL_RANK", "0")) if torch.cuda.is_available() else "cpu"
    n, nindex, nlist, stream = make_workload(args, device)
    import oracle as O
    orc0 = O.Oracle.from_csr(nindex, nlist)          # flags against the base graph
    orc = O.Oracle.from_csr(nindex, nlist)           # the evolving state
    orc.set_mis(O.greedy_mis(nindex, nlist))
    cores = os.cpu_count()
    budget = max(2.0, args.cpu_seconds / 2)
    timed_lines, timed_s, per_step = 0, 0.0, []
    for i in range(args.warmup + args.steps):
        u, v = stream.next_batch(args.batch)
        ins = orc0.flag_updates(u, v)
        done, spent, chunk = 0, 0.0, 16
        while done < u.size and spent < budget:
            k = min(chunk, u.size - done)
            t = time.perf_counter()
            orc.apply_batch(u[done:done + k], v[done:done + k], ins[done:done + k])
            spent += time.perf_counter() - t
            done += k
            chunk *= 2
        if done < u.size:
            orc.apply_overlay(u[done:], v[done:], ins[done:])
        if i >= args.warmup:
            timed_lines += done
            timed_s += spent
            per_step.append(done)
    orc.close()
    orc0.close()
    value = timed_lines / timed_s
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": timed_s / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded R-MAT + toggle stream)", "config": workload_config(args),
        "step": "a bounded sample of one batch: its leading lines through the whole path, ~%.0f s each, "
                "on the state every earlier batch left (graph: all lines; membership: the timed lines)" % budget,
        "lines_timed_per_step": per_step, "sampled_fraction": timed_lines / float(args.steps * args.batch),
        "extrapolated": False,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "oracle (reference path restated, OpenMP %d threads): %d lines over %d steps "
                                   "(%.1f s), the leading lines of each batch on the evolving state"
                                   % (cores, timed_lines, args.steps, timed_s)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---- the 64-bit layout at scale ---------------------------------------------------------

def run_large(args, local):
    """R-MAT scale 26 (67,108,864 vertices), 20 undirected samples per vertex,
    a,b,c,d = .57/.19/.19/.05, symmetrised and de-duplicated: more than 2^31
    directed entries, so the .egr file takes the int64-sentinel layout.  The
    graph is written to disk and opened through mf_open_egr (chunked pinned
    reads, asynchronous copies).  Batches hold 1,000,000 toggles, 50/50
    deletes and inserts, both endpoints proportional to current degree
    (deletes: uniform over the edges; inserts: endpoints drawn by degree,
    pairs not adjacent in the base graph).  Under the reference's split rule
    a batch with hub endpoints packs 2-hop lists of tens of millions of
    entries per seed, so the leg times a bounded sample: consecutive
    prefixes of the first batch (25 lines, then doubling), each applied as a
    batch, until a quarter of the budget of device time is spent; then one
    last prefix sized to fill the rest, the largest (a batch keeps its
    exact 2-hop sizes for all its sub-batches, as a full batch would);
    then one more 25-line prefix in exact-MIS mode, after which the
    membership is checked for independence and maximality on the whole
    graph."""
    import torch
    from misfit_gb300 import native
    from misfit_gb300 import workloads as W
    import tempfile
    dev = "cuda:%d" % local
    out = {"workload": "R-MAT scale %d, %d samples/vertex, abcd .57/.19/.19/.05, seed %d; batches of %d toggles, "
                       "50/50, endpoints proportional to degree" % (args.large_scale, args.large_edge_factor,
                                                                     args.seed, args.large_batch)}
    t = time.perf_counter()
    n, (nindex, nlist) = W.rmat_graph_torch(args.large_scale, args.large_edge_factor, args.seed, device=dev)
    torch.cuda.empty_cache()
    out["generate_s"] = time.perf_counter() - t
    out["vertices"] = int(n)
    out["directed_entries"] = int(nlist.size)
    out["beyond_2_31"] = bool(nlist.size > 0x7FFFFFFF)
    folder = args.large_dir or tempfile.gettempdir()
    path = os.path.join(folder, "misfit_rmat%d_%d.egr" % (args.large_scale, os.getpid()))
    g = None
    try:
        t = time.perf_counter()
        W.write_egr(path, n, nindex, nlist)
        out["write_s"] = time.perf_counter() - t
        out["file_bytes"] = os.path.getsize(path)
        with open(path, "rb") as f:
            out["layout"] = "int64-sentinel" if struct_unpack_second_int(f.read(8)) == -1 else "int32"
        t = time.perf_counter()
        g = native.Graph.open_egr(path, gpu=local)
        out["ingest_s"] = time.perf_counter() - t
        if args.large_max_csr > 0:
            g.max_csr = args.large_max_csr
            out["max_csr_start"] = args.large_max_csr
        if args.large_pull_sizes >= 0:
            g.set_tuning(pull_sizes=args.large_pull_sizes)
            out["pull_sizes"] = args.large_pull_sizes
        out["ingest_gbs"] = out["file_bytes"] / out["ingest_s"] / 1e9
        t = time.perf_counter()
        mis0 = g.greedy_mis()
        g.set_mis(mis0)
        out["greedy_seed_s"] = time.perf_counter() - t

        def adjacent(a, b):
            f = g.flag_updates(a.to(torch.int32).cpu().numpy(), b.to(torch.int32).cpu().numpy())
            return torch.from_numpy(f == 0).to(a.device)

        toggles = W.DeviceToggles(nindex, nlist, args.seed + 1, device=dev, adjacent=adjacent)
        del nlist
        u, v, ins = toggles.next_batch(args.large_batch, endpoints="preferential")
        del toggles
        torch.cuda.empty_cache()
        g.profile(1)
        g.profile_reset()
        budget_ms = args.large_seconds * 1e3
        done, dev_ms, sub, chunk, samples = 0, 0.0, 0, 25, []
        while done < u.size:
            k = min(chunk, u.size - done)
            if samples:
                # the next prefix's expected time from the last one's per-line
                # time; the last prefix takes what fits in the rest of the budget
                last = samples[-1]
                per_line = last["device_ms"] / last["lines"]
                fit = int(0.85 * (budget_ms - dev_ms) / per_line)
                # past a quarter of the budget, one last prefix takes the rest
                k = min(fit if dev_ms >= budget_ms / 4 else min(k, fit), u.size - done)
                if k < 25:
                    break
            g.apply_batch(u[done:done + k], v[done:done + k], ins[done:done + k])
            st = g.stats()
            dev_ms += st["device_ms"]
            sub += st["sub_batches"]
            samples.append({"lines": k, "device_ms": round(st["device_ms"], 3), "sub_batches": st["sub_batches"],
                            "max_csr": st["max_csr"]})
            done += k
            chunk *= 2
        prof = g.profile_read()
        g.profile(False)
        rate = done / (dev_ms / 1e3)
        out.update({"value": rate, "unit": UNIT, "lines_timed": done, "device_ms": dev_ms,
                    "sub_batches": sub, "sub_batches_per_line": sub / max(done, 1), "samples": samples,
                    "projected_s_per_batch": args.large_batch / rate,
                    "stage_ms": {s: round(x[0], 1) for s, x in prof.items() if x[0] > 0},
                    "timing": "library CUDA events per applied prefix (host-buffer batches); prefixes of 25 "
                              "lines, doubling, until a quarter of the budget is spent, then one prefix "
                              "sized to fill the rest"})
        ms, calls, nbytes = prof["push_hop"]
        peak, peak_kind = measured_peaks()
        if ms > 0:
            ach = nbytes / (ms / 1e3) / 1e9
            out["roofline"] = {"bound": "hbm", "kernel": "k_lb_push_hop", "achieved": ach, "peak": peak,
                               "unit": "GB/s", "frac": ach / peak, "peak_kind": peak_kind, "launches": int(calls)}
        # exact-MIS mode on one more prefix, then the checks on the whole graph
        k = min(25, u.size - done)
        if k > 0:
            g.set_exact(True)
            g.apply_batch(u[done:done + k], v[done:done + k], ins[done:done + k])
            viol, unc = g.check_mis()
            g.set_exact(False)
            out["exact_check"] = {"lines": int(k), "device_ms": g.stats()["device_ms"],
                                  "violations": int(viol), "uncovered": int(unc)}
    finally:
        if g is not None:
            g.close()
        if os.path.exists(path):
            os.remove(path)
    return out


def struct_unpack_second_int(head):
    import struct
    return struct.unpack("<ii", head)[1]


# ---- served and batched forms (many graphs on one GPU) ------------------------------

def graph_set(count, nmin, nmax, seed, device="cuda"):
    """2-D random geometric graphs with log-uniform vertex counts in [nmin,
    nmax] and mean degree uniform in 4..32, one seed per graph, built on the
    GPU (workloads.rgg_graph_torch)."""
    from misfit_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        nindex, nlist = W.rgg_graph_torch(n, float(rng.uniform(4, 32)), seed * 1000 + k, device=device)
        out.append((n, nindex, nlist))
    return out


def initial_mis(graphs):
    from misfit_gb300 import native
    mis = []
    for n, nindex, nlist in graphs:
        g = native.Graph.from_csr(nindex, nlist)
        mis.append(g.greedy_mis())
        g.close()
    return mis


def plain_loop(graphs, mis0, reqs):
    """One dedicated context per graph, requests applied one after another in
    arrival order (waiting for each arrival).  Returns (updates/s, latencies
    ms, final memberships)."""
    from misfit_gb300 import native
    ctxs = []
    for (n, nindex, nlist), m in zip(graphs, mis0):
        g = native.Graph.from_csr(nindex, nlist)
        g.set_mis(m)
        ctxs.append(g)
    lat = []
    t0 = time.perf_counter()
    for t, gid, u, v, ins in reqs:
        wait = t - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        ctxs[gid].apply_batch(u, v, ins)
        lat.append((time.perf_counter() - t0 - t) * 1e3)
    span = time.perf_counter() - t0
    out = [c.get_mis() for c in ctxs]
    for c in ctxs:
        c.close()
    updates = sum(int(r[2].size) for r in reqs)
    return updates / span, lat, out


def pooled(graphs, mis0, reqs, workers, budget_frac, batching=None):
    """The same requests through a serving pool: submitted at their arrival
    times, served by `workers` threads under budget_frac of the graphs' HBM
    footprint (with `batching` mf_batched_opts: small requests in
    continuous-batching steps of the persistent kernel).  Returns
    (updates/s, latencies ms, memberships, pool stats)."""
    from misfit_gb300 import native
    pool = native.Pool(1 << 40, workers=workers)
    if batching is not None:
        pool.set_batching(batching)
    gids = [pool.add_graph(nindex, nlist, m) for (n, nindex, nlist), m in zip(graphs, mis0)]
    footprint = pool.stats()["resident_bytes"]
    pool.set_budget(max(1, int(footprint * budget_frac)))
    rids = []
    t0 = time.perf_counter()
    for t, gid, u, v, ins in reqs:
        wait = t - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        rids.append(pool.submit(gids[gid], u, v, ins))
    lat = [pool.wait(r) for r in rids]
    span = time.perf_counter() - t0
    out = [pool.get_mis(g) for g in gids]
    st = pool.stats()
    st["footprint_bytes"] = footprint
    pool.close()
    updates = sum(int(r[2].size) for r in reqs)
    return updates / span, lat, out, st


SIZE_BUCKETS = ((10, 100), (101, 1000), (1001, 10000), (10001, 20000))


def latency_summary(lat, sizes):
    lat = np.asarray(lat, dtype=np.float64)
    sizes = np.asarray(sizes)
    out = {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
           "by_size": {}}
    for lo, hi in SIZE_BUCKETS:
        sel = (sizes >= lo) & (sizes <= hi)
        if sel.any():
            out["by_size"]["%d-%d" % (lo, hi)] = {"requests": int(sel.sum()),
                                                 "p50_ms": float(np.percentile(lat[sel], 50)),
                                                 "p99_ms": float(np.percentile(lat[sel], 99))}
    return out


def run_served(args, graphs, mis0, batching, device):
    """Serving form: resident graphs drawn as in the batched form; for each
    Poisson arrival rate of the sweep, `served_requests` requests, each one
    batch of log-uniform 10..20,000 toggles to a graph chosen Zipf(1.1),
    endpoints uniform, preferential or low-degree (1/3 each), drawn on the
    GPU against the graph's base CSR.  The rates run one after another on
    the same graphs, in the pool (worker threads, HBM budget 60% of the
    graphs' footprint, so graphs are evicted to pinned host memory and
    restored), in the pool with continuous batching of the small requests,
    and in the plain sequential loop (one dedicated context per graph, each
    request applied at its arrival or when the previous one ends).  Latency
    is arrival to completion; every graph's final membership must be the
    same in all three."""
    from misfit_gb300 import native
    from misfit_gb300 import workloads as W
    rates = [float(x) for x in args.served_rates.split(",")]
    rng = np.random.default_rng(11)
    zipf = np.arange(1, len(graphs) + 1, dtype=np.float64) ** -1.1
    zipf /= zipf.sum()
    modes = ["uniform", "preferential", "low_degree"]
    plan = []
    for ri, rate in enumerate(rates):
        t = 0.0
        for _ in range(args.served_requests):
            t += float(rng.exponential(1.0 / rate))
            gid = int(rng.choice(len(graphs), p=zipf))
            size = int(round(np.exp(rng.uniform(np.log(10), np.log(20000)))))
            plan.append((ri, t, gid, size, modes[int(rng.integers(3))]))
    t0 = time.perf_counter()
    by_gid = {}
    for idx, r in enumerate(plan):
        by_gid.setdefault(r[2], []).append(idx)
    batch_of = [None] * len(plan)
    for gid, idxs in by_gid.items():
        n, ni, nl = graphs[gid]
        dt = W.DeviceToggles(ni, nl, 500 + gid, device=device)
        for idx in idxs:
            batch_of[idx] = dt.next_batch(plan[idx][3], endpoints=plan[idx][4])
        del dt
    gen_s = time.perf_counter() - t0
    per_rate = [[(plan[i][1], plan[i][2]) + batch_of[i] for i in range(len(plan)) if plan[i][0] == ri]
                for ri in range(len(rates))]

    p_res = plain_sweep(graphs, mis0, per_rate)
    s_res = pool_sweep(graphs, mis0, per_rate, args.served_workers, args.served_budget)
    lat_opts = native.batched_opts(block=batching.block, ctas_per_sm=batching.ctas_per_sm,
                                   max_cta_updates=min(int(args.served_cta_limit), batching.max_cta_updates),
                                   max_cta_vertices=min(int(args.served_cta_vertices), batching.max_cta_vertices))
    c_res = pool_sweep(graphs, mis0, per_rate, args.served_workers, args.served_budget, lat_opts)
    same = all(np.array_equal(a, b) for a, b in zip(p_res["mis"], s_res["mis"]))
    same_c = all(np.array_equal(a, b) for a, b in zip(p_res["mis"], c_res["mis"]))
    sweep = []
    for ri, rate in enumerate(rates):
        sizes = [int(r[2].size) for r in per_rate[ri]]
        updates = int(sum(sizes))
        sweep.append({
            "rate_per_s": rate, "requests": len(sizes), "updates": updates,
            "pool": {"value": updates / s_res["span"][ri], "unit": UNIT,
                     **latency_summary(s_res["lat"][ri], sizes)},
            "pool_continuous_batching": {"value": updates / c_res["span"][ri], "unit": UNIT,
                                         **latency_summary(c_res["lat"][ri], sizes)},
            "plain_loop": {"value": updates / p_res["span"][ri], "unit": UNIT,
                           **latency_summary(p_res["lat"][ri], sizes)},
            "pool_vs_plain": (updates / s_res["span"][ri]) / (updates / p_res["span"][ri]),
        })
    st = s_res["stats"]
    return {
        "workload": "%d RGGs (n log-uniform 1e3..%.0e, mean degree 4..32, built on the GPU); per rate %d "
                    "requests, Poisson arrivals, batches log-uniform 10..20000 toggles, graph Zipf(1.1), endpoints "
                    "uniform/preferential/low-degree" % (len(graphs), args.graphs_nmax, args.served_requests),
        "sweep": sweep, "value": sweep[0]["pool"]["value"], "unit": UNIT,
        "p50_ms": sweep[0]["pool"]["p50_ms"], "p99_ms": sweep[0]["pool"]["p99_ms"],
        "p99_target_ms": 5.0, "workers": args.served_workers, "hbm_budget_fraction": args.served_budget,
        "footprint_bytes": st["footprint_bytes"], "peak_resident_bytes": st["peak_resident_bytes"],
        "evictions": st["evictions"], "restores": st["restores"], "scratch_trims": st["trims"],
        "continuous_batching": {"steps": c_res["stats"]["batched_steps"],
                                "requests_in_steps": c_res["stats"]["batched_requests"],
                                "handed_to_idle_workers": c_res["stats"]["handed_to_workers"],
                                "settings": {k: getattr(lat_opts, k) for k, _ in lat_opts._fields_}},
        "identical_to_plain_loop": bool(same), "continuous_batching_identical_to_plain_loop": bool(same_c),
        "request_generation_s": gen_s,
        "timing": "host wall clock from each request's arrival to its completion; host buffers in",
    }


def plain_sweep(graphs, mis0, per_rate):
    """The plain sequential loop over the rates' requests (dedicated contexts,
    state carried from rate to rate)."""
    from misfit_gb300 import native
    ctxs = []
    for (n, nindex, nlist), m in zip(graphs, mis0):
        g = native.Graph.from_csr(nindex, nlist)
        g.set_mis(m)
        ctxs.append(g)
    lats, spans = [], []
    for reqs in per_rate:
        lat = []
        t0 = time.perf_counter()
        for t, gid, u, v, ins in reqs:
            wait = t - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            ctxs[gid].apply_batch(u, v, ins)
            lat.append((time.perf_counter() - t0 - t) * 1e3)
        spans.append(time.perf_counter() - t0)
        lats.append(lat)
    out = [c.get_mis() for c in ctxs]
    for c in ctxs:
        c.close()
    return {"lat": lats, "span": spans, "mis": out}


def pool_sweep(graphs, mis0, per_rate, workers, budget_frac, batching=None):
    """The same requests through one serving pool, rate after rate."""
    from misfit_gb300 import native
    pool = native.Pool(1 << 40, workers=workers)
    if batching is not None:
        pool.set_batching(batching)
    gids = [pool.add_graph(nindex, nlist, m) for (n, nindex, nlist), m in zip(graphs, mis0)]
    footprint = pool.stats()["resident_bytes"]
    pool.set_budget(max(1, int(footprint * budget_frac)))
    lats, spans = [], []
    for reqs in per_rate:
        rids = []
        t0 = time.perf_counter()
        for t, gid, u, v, ins in reqs:
            wait = t - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            rids.append(pool.submit(gids[gid], u, v, ins))
        lat = [pool.wait(r) for r in rids]
        spans.append(time.perf_counter() - t0)
        lats.append(lat)
    out = [pool.get_mis(g) for g in gids]
    st = pool.stats()
    st["footprint_bytes"] = footprint
    pool.close()
    return {"lat": lats, "span": spans, "mis": out, "stats": st}


def run_batched(args, graphs, mis0, device):
    """Batched form: independent graphs, one batch each (log-uniform
    10..50,000 toggles, low-degree and uniform endpoints 50/50, drawn on the
    GPU against each graph's base CSR),
    all applied in one mf_apply_batches step -- the batches one CTA can carry
    in one persistent kernel driven by a device work queue and launched as a
    CUDA graph, the rest through the multi-launch path meanwhile -- with the
    kernel's settings chosen by the autotuner on this workload.  Compared
    with the plain per-graph loop and with the serving pool given every
    batch at once; per-graph memberships must be identical."""
    from misfit_gb300 import autotune
    from misfit_gb300 import workloads as W
    rng = np.random.default_rng(12)
    reqs = []
    for k, (n, ni, nl) in enumerate(graphs):
        size = int(round(np.exp(rng.uniform(np.log(10), np.log(50000)))))
        mode = "low_degree" if k % 2 == 0 else "uniform"
        u, v, ins = W.DeviceToggles(ni, nl, 900 + k, device=device).next_batch(size, endpoints=mode)
        reqs.append((0.0, k, u, v, ins))
    batches = [(u, v, ins) for _, _, u, v, ins in reqs]
    updates = sum(int(b[0].size) for b in batches)
    p_rate, _, p_mis = plain_loop(graphs, mis0, reqs)
    s_rate, _, s_mis, st = pooled(graphs, mis0, reqs, args.served_workers, 1.0)
    if getattr(args, "no_autotune", False):
        from misfit_gb300 import native
        opts, report = native.batched_opts(), {"trials": []}
    else:
        opts, report = autotune.tune_batched(graphs, mis0, batches, use_cache=False)
    secs, b_mis, bst = [], None, None
    for _ in range(3):
        sec, b_mis, bst = autotune.run_step(graphs, mis0, batches, opts)
        secs.append(sec)
    b_rate = updates / float(np.median(secs))
    same = all(np.array_equal(a, b) for a, b in zip(p_mis, s_mis))
    same_b = all(np.array_equal(a, b) for a, b in zip(p_mis, b_mis))
    chosen = {k: getattr(opts, k) for k, _ in opts._fields_}
    return {
        "workload": "%d RGGs (n log-uniform 1e3..%.0e), one batch each of log-uniform 10..50000 toggles" % (
            len(graphs), args.graphs_nmax),
        "value": b_rate, "unit": UNIT,
        "step_ms": float(np.median(secs)) * 1e3, "kernel_ms": bst["kernel_ms"],
        "kernel_items": bst["kernel_items"], "path_items": bst["path_items"],
        "kernel_updates": int(sum(int(b[0].size) for b in batches if b[0].size <= chosen["max_cta_updates"])),
        "autotuned": chosen, "autotune_trials": [(t["opts"], round(t["seconds"] * 1e3, 2)) for t in report["trials"]],
        "plain_loop": {"value": p_rate, "unit": UNIT},
        "pool": {"value": s_rate, "unit": UNIT, "workers": args.served_workers,
                 "identical_to_plain_loop": bool(same)},
        "identical_to_plain_loop": bool(same_b),
        "timing": "host wall clock of one step on fresh contexts (median of 3), host buffers in, memberships out",
    }, opts


def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "misfit" else "gloo")
    if args.impl == "reference":
        run_reference(args, rank)
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        return

    import torch
    torch.cuda.set_device(local)
    from misfit_gb300 import build, native
    build.build()
    dev = "cuda:%d" % local
    if args.profile_step:
        from misfit_gb300 import autotune
        from misfit_gb300 import workloads as W
        graphs = graph_set(args.batched_graphs, 1000, args.graphs_nmax, 12, dev)
        mis0 = initial_mis(graphs)
        rng = np.random.default_rng(12)
        batches = []
        for k, (n, ni, nl) in enumerate(graphs):
            size = min(8192, int(round(np.exp(rng.uniform(np.log(10), np.log(50000))))))
            batches.append(W.DeviceToggles(ni, nl, 900 + k, device=dev).next_batch(size))
        opts = native.batched_opts(max_cta_updates=1 << 20, use_graph=0)
        sec, _, st = autotune.run_step(graphs, mis0, batches, opts)
        print(json.dumps({"graphs": len(graphs), "updates": int(sum(b[0].size for b in batches)),
                          "step_ms": sec * 1e3, **st}))
        return
    if args.served_only:
        graphs = graph_set(args.served_graphs, 1000, args.graphs_nmax, 11, dev)
        print(json.dumps(run_served(args, graphs, initial_mis(graphs), native.batched_opts(), dev)))
        return
    if args.batched_only:
        graphs = graph_set(args.batched_graphs, 1000, args.graphs_nmax, 12, dev)
        res, _ = run_batched(args, graphs, initial_mis(graphs), dev)
        res["gpu_launches_total"] = int(native.load_library().mf_kernel_launches())
        print(json.dumps(res))
        return
    if args.large_only:
        print(json.dumps(run_large(args, local)))
        return
    n, nindex, nlist, stream = make_workload(args, "cuda:%d" % local)
    g = native.Graph.from_csr(nindex, nlist, gpu=local)
    g.set_mis(g.greedy_mis())
    # warm-up, timed, e2e, one untimed batch with every stage timed, then the
    # exact-MIS leg (one warm-up and `steps` timed batches)
    exact_steps = 0 if args.no_exact else 1 + args.steps
    total = args.warmup + args.steps + (0 if args.no_e2e else args.steps) + 2 + exact_steps
    batches = [stream.next_batch(args.batch) for _ in range(total)]
    flags = [g.flag_updates(u, v) for u, v in batches]  # against the base graph, before any batch

    dev_inputs = []
    for (u, v), ins in zip(batches[: args.warmup + args.steps], flags):
        dev_inputs.append((torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda(), torch.from_numpy(ins).cuda()))
    torch.cuda.synchronize()

    def dist_barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # the sampler starts before the warm-up so that its own start-up is not
    # inside the timed region; only the samples taken during it are summarised
    clocks = ClockSampler(local)
    clocks.start()
    for i in range(args.warmup):
        du, dv, di = dev_inputs[i]
        g.apply_batch_device(du.data_ptr(), dv.data_ptr(), di.data_ptr(), du.numel())

    # ---- timed: inputs resident in HBM
    # only the k_lb_push_hop launches carry events inside the timed region (the
    # roofline kernel); the per-stage breakdown comes from a separate batch
    g.profile(2)
    g.profile_reset()
    dist_barrier()
    torch.cuda.synchronize()
    launches0 = native.kernel_launches()
    t0 = time.perf_counter()
    lat = []
    for i in range(args.warmup, args.warmup + args.steps):
        du, dv, di = dev_inputs[i]
        g.apply_batch_device(du.data_ptr(), dv.data_ptr(), di.data_ptr(), du.numel())
        lat.append(g.stats()["device_ms"])
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    wall = t1 - t0
    launches = native.kernel_launches() - launches0
    clk = clocks.stop(window=(t0, t1))
    dist_barrier()
    prof = g.profile_read()
    g.profile(False)
    dev_ms = float(np.sum(lat))
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([dev_ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        dev_ms = float(tt.item())
    value = world * args.steps * args.batch / (dev_ms / 1e3)

    # ---- end to end through the host-buffer C-ABI call
    e2e = None
    if not args.no_e2e:
        e2e_ms = []
        base = args.warmup + args.steps
        for i in range(base, base + args.steps):
            u, v = batches[i]
            t = time.perf_counter()
            g.apply_batch(u, v, flags[i])
            g.get_mis()
            e2e_ms.append((time.perf_counter() - t) * 1e3)
        e2e = {"value": world * args.steps * args.batch / (float(np.sum(e2e_ms)) / 1e3), "unit": UNIT,
               "h2d_bytes_per_step": int(args.batch * 9), "d2h_bytes_per_step": int(n)}

    # ---- per-stage breakdown: one more batch, untimed, with every stage timed
    nxt = args.warmup + args.steps + (0 if args.no_e2e else args.steps)
    g.profile(True)
    g.profile_reset()
    u, v = batches[nxt]
    g.apply_batch(u, v, flags[nxt])
    stage_prof = g.profile_read()
    g.profile(False)
    nxt += 1

    # ---- algorithmic bytes of one batch (the per-batch roofline): one more
    # untimed batch with the library's accounting on (every sub-batch then
    # computes its exact packed size; results are unchanged)
    g.profile(4)
    u, v = batches[nxt]
    g.apply_batch(u, v, flags[nxt])
    acct = g.stats()
    g.profile(False)
    nxt += 1

    # ---- exact-MIS mode on the same context: the fix-up after every batch
    exact = None
    if exact_steps:
        g.set_exact(True)
        ex_ms = []
        for k in range(exact_steps):
            u, v = batches[nxt + k]
            g.apply_batch(u, v, flags[nxt + k])
            if k >= 1:
                ex_ms.append(g.stats()["device_ms"])
        viol, unc = g.check_mis()
        g.set_exact(False)
        exact = {"value": len(ex_ms) * args.batch / (float(np.sum(ex_ms)) / 1e3), "unit": UNIT,
                 "ms_per_step": float(np.mean(ex_ms)), "steps": len(ex_ms), "warmup": 1,
                 "violations_after": int(viol), "uncovered_after": int(unc),
                 "timing": "library CUDA events per batch, host-buffer batches"}

    # ---- roofline of the two largest kernels, each timed by CUDA events
    # around its launches on the library's stream inside the timed region:
    # k_lb_push_hop (the hop-2 reach of the clustering write), 12 B per
    # pushed element (4 B row entry read + 4 B state read + 4 B cid write),
    # and the candidates' pull (k_pull_cand), 28 B per vertex + 4 B per row
    # entry read.  The one with more device time is the line's "roofline".
    peak, peak_kind = measured_peaks()
    ms, calls, nbytes = prof["push_hop"]
    achieved = nbytes / (ms / 1e3) / 1e9 if ms > 0 else 0.0
    per_launch = nbytes / max(calls, 1)
    elements = per_launch / 12.0
    traffic = None if PUSH_HOP_DRAM_BYTES_PER_ELEMENT is None else PUSH_HOP_DRAM_BYTES_PER_ELEMENT * elements
    top = max(((k, v) for k, v in stage_prof.items() if k != "push_hop"), key=lambda kv: kv[1][0])
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "kernel": "k_lb_push_hop", "peak_kind": peak_kind,
            "algorithmic_bytes_per_launch": per_launch, "avg_launch_ms": ms / max(calls, 1),
            "launches": int(calls),
            "traffic_note": "DRAM bytes per pushed element from an ncu capture of three launches of this "
                            "workload (cold L2, 13.95 B against 12 B algorithmic), times this workload's "
                            "elements per launch"}

    # per-batch roofline: the algorithmic bytes of a whole batch, summed over
    # the reference's sub-batches, against the timed batches' mean time:
    #   B = sum_SB [ 32*|E_SB| + sum_{r in S u H} (2*w_idx + 4*deg(r)) + 8*A_SB + 8*rows_SB ]
    # (edge record in + overlay write; each mapped row's offsets and entries
    # read once; state read + cluster-id write per packed element; final state
    # read + write per mapped row), w_idx = 4 for the int32 .egr layout
    rows = int(acct["seeds"] + acct["candidates"])
    w_idx = 4
    bbytes = (32.0 * args.batch + (2 * w_idx + 8) * rows + 4.0 * acct["row_degree_total"]
              + 8.0 * acct["packed_total"])
    batch_ms = dev_ms / args.steps
    roof["batch"] = {
        "bytes": bbytes, "packed_total": int(acct["packed_total"]), "rows": rows,
        "row_degree_total": int(acct["row_degree_total"]), "sub_batches": int(acct["sub_batches"]),
        "batch_ms": batch_ms, "achieved": bbytes / (batch_ms / 1e3) / 1e9,
        "frac": bbytes / (batch_ms / 1e3) / 1e9 / peak,
        "formula": "B = 32*|E| + (2*w_idx + 8)*rows + 4*sum deg(rows) + 8*packed, w_idx 4; counted on one "
                   "untimed batch of the same stream (library accounting), timed against the timed batches' "
                   "mean device time",
    }
    roof["batch_frac"] = roof["batch"]["frac"]
    ms_p, calls_p, bytes_p = prof.get("pull", (0.0, 0, 0.0))
    if ms_p > 0:
        ach_p = bytes_p / (ms_p / 1e3) / 1e9
        pull = {"bound": "hbm", "achieved": ach_p, "peak": peak, "unit": "GB/s", "frac": ach_p / peak,
                "traffic": PULL_DRAM_BYTES_PER_LAUNCH, "kernel": "k_pull_cand", "peak_kind": peak_kind,
                "algorithmic_bytes_per_launch": bytes_p / max(calls_p, 1), "avg_launch_ms": ms_p / max(calls_p, 1),
                "launches": int(calls_p),
                "timed": "per sub-batch: k_cand_bits, k_pull_cand and k_pull_cand_long (the pull step)",
                "bytes_note": "28 B per vertex (row bounds, tombstone count, tag, id) + 4 B per row entry read "
                              "(device counter)",
                "traffic_note": "DRAM bytes per launch of k_pull_cand from an ncu capture of this workload "
                                "(cold L2)" if PULL_DRAM_BYTES_PER_LAUNCH else "not captured"}
        push_hop = roof
        if ms_p > ms:
            roof = dict(pull, batch=push_hop.pop("batch"), batch_frac=push_hop.pop("batch_frac"))
            roof["next"] = push_hop
        else:
            roof["next"] = pull

    line = {
        "metric": METRIC, "value_is": VALUE_IS, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded R-MAT + toggle stream)", "config": workload_config(args),
        "p50_batch_ms": float(np.percentile(lat, 50)), "p99_batch_ms": float(np.percentile(lat, 99)),
        "wall_s_timed": wall, "gpu_launches": int(launches), "clocks": clk, "roofline": roof,
        "stage_ms": {k: round(v[0], 3) for k, v in stage_prof.items()}, "slowest_stage": top[0],
        "stage_ms_note": "one untimed batch after the timed ones, every stage timed with CUDA events "
                         "(the push_hop launches and the pull step are timed apart from the rest of "
                         "cluster_write)",
    }
    if e2e:
        line["e2e"] = e2e
    if exact:
        line["exact_mode"] = exact
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        u, v = batches[0]
        rate, lines, spent = cpu_sample(n, nindex, nlist, (u, v), flags[0], args.cpu_seconds)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                "sample": "oracle on the first %d lines of batch 1 from the initial state "
                                          "(%.1f s)" % (lines, spent)}
        try:
            line["cpu_greedy_recompute"] = cpu_greedy(nindex, nlist, batches[:2], flags[:2])
        except Exception as e:  # a baseline must not cost the line
            line["cpu_greedy_recompute"] = {"error": str(e)}
    g.close()
    del dev_inputs
    torch.cuda.empty_cache()
    # the configuration legs; a leg that fails records its error instead of
    # costing the line
    def leg(name, fn):
        t = time.perf_counter()
        try:
            res = fn()
        except Exception as e:  # noqa: BLE001
            import traceback
            res = {"error": "%s: %s" % (type(e).__name__, e), "trace": traceback.format_exc()[-1500:]}
        if isinstance(res, dict):
            res["leg_wall_s"] = time.perf_counter() - t
        line[name] = res
        torch.cuda.empty_cache()
        return res

    if rank == 0 and not args.no_large:
        leg("large_int64", lambda: run_large(args, local))
    if rank == 0 and not args.no_served:
        tuned_box = {}

        def batched_leg():
            graphs = graph_set(args.batched_graphs, 1000, args.graphs_nmax, 12, dev)
            res, tuned_box["opts"] = run_batched(args, graphs, initial_mis(graphs), dev)
            return res

        def served_leg():
            graphs = graph_set(args.served_graphs, 1000, args.graphs_nmax, 11, dev)
            return run_served(args, graphs, initial_mis(graphs), tuned_box.get("opts") or native.batched_opts(), dev)

        leg("batched", batched_leg)
        leg("served", served_leg)
    if rank == 0:
        print(json.dumps(line), flush=True)
    dist_barrier()


if __name__ == "__main__":
    main()
