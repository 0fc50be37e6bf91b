"""Autotuner of the batched form (mf_apply_batches).

The batched step's knobs (mf_batched_opts): the persistent kernel's block
size, its CTAs per SM, the two limits that decide which batches it carries
(lines per batch, vertices per graph) -- everything above them takes the
multi-launch path concurrently -- and the host threads of that path.  Which setting is fastest depends on the
GPU and on the mix of graph and batch sizes, so the tuner measures: it runs
the caller's step once per candidate setting, each time on fresh contexts
from the same initial state, and keeps the fastest.  Every candidate must
leave every graph with the same membership (the setting changes the
schedule of independent graphs, never a result); a disagreement raises.

Results are cached in a JSON file keyed by the GPU name and a shape bucket
of the workload (graph count, log2 of the median vertex count and of the
median batch size), so later runs with a similar mix skip the search.

tune_plain does the same for the per-batch path (mf_apply_batch): its
load-balancing settings (mf_tuning: pull or push for the candidate rows'
cluster ids, the candidate pull's long-row cut, the heavy-vertex row length
of the exact sizes, the hop-2 volume that defers the insertion rule's
search to the grid-wide kernel, and the warp level of the
first-cluster-id search) are searched one after another on
the caller's batches, each candidate on a fresh context, every candidate
required to give the same memberships.
"""
import json
import os
import time

import numpy as np

from . import native

CACHE_ENV = "MISFIT_GB_AUTOTUNE_CACHE"

# Coordinate search: the batch-size limit first (it moves the most work),
# then block size and CTAs per SM at the best limit, then the host threads
# of the multi-launch path.
LIMITS = (2048, 4096, 8192, 16384, 32768)
SHAPES = ((512, 2), (256, 4), (1024, 1), (256, 2))
PATH_THREADS = (4, 8, 16)


def cache_path():
    return os.environ.get(CACHE_ENV) or os.path.join(os.path.expanduser("~"), ".cache", "misfit_gb",
                                                       "autotune.json")


def _gpu_name():
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:
        return "unknown-gpu"


def shape_key(graphs, batches):
    ns = [int(g[0]) for g in graphs]
    ms = [int(np.asarray(b[0]).size) for b in batches]
    return "%s|g%d|n2^%d|m2^%d" % (_gpu_name(), len(graphs), int(np.log2(max(1, np.median(ns)))),
                                   int(np.log2(max(1, np.median(ms)))))


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, data):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp%d" % os.getpid()
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def run_step(graphs, mis0, batches, opts):
    """Fresh contexts, one batched step.  Returns (wall seconds, memberships, stats)."""
    ctxs = []
    try:
        for (n, nindex, nlist), m in zip(graphs, mis0):
            g = native.Graph.from_csr(nindex, nlist)
            g.set_mis(m)
            ctxs.append(g)
        t0 = time.perf_counter()
        st = native.apply_batches(ctxs, batches, opts)
        mis = [g.get_mis() for g in ctxs]
        return time.perf_counter() - t0, mis, st
    finally:
        for g in ctxs:
            g.close()


def tune_batched(graphs, mis0, batches, use_cache=True):
    """graphs: [(n, nindex, nlist)], mis0: initial memberships, batches:
    [(u, v, ins)] one per graph.  Returns (opts, report)."""
    path = cache_path()
    key = shape_key(graphs, batches)
    cache = _load(path) if use_cache else {}
    if key in cache:
        c = cache[key]
        return native.batched_opts(**c["opts"]), {"cached": True, "key": key, **c}
    trials = []
    ref = None

    def trial(**kw):
        nonlocal ref
        opts = native.batched_opts(**kw)
        sec, mis, st = run_step(graphs, mis0, batches, opts)
        if ref is None:
            ref = mis
        elif not all(np.array_equal(a, b) for a, b in zip(ref, mis)):
            raise RuntimeError("batched step results differ between settings %s" % kw)
        trials.append({"opts": kw, "seconds": sec, "kernel_items": st["kernel_items"],
                       "path_items": st["path_items"]})
        return sec

    run_step(graphs, mis0, batches, native.batched_opts())   # warm-up: library, allocations
    best_limit = min(LIMITS, key=lambda lim: trial(max_cta_updates=lim))
    best_shape = min(SHAPES, key=lambda s: trial(max_cta_updates=best_limit, block=s[0], ctas_per_sm=s[1]))
    best_threads = min(PATH_THREADS, key=lambda t: trial(max_cta_updates=best_limit, block=best_shape[0],
                                                         ctas_per_sm=best_shape[1], path_threads=t))
    chosen = {"max_cta_updates": best_limit, "block": best_shape[0], "ctas_per_sm": best_shape[1],
              "path_threads": best_threads}
    entry = {"opts": chosen, "trials": trials}
    if use_cache:
        cache[key] = entry
        try:
            _store(path, cache)
        except OSError:
            pass
    return native.batched_opts(**chosen), {"cached": False, "key": key, **entry}


# The library's defaults of mf_tuning (a GPU test checks that a new context
# reports these), and the candidate values, searched one at a time.
DEFAULT_TUNING = {"pull_long": 2048, "heavy_min": 2048, "big_threshold": 64, "first_bound": 256, "cand_push": 0,
                  "pull_sizes": 1}
PLAIN_KNOBS = (
    ("cand_push", (0, 1, 2)),
    ("pull_sizes", (1, 0, 2)),
    ("big_threshold", (64, 256, 1024, 4096)),
    ("first_bound", (64, 256, 1024)),
    ("pull_long", (512, 2048, 8192)),
    ("heavy_min", (1024, 2048, 8192)),
)


def run_plain(nindex, nlist, mis0, batches, tuning):
    """A fresh context with `tuning`, the batches applied in order.  Returns
    (device seconds summed over the batches, final membership)."""
    g = native.Graph.from_csr(nindex, nlist)
    try:
        g.set_tuning(**tuning)
        g.set_mis(mis0)
        ms = 0.0
        for u, v, ins in batches:
            g.apply_batch(u, v, ins)
            ms += g.stats()["device_ms"]
        return ms / 1e3, g.get_mis()
    finally:
        g.close()


def tune_plain(nindex, nlist, mis0, batches, use_cache=True):
    """Coordinate search of the per-batch path's thresholds on `batches`
    (a list of (u, v, ins)).  Returns (tuning dict, report)."""
    path = cache_path()
    key = "plain|%s|n2^%d|m2^%d" % (_gpu_name(), int(np.log2(max(1, np.asarray(nindex).size - 1))),
                                    int(np.log2(max(1, np.median([np.asarray(b[0]).size for b in batches])))))
    cache = _load(path) if use_cache else {}
    if key in cache:
        return dict(cache[key]["tuning"]), {"cached": True, "key": key, **cache[key]}
    best = dict(DEFAULT_TUNING)
    trials = []
    ref = None
    run_plain(nindex, nlist, mis0, batches[:1], best)   # warm-up
    for name, values in PLAIN_KNOBS:
        scores = {}
        for val in values:
            cand = dict(best, **{name: val})
            sec, mis = run_plain(nindex, nlist, mis0, batches, cand)
            if ref is None:
                ref = mis
            elif not np.array_equal(ref, mis):
                raise RuntimeError("per-batch results differ between settings %s" % cand)
            trials.append({"tuning": cand, "seconds": sec})
            scores[val] = sec
        best[name] = min(scores, key=scores.get)
    entry = {"tuning": best, "trials": trials}
    if use_cache:
        cache[key] = entry
        try:
            _store(path, cache)
        except OSError:
            pass
    return dict(best), {"cached": False, "key": key, **entry}
