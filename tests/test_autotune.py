"""Host logic of the batched form's autotuner (misfit_gb300/autotune.py):
the coordinate search keeps the fastest setting, refuses settings whose
results differ, and caches the winner by GPU and workload shape.  The step
itself is replaced by a fake, so this runs without a GPU."""
import json

import numpy as np
import pytest

from misfit_gb300 import autotune, native


class _Opts:
    """Stands in for native.BatchedOpts (no library needed)."""

    _fields_ = [("block", None), ("ctas_per_sm", None), ("max_cta_updates", None), ("max_cta_vertices", None),
                ("use_graph", None), ("path_threads", None)]

    def __init__(self, **kw):
        self.block, self.ctas_per_sm, self.max_cta_updates = 512, 2, 8192
        self.max_cta_vertices, self.use_graph, self.path_threads = 1 << 20, 1, 8
        for k, v in kw.items():
            setattr(self, k, v)


def _setup(monkeypatch, tmp_path, cost, results=None):
    monkeypatch.setattr(native, "batched_opts", lambda **kw: _Opts(**kw))
    monkeypatch.setenv(autotune.CACHE_ENV, str(tmp_path / "cache.json"))
    monkeypatch.setattr(autotune, "_gpu_name", lambda: "test-gpu")
    calls = []

    def fake_step(graphs, mis0, batches, opts):
        calls.append(opts)
        mis = results(opts) if results else [np.zeros(3, np.uint8)]
        return cost(opts), mis, {"kernel_items": 1, "path_items": 0}

    monkeypatch.setattr(autotune, "run_step", fake_step)
    graphs = [(1000, None, None), (4000, None, None)]
    batches = [(np.zeros(100, np.int32), None, None), (np.zeros(300, np.int32), None, None)]
    return graphs, batches, calls


def test_search_keeps_fastest_and_caches(monkeypatch, tmp_path):
    def cost(o):
        return (abs(o.max_cta_updates - 32768) / 1e6 + abs(o.block - 256) / 1e5 + abs(o.ctas_per_sm - 4) / 1e4
                + abs(o.path_threads - 16) / 1e3)

    graphs, batches, calls = _setup(monkeypatch, tmp_path, cost)
    opts, rep = autotune.tune_batched(graphs, None, batches)
    assert (opts.max_cta_updates, opts.block, opts.ctas_per_sm, opts.path_threads) == (32768, 256, 4, 16)
    assert not rep["cached"]
    n_trials = len(calls)
    # warm-up + coordinate search
    assert n_trials == 1 + len(autotune.LIMITS) + len(autotune.SHAPES) + len(autotune.PATH_THREADS)
    data = json.load(open(tmp_path / "cache.json"))
    assert list(data) == [autotune.shape_key(graphs, batches)]
    assert data[rep["key"]]["opts"] == {"max_cta_updates": 32768, "block": 256, "ctas_per_sm": 4, "path_threads": 16}
    # the second call with the same shape is served from the cache
    opts2, rep2 = autotune.tune_batched(graphs, None, batches)
    assert rep2["cached"] and len(calls) == n_trials
    assert (opts2.max_cta_updates, opts2.block, opts2.ctas_per_sm) == (32768, 256, 4)


def test_search_refuses_disagreeing_settings(monkeypatch, tmp_path):
    def results(o):
        return [np.full(3, 1 if o.max_cta_updates == autotune.LIMITS[-1] else 0, np.uint8)]

    graphs, batches, _ = _setup(monkeypatch, tmp_path, lambda o: 1.0, results)
    with pytest.raises(RuntimeError):
        autotune.tune_batched(graphs, None, batches, use_cache=False)


def test_shape_key_buckets():
    g = [(1024, None, None)] * 4
    b = [(np.zeros(100, np.int32), None, None)] * 4
    k1 = autotune.shape_key(g, b)
    k2 = autotune.shape_key([(2000, None, None)] * 4, b)     # same power-of-two bucket
    k3 = autotune.shape_key([(9000, None, None)] * 4, b)
    assert k1 == k2 and k1 != k3


def test_plain_search_keeps_fastest_refuses_disagreement_and_caches(monkeypatch, tmp_path):
    """tune_plain: one threshold at a time from the defaults, the fastest
    value kept, a setting with a different membership refused, the winner
    cached by GPU and shape."""
    monkeypatch.setenv(autotune.CACHE_ENV, str(tmp_path / "cache.json"))
    monkeypatch.setattr(autotune, "_gpu_name", lambda: "test-gpu")
    want = {"pull_long": 8192, "heavy_min": 1024, "big_threshold": 1024, "first_bound": 64, "cand_push": 1,
            "pull_sizes": 2}
    calls = []

    def fake_plain(nindex, nlist, mis0, batches, tuning):
        calls.append(dict(tuning))
        sec = sum(abs(np.log2(tuning[k] + 1) - np.log2(v + 1)) for k, v in want.items())
        return sec, np.zeros(4, np.uint8)

    monkeypatch.setattr(autotune, "run_plain", fake_plain)
    nindex = np.zeros(1025, np.int64)
    batches = [(np.zeros(100, np.int32), None, None)]
    best, rep = autotune.tune_plain(nindex, None, None, batches)
    assert best == want and not rep["cached"]
    assert len(calls) == 1 + sum(len(v) for _, v in autotune.PLAIN_KNOBS)
    best2, rep2 = autotune.tune_plain(nindex, None, None, batches)
    assert rep2["cached"] and best2 == want and len(calls) == 1 + sum(len(v) for _, v in autotune.PLAIN_KNOBS)

    def bad_plain(nindex, nlist, mis0, batches, tuning):
        return 1.0, np.full(4, 1 if tuning["pull_long"] == 8192 else 0, np.uint8)

    monkeypatch.setattr(autotune, "run_plain", bad_plain)
    with pytest.raises(RuntimeError):
        autotune.tune_plain(nindex, None, None, batches, use_cache=False)
