"""bench.py's contract on CPU.  Multi-rank: under torchrun with two ranks
(gloo) the reference arm runs on rank 0 only, every rank meets the final
barrier, and exactly one JSON line comes out.  The path does not shard
(replicas only), so no data-path collective is involved.  Measurement
helpers: the clocks record of the timed window, the latency buckets and the
roofline's peak source."""
import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_two_ranks_gloo():
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--scale", "10",
           "--batch", "200", "--steps", "1", "--warmup", "0", "--cpu-seconds", "1"]
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="2")
    out = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0


def test_reference_arm_evolving_state_single_rank():
    """The reference arm carries its state across steps and reports what it
    actually timed: the lines of each step, the time spent on them."""
    pytest.importorskip("torch")
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--scale", "10",
           "--batch", "300", "--steps", "2", "--warmup", "1", "--cpu-seconds", "30"]
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="2")
    out = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads([l for l in out.stdout.splitlines() if l.startswith("{")][0])
    assert d["lines_timed_per_step"] == [300, 300]     # a small batch fits the budget whole
    assert d["sampled_fraction"] == 1.0 and d["extrapolated"] is False
    assert abs(d["value"] - 600 / (d["ms_per_step"] * 2 / 1e3)) < 1e-6 * d["value"]


def _bench_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class _Stopped:
    """Stands in for the nvidia-smi process (already read)."""

    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def test_clock_summary_keeps_the_timed_window_and_names_throttle_reasons():
    """The clocks record of a bench line: the median SM clock and the maximum
    over the samples inside the timed window (one sampling period of slack),
    and every throttle reason seen Active there; samples outside the window,
    short lines and unparsable ones are ignored."""
    bench = _bench_module()
    cs = bench.ClockSampler(0)
    cs.proc = _Stopped()
    row = "0, {sm}, 2070, 900.0, 0x0, {hw}, Not Active, Not Active, {cap}"
    cs.lines = [
        (0.5, row.format(sm=1000, hw="Active", cap="Not Active")),       # before the window
        (1.0, row.format(sm=2070, hw="Not Active", cap="Not Active")),
        (1.2, row.format(sm=2055, hw="Not Active", cap="Active")),
        (1.4, row.format(sm=2070, hw="Not Active", cap="Not Active")),
        (1.5, "0, [N/A], 2070"),                                          # short line
        (1.6, row.format(sm="[N/A]", hw="Not Active", cap="Not Active")),  # unparsable clock
        (2.2, row.format(sm=2070, hw="Not Active", cap="Not Active")),   # within the slack
        (2.6, row.format(sm=500, hw="Active", cap="Not Active")),        # after the window
    ]
    s = cs.stop(window=(1.0, 2.0))
    assert s["samples"] == 4 and s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    assert bench.ClockSampler(0).stop() == {"sm_mhz": None, "sm_max_mhz": None,
                                            "reasons": ["nvidia-smi unavailable"]}


def test_latency_summary_buckets_by_batch_size():
    bench = _bench_module()
    lat = [1.0, 2.0, 3.0, 4.0, 100.0]
    sizes = [10, 50, 500, 5000, 20000]
    s = bench.latency_summary(lat, sizes)
    assert s["p50_ms"] == 3.0
    got = {k: v["requests"] for k, v in s["by_size"].items()}
    assert sum(got.values()) == 5
    for k, v in s["by_size"].items():
        lo, hi = (int(x) for x in k.split("-"))
        members = [x for x, n in zip(lat, sizes) if lo <= n <= hi]
        assert v["requests"] == len(members) and v["p50_ms"] == float(np.percentile(members, 50))


def test_measured_peaks_fall_back_when_absent(tmp_path, monkeypatch):
    bench = _bench_module()
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.measured_peaks() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text('{"hbm_gbs": 6786.2, "bf16_tflops": 1900}')
    assert bench.measured_peaks() == (6786.2, "measured")
