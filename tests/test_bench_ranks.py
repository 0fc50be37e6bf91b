"""bench.py's multi-rank contract on CPU: under torchrun with two ranks (gloo)
the reference arm runs on rank 0 only, every rank meets the final barrier,
and exactly one JSON line comes out.  The path does not shard (replicas
only), so no data-path collective is involved."""
import json
import os
import socket
import subprocess
import sys

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
