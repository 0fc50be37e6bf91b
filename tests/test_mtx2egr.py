"""The .mtx -> .egr converter (misfit_gb300/bin/mtx2egr, host code) against
the bytes the reference's own converter writes (tests/golden/mtx2egr.json,
made by tests/golden/make_mtx_golden.py from tools/efficient_converter.py),
its int32 layout against the int64 one, and its refusals."""
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

from misfit_gb300 import build
from misfit_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mtx2egr.json")


@pytest.fixture(scope="module")
def tool():
    build.build()
    path = os.path.join(build.BIN_DIR, "mtx2egr")
    assert os.path.exists(path)
    return path


def _convert(tool, tmp_path, text, *extra):
    src, dst = tmp_path / "in.mtx", tmp_path / "out.egr"
    src.write_bytes(text.encode())
    r = subprocess.run([tool, str(src), str(dst), *extra], capture_output=True, text=True)
    return r, dst


@pytest.mark.parametrize("name", sorted(json.load(open(GOLDEN))))
def test_bytes_equal_reference_converter(tool, tmp_path, name):
    case = json.load(open(GOLDEN))[name]
    r, dst = _convert(tool, tmp_path, case["mtx"])
    assert r.returncode == 0, r.stderr
    data = dst.read_bytes()
    assert len(data) == case["size"]
    assert hashlib.sha256(data).hexdigest() == case["sha256"]


@pytest.mark.parametrize("name", sorted(json.load(open(GOLDEN))))
def test_int32_layout_same_graph(tool, tmp_path, name):
    case = json.load(open(GOLDEN))[name]
    r, wide = _convert(tool, tmp_path, case["mtx"])
    assert r.returncode == 0
    n1, i1, l1, w1 = W.read_egr(str(wide))
    r, narrow = _convert(tool, tmp_path, case["mtx"], "--int32")
    assert r.returncode == 0, r.stderr
    n2, i2, l2, w2 = W.read_egr(str(narrow))
    assert w1 and not w2
    assert n1 == n2 and np.array_equal(i1, i2) and np.array_equal(l1, l2)


@pytest.mark.parametrize("text", [
    "3 3\n1 2\n% late comment line\n",       # a comment after the size line
    "3 3\n1 x\n",                             # not an integer
    "3 3\n0 2\n",                             # ids are 1-based
    "3 3\n1 4\n",                             # destination beyond the vertex count
    "% only comments\n",                      # no size line
])
def test_refuses_malformed(tool, tmp_path, text):
    r, dst = _convert(tool, tmp_path, text)
    assert r.returncode == 1 and "mtx2egr:" in r.stderr
    assert not dst.exists()
