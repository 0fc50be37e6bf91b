"""The batch-folder sampler (misfit_gb300/bin/mkbatches, host code): the
recipe of the reference's three generators -- distinct existing edges,
shuffled, "min max" lines, 1-based, batch k in k.mtx -- with uniform,
low-degree and preferential endpoints.  Its draws come from its own
generator, so the checks are the recipe's properties and the direction of
each mode's degree bias, not the reference's exact files."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from misfit_gb300 import build
from misfit_gb300 import workloads as W


@pytest.fixture(scope="module")
def tool():
    build.build()
    path = os.path.join(build.BIN_DIR, "mkbatches")
    assert os.path.exists(path)
    return path


@pytest.fixture(scope="module")
def graph(tmp_path_factory):
    n, (ni, nl) = W.rmat_graph(11, 8, 5)
    p = str(tmp_path_factory.mktemp("g") / "rmat11.egr")
    W.write_egr(p, n, ni, nl)
    return p, n, ni, nl


def _run(tool, egr, out, *args):
    return subprocess.run([tool, egr, str(out), *map(str, args)], capture_output=True, text=True)


def _read(out, k):
    return [W.read_batch_file(str(out / ("%d.mtx" % i))) for i in range(1, k + 1)]


@pytest.mark.parametrize("mode", ["uniform", "low_degree", "preferential"])
def test_recipe(tool, graph, tmp_path, mode):
    egr, n, ni, nl = graph
    r = _run(tool, egr, tmp_path / "b", 300, 4, mode, 7)
    assert r.returncode == 0, r.stderr
    batches = _read(tmp_path / "b", 4)
    keys = set()
    orc = O.Oracle.from_csr(ni, nl)
    for u, v in batches:
        assert u.size == 300
        assert np.all(u < v) and np.all(u >= 0) and np.all(v < n)
        keys.update((u * n + v).tolist())
        # existing edges only: every line is a delete against the base graph
        assert not orc.flag_updates(u.astype(np.int32), v.astype(np.int32)).any()
    assert len(keys) == 1200


def test_deterministic_by_seed(tool, graph, tmp_path):
    egr = graph[0]
    for d in ("a", "b", "c"):
        assert _run(tool, egr, tmp_path / d, 200, 2, "uniform", 3 if d != "c" else 4).returncode == 0
    read = lambda d: [open(tmp_path / d / ("%d.mtx" % i)).read() for i in (1, 2)]
    assert read("a") == read("b") and read("a") != read("c")


def test_degree_bias_direction(tool, graph, tmp_path):
    egr, n, ni, nl = graph
    deg = np.diff(ni)
    mean = {}
    for mode in ("low_degree", "uniform", "preferential"):
        assert _run(tool, egr, tmp_path / mode, 1500, 1, mode, 11).returncode == 0
        u, v = _read(tmp_path / mode, 1)[0]
        mean[mode] = float(np.mean(np.minimum(deg[u], deg[v])))
    # 1/deg vertex weights pull toward low-degree endpoints; deg weights then
    # a uniform entry of the row draw every entry alike, as uniform does
    assert mean["low_degree"] < 0.8 * mean["uniform"]
    assert mean["low_degree"] < 0.8 * mean["preferential"]
    assert 0.8 < mean["preferential"] / mean["uniform"] < 1.25


def test_refusals(tool, graph, tmp_path):
    egr, n, ni, nl = graph
    r = _run(tool, egr, tmp_path / "x", nl.size, 2)          # more pairs than entries
    assert r.returncode == 1 and "mkbatches:" in r.stderr
    r = _run(tool, egr, tmp_path / "x", 10, 1, "bogus")
    assert r.returncode == 1
    bad = tmp_path / "bad.egr"
    bad.write_bytes(b"\x05\x00\x00\x00")
    r = _run(tool, str(bad), tmp_path / "x", 1, 1)
    assert r.returncode == 1


def test_folder_reads_through_the_library(tool, graph, tmp_path):
    """The folder is what the drop-in binaries read: mf_list_batch_files
    orders it 1..k, mf_read_batch_file returns every line, 0-based."""
    from misfit_gb300 import native
    native.load_library()
    egr, n, ni, nl = graph
    assert _run(tool, egr, tmp_path / "f", 50, 12, "low_degree", 5).returncode == 0
    assert native.list_batch_files(str(tmp_path / "f")) == ["%d.mtx" % k for k in range(1, 13)]
    for k in (1, 12):
        u, v = native.read_batch_file(str(tmp_path / "f" / ("%d.mtx" % k)), n)
        uu, vv = W.read_batch_file(str(tmp_path / "f" / ("%d.mtx" % k)))
        assert np.array_equal(u, uu) and np.array_equal(v, vv) and u.size == 50
