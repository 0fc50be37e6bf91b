"""The drop-in binaries (misfit, misfit_async): same 5 arguments, same files,
same stdout lines as the reference engines."""
import hashlib
import os
import re
import subprocess

import numpy as np
import pytest

from misfit_gb300 import build
from misfit_gb300 import workloads as W
from tests import _golden as G

pytestmark = pytest.mark.gpu

BIN = os.path.join(os.path.dirname(build.LIB), "..", "bin")


def _setup(tmp_path, name="sample"):
    g = G.load(name)
    n = int(g["n"])
    egr = tmp_path / (name + ".egr")
    W.write_egr(str(egr), n, g["nindex"], g["nlist"], wide=bool(g["wide"]) if "wide" in g else False)
    W.write_mis_file(str(tmp_path / "mis.txt"), G.mis0(g))
    folder = tmp_path / "batches"
    W.write_batch_folder(str(folder), [(u, v) for u, v, _ in G.batches(g)])
    return g, n, egr, folder


@pytest.mark.parametrize("engine", ["misfit", "misfit_async"])
def test_cli_final_mis_and_compaction(engine, gpu_lib, tmp_path):
    g, n, egr, folder = _setup(tmp_path, "er1500")
    nb = int(g["num_batches"])
    exe = os.path.abspath(os.path.join(BIN, engine))
    # 1) skip compaction: the .egr stays, the final MIS matches
    env = dict(os.environ, MISFIT_SKIP_COMPACTION="1")
    out = subprocess.run([exe, str(egr), str(tmp_path / "mis.txt"), str(folder), str(nb), "0"], cwd=str(tmp_path),
                         env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    mis = W.read_mis_file(str(tmp_path / "datasets" / "Final_MISs" / "er1500_flash_final_mis.txt"), n)
    assert np.array_equal(mis, g["b%d_mis_oracle" % (nb - 1)])
    # the reference's own binary (its main() run on the CPU) wrote this file
    assert np.array_equal(mis, G.main_final_mis(g, "sync" if engine == "misfit" else "async"))
    assert "Total processing time:" in out.stdout
    assert re.search(r"Final MIS cardinality:\s+%d" % int(mis.sum()), out.stdout)
    if engine == "misfit":
        assert len(re.findall(r"Processing batch \d+/%d \| Edges: \d+" % nb, out.stdout)) == nb
        assert out.stdout.count("Total Batch Time:") == nb
    else:
        assert len(re.findall(r"Batch \d+/%d \| edges=\d+ \| time=[0-9.]+ms" % nb, out.stdout)) == nb
    before = egr.read_bytes()
    # 2) with compaction: the input .egr is replaced by the merged graph
    out = subprocess.run([exe, str(egr), str(tmp_path / "mis.txt"), str(folder), str(nb), "0"], cwd=str(tmp_path),
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    after = egr.read_bytes()
    assert after != before
    assert hashlib.sha256(after).digest() == bytes(g["compact_sha256"])
    assert hashlib.sha256(after).digest() == bytes(g["main_%s_compact_sha256" % ("sync" if engine == "misfit" else "async")])


@pytest.mark.parametrize("engine", ["misfit", "misfit_async"])
def test_cli_config1_against_reference_binary(engine, gpu_lib, tmp_path):
    """Config 1 (ER G(10000, 8), 10 x 2000 toggles) through the drop-in binary:
    the final-MIS file and the in-place compaction equal what the reference's
    own bin/misfit / bin/misfit_async (main() run on the CPU) wrote."""
    g, n, egr, folder = _setup(tmp_path, "cfg1")
    nb = int(g["num_batches"])
    exe = os.path.abspath(os.path.join(BIN, engine))
    out = subprocess.run([exe, str(egr), str(tmp_path / "mis.txt"), str(folder), str(nb), "0"], cwd=str(tmp_path),
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    mis = W.read_mis_file(str(tmp_path / "datasets" / "Final_MISs" / "cfg1_flash_final_mis.txt"), n)
    ref = "sync" if engine == "misfit" else "async"
    assert np.array_equal(mis, G.main_final_mis(g, ref))
    assert hashlib.sha256(egr.read_bytes()).digest() == bytes(g["main_%s_compact_sha256" % ref])


def test_cli_usage_and_errors(gpu_lib, tmp_path):
    exe = os.path.abspath(os.path.join(BIN, "misfit"))
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 1 and "Usage" in out.stderr
    out = subprocess.run([exe, str(tmp_path / "none.egr"), "m", "b", "1", "0"], capture_output=True, text=True)
    assert out.returncode == 1 and "ERROR" in out.stderr


def test_cli_compaction_interrupted_before_rename(gpu_lib, tmp_path):
    """Crash safety of the end-of-run compaction (core/flash_compactor.h:88-104:
    write <egr>.tmp.<pid>, fsync, rename over the input, fsync the folder).
    The process is ended after the temporary file is complete and before the
    rename: the input .egr must be untouched and the final MIS already saved;
    the temporary file holds the whole compacted graph; a rerun from the same
    inputs then compacts normally."""
    g, n, egr, folder = _setup(tmp_path, "er1500")
    nb = int(g["num_batches"])
    exe = os.path.abspath(os.path.join(BIN, "misfit"))
    before = egr.read_bytes()
    env = dict(os.environ, MISFIT_GB_EXIT_BEFORE_RENAME="1")
    out = subprocess.run([exe, str(egr), str(tmp_path / "mis.txt"), str(folder), str(nb), "0"], cwd=str(tmp_path),
                         env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 86, (out.returncode, out.stderr)
    assert egr.read_bytes() == before
    mis = W.read_mis_file(str(tmp_path / "datasets" / "Final_MISs" / "er1500_flash_final_mis.txt"), n)
    assert np.array_equal(mis, G.main_final_mis(g, "sync"))
    tmps = [p for p in os.listdir(str(tmp_path)) if p.startswith(egr.name + ".tmp.")]
    assert len(tmps) == 1
    assert hashlib.sha256((tmp_path / tmps[0]).read_bytes()).digest() == bytes(g["compact_sha256"])
    out = subprocess.run([exe, str(egr), str(tmp_path / "mis.txt"), str(folder), str(nb), "0"], cwd=str(tmp_path),
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    assert hashlib.sha256(egr.read_bytes()).digest() == bytes(g["compact_sha256"])
