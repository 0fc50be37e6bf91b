"""Build recipe for the oracle (test infrastructure only).

* ``oracle/_build/libmisfit_oracle.so`` -- the CPU restatement
  (``misfit_oracle.cpp``), built with g++ on any machine.
* ``oracle/_ref/libmisfit_ref.so`` -- the reference's own host code, built
  with nvcc from the reference sources where they lie.  Only built when the
  reference tree is present (it is not on GPU machines); nothing in the GPU
  tests or the benchmark needs it.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "libmisfit_oracle.so")
REF_SO = os.path.join(REF_DIR, "libmisfit_ref.so")
DEFAULT_REFERENCE_ROOT = "/root/reference"


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    src = os.path.join(HERE, "misfit_oracle.cpp")
    hdr = os.path.join(HERE, "misfit_oracle.h")
    if not force and not _stale(ORACLE_SO, [src, hdr]):
        return ORACLE_SO
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = ORACLE_SO + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", src, "-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref(reference_root=DEFAULT_REFERENCE_ROOT, force=False):
    """Compile the reference host path; returns None when the tree is absent."""
    entry = os.path.join(reference_root, "src", "misfit_async", "misfit_async.cu")
    if not os.path.exists(entry):
        return None
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    harness = os.path.join(HERE, "ref_harness.cu")
    deps = [harness, entry] + [os.path.join(reference_root, "core", f)
                               for f in ("FlashGraph.h", "flash_compactor.h", "cli_setup.h",
                                         "gpu_common.h", "reporting.h")]
    if not force and not _stale(REF_SO, deps):
        return REF_SO
    os.makedirs(REF_DIR, exist_ok=True)
    tmp = REF_SO + ".tmp%d" % os.getpid()
    cmd = [nvcc, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC,-fopenmp",
           "-gencode", "arch=compute_103a,code=sm_103a", "-w",
           "-I" + reference_root, harness, "-o", tmp, "-lgomp"]
    subprocess.check_call(cmd)
    os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
