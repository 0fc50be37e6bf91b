"""Build libmisfit_gb.so and the misfit / misfit_async drop-in binaries.

nvcc for sm_103a only, one translation unit per process in parallel, objects
under misfit_gb300/_build/, outputs under misfit_gb300/lib/ and
misfit_gb300/bin/ (all git-ignored).  Rebuilds only what changed.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
BIN_DIR = os.path.join(HERE, "bin")
LIB = os.path.join(LIB_DIR, "libmisfit_gb.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB_SOURCES = ["mf_prims.cu", "mf_overlay.cu", "mf_repair.cu", "mf_api.cu", "mf_pool.cu", "mf_parse.cu", "mf_batched.cu"]
CLI_SOURCE = "misfit_main.cpp"
HEADERS = [os.path.join(CSRC, "mf_internal.cuh"), os.path.join(CSRC, "mf_cta.cuh"), os.path.join(CSRC, "mf_scan.cuh"),
           os.path.join(ROOT, "include", "misfit_gb.h")]


def nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, extra=()):
    out = os.path.join(OBJ, os.path.splitext(os.path.basename(src))[0] + ".o")
    if not _stale(out, [src] + HEADERS):
        return out
    cmd = [nvcc(), "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills",
           *ARCH, "-I" + os.path.join(ROOT, "include"), "-c", src, "-o", out + ".tmp", *extra]
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


def build(verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(BIN_DIR, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in LIB_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(_compile, srcs))
    if _stale(LIB, objs):
        subprocess.check_call([nvcc(), "-shared", *ARCH, "-o", LIB + ".tmp", *objs, "-lcudart"])
        os.replace(LIB + ".tmp", LIB)
    cli_src = os.path.join(CSRC, CLI_SOURCE)
    if os.path.exists(cli_src):
        for name in ("misfit", "misfit_async"):
            exe = os.path.join(BIN_DIR, name)
            if _stale(exe, [cli_src, LIB] + HEADERS):
                flag = ["-DMISFIT_ASYNC=1"] if name == "misfit_async" else []
                subprocess.check_call(["g++", "-O2", "-std=c++17", *flag, "-I" + os.path.join(ROOT, "include"),
                                       cli_src, "-o", exe + ".tmp", "-L" + LIB_DIR, "-lmisfit_gb",
                                       "-Wl,-rpath,$ORIGIN/../lib"])
                os.replace(exe + ".tmp", exe)
    # offline tools (host code only): .mtx edge list -> .egr, batch folders
    for src_name, tool_name in (("mf_mtx2egr.cpp", "mtx2egr"), ("mf_mkbatches.cpp", "mkbatches")):
        tool_src = os.path.join(CSRC, src_name)
        tool = os.path.join(BIN_DIR, tool_name)
        if os.path.exists(tool_src) and _stale(tool, [tool_src]):
            subprocess.check_call(["g++", "-O2", "-std=c++17", tool_src, "-o", tool + ".tmp"])
            os.replace(tool + ".tmp", tool)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
