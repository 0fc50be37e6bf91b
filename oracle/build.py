"""Build recipe for the oracle (test infrastructure only).

* ``oracle/_build/libmisfit_oracle.so`` -- the CPU restatement
  (``misfit_oracle.cpp``), built with g++ on any machine.
* ``oracle/_ref/libmisfit_ref.so`` -- the reference's own host code, built
  with nvcc from the reference sources where they lie.
* ``oracle/_ref/libref_sync_emul.so`` and ``libref_async_emul.so`` -- the
  reference's whole engines (``src/misfit/misfit.cu`` and
  ``src/misfit_async/misfit_async.cu``: host path, the six kernels, main)
  compiled with g++ for the CPU against the host-only CUDA stand-in in
  ``oracle/ref_emul/``.  The recipe writes a copy of each engine source into
  ``oracle/_ref/`` with every kernel launch rewritten as a call of the
  emulated launch (and, by default, the seed set and candidate map given the
  canonical iteration orders), checking that each rewrite applies exactly
  where expected.

The reference libraries are built only where the reference tree is present:
its root is the ``reference_root`` argument or the ``MISFIT_REF_ROOT``
environment variable (remembered in ``oracle/_ref/reference_root.txt`` for
later builds on the same machine).  Nothing in the GPU tests or the benchmark needs
them; outputs go to ``oracle/_ref/``, which is never committed.

Usage: ``MISFIT_REF_ROOT=<reference tree> python oracle/build.py [--force]``
"""
import os
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
EMUL_DIR = os.path.join(HERE, "ref_emul")
ORACLE_SO = os.path.join(BUILD_DIR, "libmisfit_oracle.so")
REF_SO = os.path.join(REF_DIR, "libmisfit_ref.so")
EMUL_SO = {"sync": os.path.join(REF_DIR, "libref_sync_emul.so"),
           "async": os.path.join(REF_DIR, "libref_async_emul.so")}
EMUL_SRC = {"sync": os.path.join("src", "misfit", "misfit.cu"),
            "async": os.path.join("src", "misfit_async", "misfit_async.cu")}
REF_HEADERS = ("FlashGraph.h", "flash_compactor.h", "cli_setup.h", "gpu_common.h", "reporting.h")


ROOT_NOTE = os.path.join(REF_DIR, "reference_root.txt")


def reference_root(explicit=None):
    """The reference tree's root, or None when it is not given or not here.
    Looked up in the argument, then MISFIT_REF_ROOT, then the note a previous
    build left in oracle/_ref/ (untracked; a root given once is remembered
    on this machine)."""
    root = explicit or os.environ.get("MISFIT_REF_ROOT")
    if not root and os.path.exists(ROOT_NOTE):
        with open(ROOT_NOTE) as f:
            root = f.read().strip()
    if root and os.path.isdir(os.path.join(root, "src")):
        if explicit or os.environ.get("MISFIT_REF_ROOT"):
            os.makedirs(REF_DIR, exist_ok=True)
            with open(ROOT_NOTE, "w") as f:
                f.write(os.path.abspath(root) + "\n")
        return root
    return None


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


def build_ref(reference_root_dir=None, force=False):
    """Compile the reference host path; returns None when the tree is absent."""
    root = reference_root(reference_root_dir)
    if root is None:
        return REF_SO if os.path.exists(REF_SO) else None
    entry = os.path.join(root, "src", "misfit_async", "misfit_async.cu")
    if not os.path.exists(entry):
        return None
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    harness = os.path.join(HERE, "ref_harness.cu")
    deps = [harness, entry] + [os.path.join(root, "core", f) for f in REF_HEADERS]
    if not force and not _stale(REF_SO, deps):
        return REF_SO
    os.makedirs(REF_DIR, exist_ok=True)
    tmp = REF_SO + ".tmp%d" % os.getpid()
    cmd = [nvcc, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC,-fopenmp",
           "-gencode", "arch=compute_103a,code=sm_103a", "-w",
           "-I" + root, harness, "-o", tmp, "-lgomp"]
    subprocess.check_call(cmd)
    os.replace(tmp, REF_SO)
    return REF_SO


# ---- host emulation of the reference engines --------------------------------

_LAUNCH = re.compile(r"\b([A-Za-z_]\w*)\s*<<<")


def _split_top(s):
    """Split s at commas outside parentheses/brackets/braces."""
    parts, depth, cur = [], 0, []
    for ch in s:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append("".join(cur).strip())
            cur = []
        else:
            cur.append(ch)
    parts.append("".join(cur).strip())
    return parts


def rewrite_launches(text):
    """`k<<<g, b, 0, s>>>(args);` -> `REFEMUL_LAUNCH(k, g, b, args);`.
    Returns (new_text, [kernel names in order])."""
    out, pos, names = [], 0, []
    while True:
        m = _LAUNCH.search(text, pos)
        if not m:
            out.append(text[pos:])
            break
        close = text.index(">>>", m.end())
        config = _split_top(text[m.end():close])
        if len(config) < 2:
            raise RuntimeError("launch configuration not understood: %r" % text[m.start():close + 3])
        j = close + 3
        while text[j].isspace():
            j += 1
        if text[j] != "(":
            raise RuntimeError("kernel launch without an argument list near %r" % text[m.start():j + 10])
        depth, k = 0, j
        while True:
            if text[k] == "(":
                depth += 1
            elif text[k] == ")":
                depth -= 1
                if depth == 0:
                    break
            k += 1
        args = text[j + 1:k]
        e = k + 1
        while text[e].isspace():
            e += 1
        if text[e] != ";":
            raise RuntimeError("kernel launch not followed by ';'")
        out.append(text[pos:m.start()])
        out.append("REFEMUL_LAUNCH(%s, %s, %s, %s);" % (m.group(1), config[0], config[1], args.strip()))
        names.append(m.group(1))
        pos = e + 1
    return "".join(out), names


# (pattern, replacement): the two containers whose iteration order the
# language leaves unspecified, given the canonical orders.
_CANONICAL_ORDERS = [
    (r"\bunordered_set<int>\s+unique_vertices\s*;", "::refemul::FirstAppearanceSet unique_vertices;"),
    (r"\bunordered_map<int,\s*vector<int>>\s+candidate_rows\s*;", "std::map<int, vector<int>> candidate_rows;"),
]
_EXPECTED_KERNELS = ["init_nodes_kernel", "build_vertex_map_kernel", "vertex_clustering_csr_kernel",
                     "assign_edges_to_clusters_kernel", "process_clusters_csr_kernel",
                     "clear_cluster_assignments_kernel"]


def emulation_source(engine_text, canonical_orders=True):
    text, names = rewrite_launches(engine_text)
    if names != _EXPECTED_KERNELS:
        raise RuntimeError("unexpected kernel launches in the engine: %s" % names)
    if canonical_orders:
        for pat, rep in _CANONICAL_ORDERS:
            text, k = re.subn(pat, rep, text)
            if k != 1:
                raise RuntimeError("expected one match of %r, found %d" % (pat, k))
    return text


def build_ref_emul(reference_root_dir=None, force=False):
    """Build oracle/_ref/libref_{sync,async}_emul.so; returns the dict of
    paths, or None when the reference tree is absent (then existing builds
    are returned if present)."""
    root = reference_root(reference_root_dir)
    if root is None:
        have = {k: p for k, p in EMUL_SO.items() if os.path.exists(p)}
        return have or None
    harness = os.path.join(EMUL_DIR, "ref_emul.cpp")
    shim = [os.path.join(EMUL_DIR, f) for f in ("cuda_runtime.h", "device_launch_parameters.h")]
    os.makedirs(REF_DIR, exist_ok=True)

    def one(engine):
        src = os.path.join(root, EMUL_SRC[engine])
        deps = [src, harness, __file__] + shim + [os.path.join(root, "core", f) for f in REF_HEADERS]
        so = EMUL_SO[engine]
        if not force and not _stale(so, deps):
            return so
        gen = os.path.join(REF_DIR, "misfit_%s_emul.inc" % engine)
        with open(src) as f:
            text = emulation_source(f.read())
        with open(gen, "w") as f:
            f.write(text)
        tmp = so + ".tmp%d" % os.getpid()
        cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-w",
               "-I" + EMUL_DIR, "-I" + REF_DIR, "-I" + os.path.dirname(src),
               '-DREFEMUL_SOURCE="misfit_%s_emul.inc"' % engine, harness, "-o", tmp]
        if engine == "sync":
            cmd.insert(1, "-DREFEMUL_FINE_API")
        subprocess.check_call(cmd)
        os.replace(tmp, so)
        return so

    with ThreadPoolExecutor(2) as ex:
        paths = list(ex.map(one, ["sync", "async"]))
    return dict(zip(["sync", "async"], paths))


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_oracle(force=force))
    print(build_ref(force=force))
    print(build_ref_emul(force=force))
