"""CPU oracle for MISFIT's dynamic-MIS path -- TEST INFRASTRUCTURE ONLY.

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package.  It wraps

* ``_build/libmisfit_oracle.so``: the C++ restatement (misfit_oracle.cpp) of
  the reference path under the pinned schedule, and
* ``_ref/libmisfit_ref.so``: the reference's own host code compiled from the
  reference tree (present only where that tree exists); used to pin the
  restatement.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_I32P = C.POINTER(C.c_int32)
_I64P = C.POINTER(C.c_int64)
_U8P = C.POINTER(C.c_uint8)
_P = C.c_void_p

_OR = None
_REF = None


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def lib():
    global _OR
    if _OR is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        sig = {
            "or_create": (_P, [C.c_int32, _I64P, _I32P]),
            "or_open_egr": (_P, [C.c_char_p]),
            "or_destroy": (None, [_P]),
            "or_num_nodes": (C.c_int32, [_P]),
            "or_base_entries": (C.c_int64, [_P]),
            "or_max_csr": (C.c_int64, [_P]),
            "or_set_max_csr": (None, [_P, C.c_int64]),
            "or_set_exact": (None, [_P, C.c_int]),
            "or_set_serial_clustering": (None, [_P, C.c_int]),
            "or_set_mis": (None, [_P, _U8P]),
            "or_get_mis": (None, [_P, _U8P]),
            "or_get_cluster_ids": (None, [_P, _I32P]),
            "or_flag_updates": (None, [_P, _I32P, _I32P, C.c_int64, _U8P]),
            "or_is_adjacent": (C.c_int, [_P, C.c_int32, C.c_int32]),
            "or_apply_batch": (C.c_int64, [_P, _I32P, _I32P, _U8P, C.c_int64]),
            "or_row": (C.c_int64, [_P, C.c_int32, _I32P, C.c_int64]),
            "or_degree": (C.c_int32, [_P, C.c_int32]),
            "or_two_hop": (C.c_int64, [_P, C.c_int32, _I32P, C.c_int64]),
            "or_trace_enable": (None, [_P, C.c_int]),
            "or_trace_count": (C.c_int64, [_P]),
            "or_trace_get": (C.c_int64, [_P, C.c_int64, C.c_int, C.c_void_p, C.c_int64]),
            "or_compact": (C.c_int, [_P, C.c_char_p]),
            "or_greedy_mis": (None, [C.c_int32, _I64P, _I32P, _U8P]),
            "or_check_mis": (None, [_P, _I64P, _I64P]),
            "or_apply_overlay": (None, [_P, _I32P, _I32P, _U8P, C.c_int64]),
            "or_greedy_current": (None, [_P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _OR = L
    return _OR


_TRACE = {0: np.int64, 1: np.int32, 2: np.int32, 3: np.int32, 4: np.int32, 5: np.uint8, 6: np.int64}


class Oracle:
    """The restated reference path on one graph."""

    def __init__(self, handle):
        if not handle:
            raise ValueError("oracle could not load the graph")
        self._h = C.c_void_p(handle)
        self.n = lib().or_num_nodes(self._h)

    @classmethod
    def from_csr(cls, nindex, nlist):
        nindex = np.ascontiguousarray(nindex, dtype=np.int64)
        nlist = np.ascontiguousarray(nlist, dtype=np.int32)
        return cls(lib().or_create(nindex.size - 1, _p(nindex, C.c_int64), _p(nlist, C.c_int32)))

    @classmethod
    def open_egr(cls, path):
        return cls(lib().or_open_egr(os.fsencode(path)))

    def close(self):
        if self._h:
            lib().or_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def max_csr(self):
        return lib().or_max_csr(self._h)

    @max_csr.setter
    def max_csr(self, v):
        lib().or_set_max_csr(self._h, int(v))

    def set_exact(self, on=True):
        """Exact-MIS mode: independent, maximal membership after every batch."""
        lib().or_set_exact(self._h, 1 if on else 0)

    def set_serial_clustering(self, on=True):
        """Clustering schedule: serial (rows one after another, each seeing the
        earlier rows' writes) instead of the default bulk-synchronous one."""
        lib().or_set_serial_clustering(self._h, 1 if on else 0)

    def set_mis(self, mis):
        mis = np.ascontiguousarray(mis, dtype=np.uint8)
        lib().or_set_mis(self._h, _p(mis, C.c_uint8))

    def get_mis(self):
        out = np.zeros(self.n, dtype=np.uint8)
        lib().or_get_mis(self._h, _p(out, C.c_uint8))
        return out

    def cluster_ids(self):
        out = np.zeros(self.n, dtype=np.int32)
        lib().or_get_cluster_ids(self._h, _p(out, C.c_int32))
        return out

    def flag_updates(self, u, v):
        u = np.ascontiguousarray(u, dtype=np.int32)
        v = np.ascontiguousarray(v, dtype=np.int32)
        out = np.zeros(u.size, dtype=np.uint8)
        lib().or_flag_updates(self._h, _p(u, C.c_int32), _p(v, C.c_int32), u.size, _p(out, C.c_uint8))
        return out

    def is_adjacent(self, u, v):
        return bool(lib().or_is_adjacent(self._h, u, v))

    def apply_batch(self, u, v, ins):
        u = np.ascontiguousarray(u, dtype=np.int32)
        v = np.ascontiguousarray(v, dtype=np.int32)
        ins = np.ascontiguousarray(ins, dtype=np.uint8)
        return lib().or_apply_batch(self._h, _p(u, C.c_int32), _p(v, C.c_int32), _p(ins, C.c_uint8), u.size)

    def row(self, x):
        k = lib().or_row(self._h, x, None, 0)
        out = np.zeros(max(k, 1), dtype=np.int32)
        lib().or_row(self._h, x, _p(out, C.c_int32), k)
        return out[:k]

    def degree(self, x):
        return lib().or_degree(self._h, x)

    def degrees(self):
        return np.array([self.degree(x) for x in range(self.n)], dtype=np.int32)

    def two_hop(self, s):
        k = lib().or_two_hop(self._h, s, None, 0)
        out = np.zeros(max(k, 1), dtype=np.int32)
        lib().or_two_hop(self._h, s, _p(out, C.c_int32), k)
        return out[:k]

    def trace(self, on=True):
        lib().or_trace_enable(self._h, 1 if on else 0)

    def trace_records(self):
        recs = []
        for i in range(lib().or_trace_count(self._h)):
            rec = {}
            for f, dt in _TRACE.items():
                k = lib().or_trace_get(self._h, i, f, None, 0)
                arr = np.zeros(max(k, 1), dtype=dt)
                lib().or_trace_get(self._h, i, f, arr.ctypes.data_as(C.c_void_p), k)
                rec[f] = arr[:k]
            recs.append(rec)
        return recs

    def compact(self, path):
        return lib().or_compact(self._h, os.fsencode(path))

    def apply_overlay(self, u, v, ins):
        """The batch applied to the overlay only (no repair)."""
        u = np.ascontiguousarray(u, dtype=np.int32)
        v = np.ascontiguousarray(v, dtype=np.int32)
        ins = np.ascontiguousarray(ins, dtype=np.uint8)
        lib().or_apply_overlay(self._h, _p(u, C.c_int32), _p(v, C.c_int32), _p(ins, C.c_uint8), u.size)

    def greedy_current(self):
        """Greedy MIS in vertex order over the current graph (becomes the membership)."""
        lib().or_greedy_current(self._h)

    def check_mis(self):
        a, b = C.c_int64(), C.c_int64()
        lib().or_check_mis(self._h, C.byref(a), C.byref(b))
        return a.value, b.value


def greedy_mis(nindex, nlist):
    nindex = np.ascontiguousarray(nindex, dtype=np.int64)
    nlist = np.ascontiguousarray(nlist, dtype=np.int32)
    out = np.zeros(nindex.size - 1, dtype=np.uint8)
    lib().or_greedy_mis(nindex.size - 1, _p(nindex, C.c_int64), _p(nlist, C.c_int32), _p(out, C.c_uint8))
    return out


# ---- the reference's own host code (oracle/_ref) ---------------------------------

def ref_lib(build_if_possible=True):
    """libmisfit_ref.so, or None when the reference tree is not on this machine."""
    global _REF
    if _REF is not None:
        return _REF
    path = _build.REF_SO
    if build_if_possible:
        built = _build.build_ref()
        if built is None and not os.path.exists(path):
            return None
    if not os.path.exists(path):
        return None
    L = C.CDLL(path)
    sig = {
        "ref_open": (_P, [C.c_char_p]),
        "ref_close": (None, [_P]),
        "ref_num_nodes": (C.c_int32, [_P]),
        "ref_base_edges": (C.c_uint64, [_P]),
        "ref_is_adjacent": (C.c_int, [_P, C.c_int32, C.c_int32]),
        "ref_apply_updates": (None, [_P, _I32P, _I32P, _U8P, C.c_int64]),
        "ref_row": (C.c_int64, [_P, C.c_int32, _I32P, C.c_int64]),
        "ref_degree": (C.c_int32, [_P, C.c_int32]),
        "ref_two_hop": (C.c_int64, [_P, C.c_int32, _I32P, C.c_int64, _I32P, C.c_int64, _I64P]),
        "ref_parse_batch_file": (C.c_int64, [_P, C.c_char_p, _I32P, _I32P, _U8P, C.c_int64]),
        "ref_list_batch_files": (C.c_int64, [C.c_char_p, C.c_char_p, C.c_int64]),
        "ref_compact": (None, [_P, C.c_char_p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _REF = L
    return L


class Reference:
    """HybridGraph of the reference, driven through oracle/_ref."""

    def __init__(self, egr_path):
        L = ref_lib()
        if L is None:
            raise RuntimeError("reference harness unavailable")
        self.L = L
        self._h = C.c_void_p(L.ref_open(os.fsencode(egr_path)))
        self.n = L.ref_num_nodes(self._h)

    def close(self):
        if self._h:
            self.L.ref_close(self._h)
            self._h = None

    def is_adjacent(self, u, v):
        return bool(self.L.ref_is_adjacent(self._h, u, v))

    def apply_updates(self, u, v, ins):
        u = np.ascontiguousarray(u, dtype=np.int32)
        v = np.ascontiguousarray(v, dtype=np.int32)
        ins = np.ascontiguousarray(ins, dtype=np.uint8)
        self.L.ref_apply_updates(self._h, _p(u, C.c_int32), _p(v, C.c_int32), _p(ins, C.c_uint8), u.size)

    def row(self, x):
        k = self.L.ref_row(self._h, x, None, 0)
        out = np.zeros(max(k, 1), dtype=np.int32)
        self.L.ref_row(self._h, x, _p(out, C.c_int32), k)
        return out[:k]

    def degree(self, x):
        return self.L.ref_degree(self._h, x)

    def two_hop(self, s):
        hl = C.c_int64()
        k = self.L.ref_two_hop(self._h, s, None, 0, None, 0, C.byref(hl))
        out = np.zeros(max(k, 1), dtype=np.int32)
        hop1 = np.zeros(max(hl.value, 1), dtype=np.int32)
        self.L.ref_two_hop(self._h, s, _p(out, C.c_int32), k, _p(hop1, C.c_int32), hl.value, C.byref(hl))
        return out[:k], hop1[: hl.value]

    def parse_batch_file(self, path):
        cap = 1 << 22
        u = np.zeros(cap, np.int32)
        v = np.zeros(cap, np.int32)
        ins = np.zeros(cap, np.uint8)
        k = self.L.ref_parse_batch_file(self._h, os.fsencode(path), _p(u, C.c_int32), _p(v, C.c_int32),
                                        _p(ins, C.c_uint8), cap)
        return u[:k].copy(), v[:k].copy(), ins[:k].copy()

    def compact(self, path):
        self.L.ref_compact(self._h, os.fsencode(path))


def ref_list_batch_files(folder):
    L = ref_lib()
    buf = C.create_string_buffer(1 << 20)
    k = L.ref_list_batch_files(os.fsencode(folder), buf, 1 << 20)
    return [x for x in buf.raw[:k].decode().split("\n") if x]


# ---- the reference's whole engines, run on the CPU (oracle/_ref/*_emul.so) ----

_EMUL = {}


def ref_emul_lib(engine="sync", build_if_possible=True):
    """libref_{sync,async}_emul.so (oracle/build.py, build_ref_emul), or None
    when it is neither built nor buildable here."""
    if engine in _EMUL:
        return _EMUL[engine]
    paths = _build.build_ref_emul() if build_if_possible else None
    path = (paths or {}).get(engine) or _build.EMUL_SO[engine]
    if not os.path.exists(path):
        return None
    L = C.CDLL(path)
    sig = {
        "re_main": (C.c_int, [C.c_int, C.POINTER(C.c_char_p)]),
        "re_set_schedule": (None, [C.c_int]),
        "re_launches": (C.c_longlong, []),
    }
    if engine == "sync":
        sig.update({
            "re_open": (_P, [C.c_char_p, C.c_longlong]),
            "re_close": (None, [_P]),
            "re_num_nodes": (C.c_int, [_P]),
            "re_set_mis": (None, [_P, _U8P]),
            "re_apply_batch": (C.c_longlong, [_P, _I32P, _I32P, _U8P, C.c_longlong]),
            "re_sub_batch": (C.c_int, [_P, C.c_longlong, _I64P]),
            "re_get_mis": (None, [_P, _U8P]),
            "re_get_cluster_ids": (None, [_P, _I32P]),
            "re_max_csr": (C.c_longlong, [_P]),
            "re_degree": (C.c_int, [_P, C.c_int]),
        })
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _EMUL[engine] = L
    return L


BULK_SYNCHRONOUS, SERIAL = 0, 1


class RefEngine:
    """The reference's sync engine (src/misfit/misfit.cu) on one graph, run on
    the CPU: HybridGraph + GPUVertexClusteringGraph driven one batch at a time
    through processBatchGPUVertexClustering, the kernels emulated thread by
    thread.  `schedule` selects how the clustering kernel's threads
    interleave (BULK_SYNCHRONOUS: every thread reads the pre-launch cluster
    ids, the highest thread index writes last -- the oracle's and the
    library's schedule; SERIAL: threads run one after another)."""

    def __init__(self, egr_path, max_csr, schedule=BULK_SYNCHRONOUS):
        L = ref_emul_lib("sync")
        if L is None:
            raise RuntimeError("reference engine emulation unavailable")
        self.L = L
        self.schedule = schedule
        self._h = C.c_void_p(L.re_open(os.fsencode(egr_path), int(max_csr)))
        self.n = L.re_num_nodes(self._h)

    def close(self):
        if self._h:
            self.L.re_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_mis(self, mis):
        mis = np.ascontiguousarray(mis, dtype=np.uint8)
        self.L.re_set_mis(self._h, _p(mis, C.c_uint8))

    def apply_batch(self, u, v, ins):
        """Returns [(edges, rows, clusters)] per sub-batch, in order."""
        u = np.ascontiguousarray(u, dtype=np.int32)
        v = np.ascontiguousarray(v, dtype=np.int32)
        ins = np.ascontiguousarray(ins, dtype=np.uint8)
        self.L.re_set_schedule(self.schedule)
        k = self.L.re_apply_batch(self._h, _p(u, C.c_int32), _p(v, C.c_int32), _p(ins, C.c_uint8), u.size)
        out = np.zeros(3, np.int64)
        recs = []
        for i in range(k):
            self.L.re_sub_batch(self._h, i, _p(out, C.c_int64))
            recs.append(tuple(int(x) for x in out))
        return recs

    def get_mis(self):
        out = np.zeros(self.n, np.uint8)
        self.L.re_get_mis(self._h, _p(out, C.c_uint8))
        return out

    def cluster_ids(self):
        out = np.zeros(self.n, np.int32)
        self.L.re_get_cluster_ids(self._h, _p(out, C.c_int32))
        return out

    @property
    def max_csr(self):
        return self.L.re_max_csr(self._h)


def run_reference_main(engine, args, cwd, schedule=BULK_SYNCHRONOUS, skip_compaction=False, timeout=600):
    """Run the reference engine's own main() (the 5-argument CLI of
    bin/misfit or bin/misfit_async) on the CPU in a child process whose
    working directory is `cwd`.  Returns (exit code, stdout)."""
    import subprocess
    import sys
    if ref_emul_lib(engine) is None:
        raise RuntimeError("reference engine emulation unavailable")
    path = _build.EMUL_SO[engine]
    code = ("import ctypes,sys\n"
            "L=ctypes.CDLL(sys.argv[1]); L.re_set_schedule(int(sys.argv[2]))\n"
            "a=[x.encode() for x in sys.argv[3:]]\n"
            "arr=(ctypes.c_char_p*len(a))(*a)\n"
            "sys.stdout.flush(); rc=L.re_main(len(a),arr)\n"
            "sys.exit(rc)\n")
    env = dict(os.environ)
    if skip_compaction:
        env["MISFIT_SKIP_COMPACTION"] = "1"
    else:
        env.pop("MISFIT_SKIP_COMPACTION", None)
    argv0 = "misfit" if engine == "sync" else "misfit_async"
    r = subprocess.run([sys.executable, "-c", code, path, str(schedule), argv0] + [str(a) for a in args],
                       cwd=cwd, env=env, capture_output=True, text=True, timeout=timeout)
    return r.returncode, r.stdout + r.stderr
