"""CPU execution of the batched form's one-CTA engine -- TEST INFRASTRUCTURE ONLY.

Builds ``cta_emul.cpp`` (which includes ``misfit_gb300/csrc/mf_cta.cuh``) with
g++ and runs one CTA of the engine on OS threads, so that the CPU test suite
can hold the engine's results against the oracle.  The library itself has no
CPU path; on a GPU the same source is the persistent kernel of
``mf_apply_batches``.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
BUILD = os.path.join(HERE, "_build")
SO = os.path.join(BUILD, "libcta_emul.so")
SRC = os.path.join(HERE, "cta_emul.cpp")
HDR = os.path.join(ROOT, "misfit_gb300", "csrc", "mf_cta.cuh")

_L = None
_P = C.c_void_p


def _ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def lib():
    global _L
    if _L is None:
        if not os.path.exists(SO) or any(os.path.getmtime(s) > os.path.getmtime(SO) for s in (SRC, HDR)):
            os.makedirs(BUILD, exist_ok=True)
            tmp = SO + ".tmp%d" % os.getpid()
            subprocess.check_call(["g++", "-O2", "-std=c++17", "-pthread", "-fPIC", "-shared", SRC, "-o", tmp])
            os.replace(tmp, SO)
        L = C.CDLL(SO)
        I32P, I64P, U8P = C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_uint8)
        sig = {
            "eg_create": (_P, [C.c_int32, I64P, I32P]),
            "eg_destroy": (None, [_P]),
            "eg_set_mis": (None, [_P, U8P]),
            "eg_get_mis": (None, [_P, U8P]),
            "eg_get_cid": (None, [_P, I32P]),
            "eg_degrees": (None, [_P, I32P]),
            "eg_max_csr": (C.c_int64, [_P]),
            "eg_set_max_csr": (None, [_P, C.c_int64]),
            "eg_last": (I64P, [_P]),
            "eg_row": (C.c_int64, [_P, C.c_int32, I32P, C.c_int64]),
            "eg_apply": (C.c_int64, [_P, I32P, I32P, U8P, C.c_int64, C.c_int]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _L = L
    return _L


class EmulGraph:
    """One graph in the engine's device layout, batches run by an emulated CTA."""

    def __init__(self, nindex, nlist):
        nindex = np.ascontiguousarray(nindex, dtype=np.int64)
        nlist = np.ascontiguousarray(nlist, dtype=np.int32)
        self.n = nindex.size - 1
        self._h = C.c_void_p(lib().eg_create(self.n, _ptr(nindex, C.c_int64), _ptr(nlist, C.c_int32)))

    def close(self):
        if self._h:
            lib().eg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def max_csr(self):
        return lib().eg_max_csr(self._h)

    @max_csr.setter
    def max_csr(self, v):
        lib().eg_set_max_csr(self._h, int(v))

    def set_mis(self, mis):
        mis = np.ascontiguousarray(mis, dtype=np.uint8)
        lib().eg_set_mis(self._h, _ptr(mis, C.c_uint8))

    def get_mis(self):
        out = np.zeros(self.n, dtype=np.uint8)
        lib().eg_get_mis(self._h, _ptr(out, C.c_uint8))
        return out

    def cluster_ids(self):
        out = np.zeros(self.n, dtype=np.int32)
        lib().eg_get_cid(self._h, _ptr(out, C.c_int32))
        return out

    def degrees(self):
        out = np.zeros(self.n, dtype=np.int32)
        lib().eg_degrees(self._h, _ptr(out, C.c_int32))
        return out

    def row(self, x):
        cap = 64
        while True:
            out = np.zeros(cap, dtype=np.int32)
            k = lib().eg_row(self._h, int(x), _ptr(out, C.c_int32), cap)
            if k <= cap:
                return out[:k]
            cap = int(k)

    def last(self):
        p = lib().eg_last(self._h)
        return [p[i] for i in range(16)]

    def apply_batch(self, u, v, ins, threads=32):
        u = np.ascontiguousarray(u, dtype=np.int32)
        v = np.ascontiguousarray(v, dtype=np.int32)
        ins = np.ascontiguousarray(ins, dtype=np.uint8)
        return lib().eg_apply(self._h, _ptr(u, C.c_int32), _ptr(v, C.c_int32), _ptr(ins, C.c_uint8), u.size,
                              int(threads))
