"""ctypes binding of libmisfit_gb (include/misfit_gb.h).

This is the reference-side binding a Python caller would add: one class per
graph context, numpy arrays in and out.  It loads the in-tree library built
by ``misfit_gb300/build.py`` and raises immediately when it is missing --
there is no fallback implementation.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libmisfit_gb.so")

# the symbols include/misfit_gb.h declares
EXPORTS = [
    "mf_version", "mf_status_string", "mf_last_error", "mf_open_egr", "mf_open_csr", "mf_close",
    "mf_num_nodes", "mf_num_base_entries", "mf_set_mis", "mf_get_mis", "mf_mis_size", "mf_greedy_mis",
    "mf_flag_updates", "mf_flag_updates_noalloc", "mf_apply_batch", "mf_apply_batch_device", "mf_apply_batch_async", "mf_collect", "mf_sync",
    "mf_last_batch_stats", "mf_get_tuning", "mf_set_tuning", "mf_get_row", "mf_get_degrees", "mf_is_adjacent", "mf_get_max_csr",
    "mf_set_max_csr", "mf_get_cluster_ids", "mf_check_mis", "mf_set_exact", "mf_compact", "mf_read_mis_file",
    "mf_write_mis_file", "mf_read_batch_file", "mf_parse_batch_file", "mf_list_batch_files", "mf_free", "mf_trace_enable",
    "mf_trace_count", "mf_trace_get", "mf_stage_name", "mf_profile_enable", "mf_profile_reset",
    "mf_profile_read", "mf_kernel_launches", "mf_allocations",
    "mf_pool_create", "mf_pool_destroy", "mf_pool_add_graph", "mf_pool_submit", "mf_pool_wait", "mf_pool_drain",
    "mf_pool_get_mis", "mf_pool_stats_get", "mf_pool_set_budget",
    "mf_batched_default_opts", "mf_apply_batches", "mf_pool_set_batching",
]


class BatchStats(C.Structure):
    _fields_ = [
        ("updates", C.c_int64), ("sub_batches", C.c_int64), ("seeds", C.c_int64),
        ("candidates", C.c_int64), ("clusters", C.c_int64), ("processed_edges", C.c_int64),
        ("exact_sizes", C.c_int64), ("max_csr", C.c_int64), ("repair_rounds", C.c_int64),
        ("device_ms", C.c_double), ("packed_total", C.c_int64), ("row_degree_total", C.c_int64),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Tuning(C.Structure):
    _fields_ = [("pull_long", C.c_int64), ("heavy_min", C.c_int64), ("big_threshold", C.c_int64),
                ("first_bound", C.c_int64), ("cand_push", C.c_int64),
                ("pull_sizes", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class PoolStats(C.Structure):
    _fields_ = [
        ("graphs", C.c_int64), ("completed", C.c_int64), ("updates", C.c_int64), ("errors", C.c_int64),
        ("evictions", C.c_int64), ("restores", C.c_int64), ("trims", C.c_int64), ("over_budget", C.c_int64),
        ("resident_bytes", C.c_int64), ("peak_resident_bytes", C.c_int64),
        ("batched_steps", C.c_int64), ("batched_requests", C.c_int64), ("handed_to_workers", C.c_int64),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchedOpts(C.Structure):
    _fields_ = [
        ("block", C.c_int), ("ctas_per_sm", C.c_int), ("max_cta_updates", C.c_int64),
        ("max_cta_vertices", C.c_int32), ("use_graph", C.c_int), ("path_threads", C.c_int),
        ("pool_idle_first", C.c_int),
    ]


class BatchedStats(C.Structure):
    _fields_ = [
        ("kernel_items", C.c_int64), ("path_items", C.c_int64), ("updates", C.c_int64),
        ("kernel_ms", C.c_double), ("wall_ms", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class MisfitError(RuntimeError):
    def __init__(self, status, what):
        super().__init__("%s (status %d): %s" % (what, status, _lib().mf_last_error().decode()))
        self.status = status


_LIB = None

NOALLOC_MAX_UPDATES = 65536  # MF_NOALLOC_MAX_UPDATES

_P = C.c_void_p
_I32P = C.POINTER(C.c_int32)
_I64P = C.POINTER(C.c_int64)
_U8P = C.POINTER(C.c_uint8)


def _lib():
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise ImportError("libmisfit_gb.so is not built (%s); run misfit_gb300/build.py" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    sig = {
        "mf_version": (C.c_int, []),
        "mf_status_string": (C.c_char_p, [C.c_int]),
        "mf_last_error": (C.c_char_p, []),
        "mf_open_egr": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(_P)]),
        "mf_open_csr": (C.c_int, [C.c_int32, _I64P, _I32P, C.c_int, C.POINTER(_P)]),
        "mf_close": (C.c_int, [_P]),
        "mf_num_nodes": (C.c_int, [_P, _I32P]),
        "mf_num_base_entries": (C.c_int, [_P, _I64P]),
        "mf_set_mis": (C.c_int, [_P, _U8P, C.c_int64]),
        "mf_get_mis": (C.c_int, [_P, _U8P, C.c_int64]),
        "mf_mis_size": (C.c_int, [_P, _I64P]),
        "mf_greedy_mis": (C.c_int, [_P, _U8P, C.c_int64]),
        "mf_flag_updates": (C.c_int, [_P, _I32P, _I32P, C.c_int64, _U8P]),
        "mf_flag_updates_noalloc": (C.c_int, [_P, _I32P, _I32P, C.c_int64, _U8P]),
        "mf_apply_batch": (C.c_int, [_P, _I32P, _I32P, _U8P, C.c_int64]),
        "mf_apply_batch_device": (C.c_int, [_P, _P, _P, _P, C.c_int64]),
        "mf_apply_batch_async": (C.c_int, [_P, _I32P, _I32P, _U8P, C.c_int64]),
        "mf_collect": (C.c_int, [_P, C.c_void_p]),
        "mf_sync": (C.c_int, [_P]),
        "mf_last_batch_stats": (C.c_int, [_P, C.POINTER(BatchStats)]),
        "mf_get_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
        "mf_set_tuning": (C.c_int, [_P, C.POINTER(Tuning)]),
        "mf_get_row": (C.c_int, [_P, C.c_int32, _I32P, C.c_int64, _I64P]),
        "mf_get_degrees": (C.c_int, [_P, _I32P, C.c_int64]),
        "mf_is_adjacent": (C.c_int, [_P, C.c_int32, C.c_int32, C.POINTER(C.c_int)]),
        "mf_get_max_csr": (C.c_int, [_P, _I64P]),
        "mf_set_max_csr": (C.c_int, [_P, C.c_int64]),
        "mf_get_cluster_ids": (C.c_int, [_P, _I32P, C.c_int64]),
        "mf_check_mis": (C.c_int, [_P, _I64P, _I64P]),
        "mf_set_exact": (C.c_int, [_P, C.c_int]),
        "mf_compact": (C.c_int, [_P, C.c_char_p, C.c_int]),
        "mf_read_mis_file": (C.c_int, [C.c_char_p, C.c_int32, _U8P, _I64P]),
        "mf_write_mis_file": (C.c_int, [C.c_char_p, _U8P, C.c_int32]),
        "mf_read_batch_file": (C.c_int, [C.c_char_p, C.c_int32, C.POINTER(_I32P), C.POINTER(_I32P), _I64P]),
        "mf_parse_batch_file": (C.c_int, [_P, C.c_char_p, C.POINTER(_I32P), C.POINTER(_I32P), C.POINTER(_U8P), _I64P]),
        "mf_list_batch_files": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p), _I64P]),
        "mf_free": (None, [C.c_void_p]),
        "mf_stage_name": (C.c_char_p, [C.c_int]),
        "mf_profile_enable": (C.c_int, [_P, C.c_int]),
        "mf_profile_reset": (C.c_int, [_P]),
        "mf_profile_read": (C.c_int, [_P, C.POINTER(C.c_double), _I64P, C.POINTER(C.c_double), C.c_int]),
        "mf_kernel_launches": (C.c_int64, []),
        "mf_allocations": (C.c_int64, []),
        "mf_trace_enable": (C.c_int, [_P, C.c_int]),
        "mf_trace_count": (C.c_int, [_P, _I64P]),
        "mf_trace_get": (C.c_int, [_P, C.c_int64, C.c_int, C.c_void_p, C.c_int64, _I64P]),
        "mf_pool_create": (C.c_int, [C.c_int, C.c_int64, C.c_int, C.POINTER(_P)]),
        "mf_pool_destroy": (C.c_int, [_P]),
        "mf_pool_add_graph": (C.c_int, [_P, C.c_int32, _I64P, _I32P, _U8P, _I32P]),
        "mf_pool_submit": (C.c_int, [_P, C.c_int32, _I32P, _I32P, _U8P, C.c_int64, _I64P]),
        "mf_pool_wait": (C.c_int, [_P, C.c_int64, C.POINTER(C.c_double)]),
        "mf_pool_drain": (C.c_int, [_P]),
        "mf_pool_get_mis": (C.c_int, [_P, C.c_int32, _U8P, C.c_int64]),
        "mf_pool_stats_get": (C.c_int, [_P, C.POINTER(PoolStats)]),
        "mf_pool_set_budget": (C.c_int, [_P, C.c_int64]),
        "mf_batched_default_opts": (C.c_int, [C.POINTER(BatchedOpts)]),
        "mf_pool_set_batching": (C.c_int, [_P, C.POINTER(BatchedOpts)]),
        "mf_apply_batches": (C.c_int, [C.POINTER(_P), C.POINTER(_I32P), C.POINTER(_I32P), C.POINTER(_U8P), _I64P,
                                       C.c_int64, C.POINTER(BatchedOpts), C.POINTER(BatchedStats)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def load_library():
    """Load libmisfit_gb.so (raises ImportError when it is not built)."""
    return _lib()


def _check(status, what):
    if status != 0:
        raise MisfitError(status, what)


def _ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _u8(a):
    return np.ascontiguousarray(a, dtype=np.uint8)


_TRACE_FIELDS = {0: np.int64, 1: np.int32, 2: np.int32, 3: np.int32, 4: np.int32, 5: np.uint8, 6: np.int64}


class Graph:
    """One device-resident graph context (mf_ctx)."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle)
        n = C.c_int32()
        _check(_lib().mf_num_nodes(self._h, C.byref(n)), "mf_num_nodes")
        self.n = n.value

    @classmethod
    def open_egr(cls, path, gpu=0):
        h = C.c_void_p()
        _check(_lib().mf_open_egr(os.fsencode(path), gpu, C.byref(h)), "mf_open_egr")
        return cls(h.value)

    @classmethod
    def from_csr(cls, nindex, nlist, gpu=0):
        nindex = np.ascontiguousarray(nindex, dtype=np.int64)
        nlist = np.ascontiguousarray(nlist, dtype=np.int32)
        h = C.c_void_p()
        n = nindex.size - 1
        _check(_lib().mf_open_csr(n, _ptr(nindex, C.c_int64), _ptr(nlist, C.c_int32), gpu, C.byref(h)),
               "mf_open_csr")
        return cls(h.value)

    def close(self):
        if self._h:
            _check(_lib().mf_close(self._h), "mf_close")
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_mis(self, mis):
        mis = _u8(mis)
        _check(_lib().mf_set_mis(self._h, _ptr(mis, C.c_uint8), mis.size), "mf_set_mis")

    def get_mis(self):
        out = np.zeros(self.n, dtype=np.uint8)
        _check(_lib().mf_get_mis(self._h, _ptr(out, C.c_uint8), self.n), "mf_get_mis")
        return out

    def greedy_mis(self):
        out = np.zeros(self.n, dtype=np.uint8)
        _check(_lib().mf_greedy_mis(self._h, _ptr(out, C.c_uint8), self.n), "mf_greedy_mis")
        return out

    def flag_updates(self, u, v):
        u, v = _i32(u), _i32(v)
        out = np.zeros(u.size, dtype=np.uint8)
        _check(_lib().mf_flag_updates(self._h, _ptr(u, C.c_int32), _ptr(v, C.c_int32), u.size,
                                      _ptr(out, C.c_uint8)), "mf_flag_updates")
        return out

    def flag_updates_noalloc(self, u, v):
        """mf_flag_updates_noalloc: at most NOALLOC_MAX_UPDATES pairs, no device allocation."""
        u, v = _i32(u), _i32(v)
        out = np.zeros(u.size, dtype=np.uint8)
        _check(_lib().mf_flag_updates_noalloc(self._h, _ptr(u, C.c_int32), _ptr(v, C.c_int32), u.size,
                                              _ptr(out, C.c_uint8)), "mf_flag_updates_noalloc")
        return out

    def apply_batch(self, u, v, ins):
        u, v, ins = _i32(u), _i32(v), _u8(ins)
        _check(_lib().mf_apply_batch(self._h, _ptr(u, C.c_int32), _ptr(v, C.c_int32), _ptr(ins, C.c_uint8),
                                     u.size), "mf_apply_batch")

    def apply_batch_device(self, d_u, d_v, d_ins, m):
        """Device pointers (ints), e.g. torch ``tensor.data_ptr()``."""
        _check(_lib().mf_apply_batch_device(self._h, C.c_void_p(d_u), C.c_void_p(d_v), C.c_void_p(d_ins), m),
               "mf_apply_batch_device")

    def apply_batch_async(self, u, v, ins):
        """Queue a batch for the pipelined engine; it runs on the context's
        worker thread.  The arrays are kept alive here until collected."""
        u, v, ins = _i32(u), _i32(v), _u8(ins)
        _check(_lib().mf_apply_batch_async(self._h, _ptr(u, C.c_int32), _ptr(v, C.c_int32),
                                           _ptr(ins, C.c_uint8), u.size), "mf_apply_batch_async")
        self._queued = getattr(self, "_queued", []) + [(u, v, ins)]

    def collect(self):
        """Wait for the oldest queued batch; its statistics (raises its error)."""
        st = BatchStats()
        try:
            _check(_lib().mf_collect(self._h, C.c_void_p(C.addressof(st))), "mf_collect")
        finally:
            q = getattr(self, "_queued", [])
            self._queued = q[1:]
        return st.as_dict()

    def sync(self):
        try:
            _check(_lib().mf_sync(self._h), "mf_sync")
        finally:
            self._queued = []

    def tuning(self):
        t = Tuning()
        _check(_lib().mf_get_tuning(self._h, C.byref(t)), "mf_get_tuning")
        return t.as_dict()

    def set_tuning(self, **kw):
        """Load-balancing settings (mf_tuning: pull_long, heavy_min,
        big_threshold, first_bound, cand_push, pull_sizes); unnamed ones keep
        their values.  Results never change."""
        cur = self.tuning()
        cur.update(kw)
        t = Tuning(**cur)
        _check(_lib().mf_set_tuning(self._h, C.byref(t)), "mf_set_tuning")

    def stats(self):
        st = BatchStats()
        _check(_lib().mf_last_batch_stats(self._h, C.byref(st)), "mf_last_batch_stats")
        return st.as_dict()

    def row(self, x):
        ln = C.c_int64()
        _check(_lib().mf_get_row(self._h, x, None, 0, C.byref(ln)), "mf_get_row")
        out = np.zeros(max(ln.value, 1), dtype=np.int32)
        _check(_lib().mf_get_row(self._h, x, _ptr(out, C.c_int32), ln.value, C.byref(ln)), "mf_get_row")
        return out[: ln.value]

    def degrees(self):
        out = np.zeros(self.n, dtype=np.int32)
        _check(_lib().mf_get_degrees(self._h, _ptr(out, C.c_int32), self.n), "mf_get_degrees")
        return out

    def cluster_ids(self):
        out = np.zeros(self.n, dtype=np.int32)
        _check(_lib().mf_get_cluster_ids(self._h, _ptr(out, C.c_int32), self.n), "mf_get_cluster_ids")
        return out

    def is_adjacent(self, u, v):
        r = C.c_int()
        _check(_lib().mf_is_adjacent(self._h, u, v, C.byref(r)), "mf_is_adjacent")
        return bool(r.value)

    @property
    def max_csr(self):
        v = C.c_int64()
        _check(_lib().mf_get_max_csr(self._h, C.byref(v)), "mf_get_max_csr")
        return v.value

    @max_csr.setter
    def max_csr(self, value):
        _check(_lib().mf_set_max_csr(self._h, int(value)), "mf_set_max_csr")

    def parse_batch_file(self, path):
        """mf_parse_batch_file: (u, v, ins) of a batch file, parsed and flagged on the device."""
        pu, pv, pi = _I32P(), _I32P(), _U8P()
        m = C.c_int64()
        _check(_lib().mf_parse_batch_file(self._h, os.fsencode(path), C.byref(pu), C.byref(pv), C.byref(pi),
                                          C.byref(m)), "mf_parse_batch_file")
        try:
            k = m.value
            u = np.ctypeslib.as_array(pu, shape=(max(k, 1),))[:k].copy()
            v = np.ctypeslib.as_array(pv, shape=(max(k, 1),))[:k].copy()
            ins = np.ctypeslib.as_array(pi, shape=(max(k, 1),))[:k].copy()
        finally:
            _lib().mf_free(C.cast(pu, C.c_void_p))
            _lib().mf_free(C.cast(pv, C.c_void_p))
            _lib().mf_free(C.cast(pi, C.c_void_p))
        return u, v, ins

    def set_exact(self, on=True):
        """Exact-MIS mode: independent, maximal membership after every batch."""
        _check(_lib().mf_set_exact(self._h, 1 if on else 0), "mf_set_exact")

    def check_mis(self):
        a, b = C.c_int64(), C.c_int64()
        _check(_lib().mf_check_mis(self._h, C.byref(a), C.byref(b)), "mf_check_mis")
        return a.value, b.value

    def compact(self, path, rebase=False):
        _check(_lib().mf_compact(self._h, os.fsencode(path), 1 if rebase else 0), "mf_compact")

    def profile(self, on=True):
        """True/1: all stages; 2: the k_lb_push_hop launches and the
        candidates' pull only; False/0: off;
        adding 4 also counts each batch's algorithmic work (stats packed_total,
        row_degree_total), at the cost of exact 2-hop sizes in every sub-batch."""
        level = 1 if on is True else (0 if on is False else int(on))
        _check(_lib().mf_profile_enable(self._h, level), "mf_profile_enable")

    def profile_reset(self):
        _check(_lib().mf_profile_reset(self._h), "mf_profile_reset")

    def profile_read(self):
        """{stage: (device ms, occurrences, algorithmic bytes)} since the last reset."""
        k = 16
        ms = (C.c_double * k)()
        calls = (C.c_int64 * k)()
        nbytes = (C.c_double * k)()
        _check(_lib().mf_profile_read(self._h, ms, calls, nbytes, k), "mf_profile_read")
        out = {}
        for i in range(k):
            name = _lib().mf_stage_name(i)
            if name is None:
                break
            out[name.decode()] = (ms[i], calls[i], nbytes[i])
        return out

    def trace(self, on=True):
        _check(_lib().mf_trace_enable(self._h, 1 if on else 0), "mf_trace_enable")

    def trace_records(self):
        cnt = C.c_int64()
        _check(_lib().mf_trace_count(self._h, C.byref(cnt)), "mf_trace_count")
        recs = []
        for i in range(cnt.value):
            rec = {}
            for field, dt in _TRACE_FIELDS.items():
                ln = C.c_int64()
                _check(_lib().mf_trace_get(self._h, i, field, None, 0, C.byref(ln)), "mf_trace_get")
                arr = np.zeros(max(ln.value, 1), dtype=dt)
                _check(_lib().mf_trace_get(self._h, i, field, arr.ctypes.data_as(C.c_void_p), ln.value,
                                           C.byref(ln)), "mf_trace_get")
                rec[field] = arr[: ln.value]
            recs.append(rec)
        return recs


def kernel_launches():
    """Kernels launched by libmisfit_gb in this process so far."""
    return int(_lib().mf_kernel_launches())


def allocations():
    """Device and pinned-host allocations made by libmisfit_gb in this
    process so far."""
    return int(_lib().mf_allocations())


def read_mis_file(path, n):
    out = np.zeros(n, dtype=np.uint8)
    lines = C.c_int64()
    _check(_lib().mf_read_mis_file(os.fsencode(path), n, _ptr(out, C.c_uint8), C.byref(lines)),
           "mf_read_mis_file")
    return out, lines.value


def write_mis_file(path, mis):
    mis = _u8(mis)
    _check(_lib().mf_write_mis_file(os.fsencode(path), _ptr(mis, C.c_uint8), mis.size), "mf_write_mis_file")


def read_batch_file(path, n):
    u = _I32P()
    v = _I32P()
    m = C.c_int64()
    _check(_lib().mf_read_batch_file(os.fsencode(path), n, C.byref(u), C.byref(v), C.byref(m)),
           "mf_read_batch_file")
    try:
        a = np.ctypeslib.as_array(u, shape=(max(m.value, 1),))[: m.value].copy()
        b = np.ctypeslib.as_array(v, shape=(max(m.value, 1),))[: m.value].copy()
    finally:
        _lib().mf_free(u)
        _lib().mf_free(v)
    return a, b


def list_batch_files(folder):
    names = C.c_void_p()
    cnt = C.c_int64()
    _check(_lib().mf_list_batch_files(os.fsencode(folder), C.byref(names), C.byref(cnt)), "mf_list_batch_files")
    try:
        s = C.string_at(names).decode() if names.value else ""
    finally:
        _lib().mf_free(names)
    return [x for x in s.split("\n") if x]


class Pool:
    """A serving pool (mf_pool): many graphs on one GPU, batches served by
    host worker threads under an HBM budget, idle graphs evicted to pinned
    host memory."""

    def __init__(self, hbm_budget, workers=4, gpu=0):
        h = C.c_void_p()
        _check(_lib().mf_pool_create(gpu, int(hbm_budget), int(workers), C.byref(h)), "mf_pool_create")
        self._h = h
        self._n = {}

    def add_graph(self, nindex, nlist, mis):
        nindex = np.ascontiguousarray(nindex, dtype=np.int64)
        nlist = np.ascontiguousarray(nlist, dtype=np.int32)
        mis = _u8(mis)
        gid = C.c_int32()
        n = nindex.size - 1
        _check(_lib().mf_pool_add_graph(self._h, n, _ptr(nindex, C.c_int64), _ptr(nlist, C.c_int32),
                                        _ptr(mis, C.c_uint8), C.byref(gid)), "mf_pool_add_graph")
        self._n[gid.value] = n
        return gid.value

    def submit(self, gid, u, v, ins):
        u, v, ins = _i32(u), _i32(v), _u8(ins)
        rid = C.c_int64()
        _check(_lib().mf_pool_submit(self._h, gid, _ptr(u, C.c_int32), _ptr(v, C.c_int32), _ptr(ins, C.c_uint8),
                                     u.size, C.byref(rid)), "mf_pool_submit")
        return rid.value

    def wait(self, rid):
        lat = C.c_double()
        _check(_lib().mf_pool_wait(self._h, rid, C.byref(lat)), "mf_pool_wait")
        return lat.value

    def drain(self):
        _check(_lib().mf_pool_drain(self._h), "mf_pool_drain")

    def get_mis(self, gid):
        out = np.zeros(self._n[gid], dtype=np.uint8)
        _check(_lib().mf_pool_get_mis(self._h, gid, _ptr(out, C.c_uint8), out.size), "mf_pool_get_mis")
        return out

    def set_batching(self, opts=None, on=True):
        """Continuous batching of small requests through mf_apply_batches
        (mf_pool_set_batching); opts None = library defaults; on=False stops it."""
        if not on:
            _check(_lib().mf_pool_set_batching(self._h, None), "mf_pool_set_batching")
            return
        o = opts if opts is not None else batched_opts()
        _check(_lib().mf_pool_set_batching(self._h, C.byref(o)), "mf_pool_set_batching")

    def set_budget(self, hbm_budget):
        _check(_lib().mf_pool_set_budget(self._h, int(hbm_budget)), "mf_pool_set_budget")

    def stats(self):
        st = PoolStats()
        _check(_lib().mf_pool_stats_get(self._h, C.byref(st)), "mf_pool_stats_get")
        return st.as_dict()

    def close(self):
        if self._h:
            _check(_lib().mf_pool_destroy(self._h), "mf_pool_destroy")
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def batched_opts(**kw):
    """mf_batched_opts with the library defaults, then the given fields."""
    o = BatchedOpts()
    _check(_lib().mf_batched_default_opts(C.byref(o)), "mf_batched_default_opts")
    for k, val in kw.items():
        setattr(o, k, val)
    return o


def apply_batches(graphs, batches, opts=None):
    """One batch per graph in one step (mf_apply_batches): graphs is a list of
    Graph, batches a list of (u, v, ins).  Returns the step's stats dict."""
    if len(graphs) != len(batches):
        raise ValueError("one batch per graph")
    k = len(graphs)
    keep = []
    hs = (_P * k)()
    us, vs, ins_ = (_I32P * k)(), (_I32P * k)(), (_U8P * k)()
    ms = np.zeros(max(k, 1), dtype=np.int64)
    for j, (g, (u, v, ins)) in enumerate(zip(graphs, batches)):
        u, v, ins = _i32(u), _i32(v), _u8(ins)
        keep.extend([u, v, ins])
        hs[j] = g._h.value
        us[j] = _ptr(u, C.c_int32)
        vs[j] = _ptr(v, C.c_int32)
        ins_[j] = _ptr(ins, C.c_uint8)
        ms[j] = u.size
    st = BatchedStats()
    o = opts if opts is not None else batched_opts()
    _check(_lib().mf_apply_batches(hs, us, vs, ins_, _ptr(ms, C.c_int64), k, C.byref(o), C.byref(st)),
           "mf_apply_batches")
    return st.as_dict()
