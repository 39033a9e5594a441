"""ctypes binding of include/slothdb_gb300.h and a thin Python host API.

The library is the in-tree ``slothdb_gb300/_build/libslothdb_gb300.so``.
Loading fails loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

GB_OK = 0
GB_ERR_INVALID = 1
GB_ERR_UNSUPPORTED = 3
GB_ERR_TIMEOUT = 4
GB_ERR_BUDGET = 8
STATUS_NAMES = {0: "OK", 1: "INVALID", 2: "OOM", 3: "UNSUPPORTED", 4: "TIMEOUT", 5: "CUDA", 6: "CORRUPT",
                7: "STATE", 8: "BUDGET"}

SMALLINT, INTEGER, BIGINT, DOUBLE, VARCHAR = 1, 2, 3, 4, 5
COUNT_STAR, COUNT, SUM, AVG, MIN, MAX, COUNT_DISTINCT = 0, 1, 2, 3, 4, 5, 6
EQ, NE, LT, LE, GT, GE = 0, 1, 2, 3, 4, 5
IN, STR_EQ, STR_NE, LIKE, NOT_LIKE = 6, 7, 8, 9, 10
MEM_HOST, MEM_DEVICE = 0, 1

NP_TYPES = {SMALLINT: np.int16, INTEGER: np.int32, BIGINT: np.int64, DOUBLE: np.float64}
AGG_NAMES = {"count_star": COUNT_STAR, "count": COUNT, "sum": SUM, "avg": AVG, "min": MIN, "max": MAX,
             "count_distinct": COUNT_DISTINCT}
CMP_NAMES = {"==": EQ, "=": EQ, "!=": NE, "<>": NE, "<": LT, "<=": LE, ">": GT, ">=": GE, "in": IN, "like": LIKE,
             "not like": NOT_LIKE}


class GbError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), msg))
        self.status = status


class AggDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("col", C.c_int32)]


class Filter(C.Structure):
    _fields_ = [("col", C.c_int32), ("op", C.c_int32), ("i_const", C.c_int64), ("d_const", C.c_double),
                ("data", C.c_void_p), ("n", C.c_uint64)]


def _filters(filters, types):
    """gb_filter array for (col, op, const) triples; returns (array, buffers
    it points into).  op: '=', '!=', '<', '<=', '>', '>=' (a VARCHAR column
    compares its bytes with const for '=' / '!='), 'in' (const: integers),
    'like' / 'not like' (const: the needle of LIKE '%needle%')."""
    fl = (Filter * max(1, len(filters)))()
    keep = []
    for i, (col, op, const) in enumerate(filters):
        opc = CMP_NAMES[op] if isinstance(op, str) else int(op)
        if opc == IN:
            a = np.ascontiguousarray(np.asarray(list(const), dtype=np.int64))
            keep.append(a)
            fl[i] = Filter(col, opc, 0, 0.0, a.ctypes.data if len(a) else None, len(a))
        elif types[col] == VARCHAR:
            if opc in (EQ, NE):
                opc += STR_EQ - EQ
            b = (C.c_char * max(1, len(const))).from_buffer_copy(bytes(const) or b"\0")
            keep.append(b)
            fl[i] = Filter(col, opc, 0, 0.0, C.addressof(b), len(const))
        elif types[col] == DOUBLE:
            fl[i] = Filter(col, opc, 0, float(const))
        else:
            fl[i] = Filter(col, opc, int(const), 0.0)
    return fl, keep


class AggSpec(C.Structure):
    _fields_ = [("n_cols", C.c_uint32), ("col_types", C.POINTER(C.c_int32)),
                ("n_groups", C.c_uint32), ("group_cols", C.POINTER(C.c_int32)),
                ("n_aggs", C.c_uint32), ("aggs", C.POINTER(AggDesc)),
                ("n_filters", C.c_uint32), ("filters", C.POINTER(Filter)),
                ("nullable_mask", C.c_uint64), ("est_groups", C.c_uint64)]


class Col(C.Structure):
    _fields_ = [("data", C.c_void_p), ("validity", C.c_void_p), ("offsets", C.c_void_p)]


class KernelStat(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_uint64), ("ms", C.c_double)]


class Result(C.Structure):
    _fields_ = [("n_rows", C.c_uint64), ("n_cols", C.c_uint32), ("types", C.POINTER(C.c_int32)),
                ("data", C.POINTER(C.c_void_p)), ("offsets", C.POINTER(C.c_void_p)),
                ("validity", C.POINTER(C.c_void_p))]


class ServerStat(C.Structure):
    _fields_ = [("batches", C.c_uint64), ("completed", C.c_uint64), ("rejected", C.c_uint64),
                ("failed", C.c_uint64), ("queued", C.c_uint64), ("peak_admitted_bytes", C.c_uint64),
                ("busy_ms", C.c_double), ("kernel_launches", C.c_uint64), ("result_bytes", C.c_uint64)]


# every exported symbol of include/slothdb_gb300.h (checked by tests)
_SIGS = {
    "gb_last_error": (C.c_char_p, []),
    "gb_abi_version": (C.c_int, []),
    "gb_agg_create": (C.c_int, [C.POINTER(AggSpec), C.POINTER(C.c_void_p)]),
    "gb_agg_set_topn": (C.c_int, [C.c_void_p, C.c_uint32, C.c_int32, C.c_uint64]),
    "gb_agg_set_row_limit": (C.c_int, [C.c_void_p, C.c_uint64]),
    "gb_agg_ingest": (C.c_int, [C.c_void_p, C.POINTER(Col), C.c_uint64, C.c_int32, C.c_void_p]),
    "gb_agg_finalize": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gb_agg_result": (C.c_int, [C.c_void_p, C.POINTER(Result)]),
    "gb_agg_result_device": (C.c_int, [C.c_void_p, C.POINTER(Result)]),
    "gb_agg_reset": (C.c_int, [C.c_void_p]),
    "gb_agg_destroy": (None, [C.c_void_p]),
    "gb_agg_kernel_launches": (C.c_uint64, [C.c_void_p]),
    "gb_agg_row_groups_pruned": (C.c_uint64, [C.c_void_p]),
    "gb_agg_set_option": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int64]),
    "gb_agg_get_mode": (C.c_int32, [C.c_void_p]),
    "gb_agg_set_profiling": (C.c_int, [C.c_void_p, C.c_int32]),
    "gb_agg_profile": (C.c_uint32, [C.c_void_p, C.POINTER(KernelStat), C.c_uint32]),
    "gb_engine_hash_aggregate": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]),
    "gb_batch_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "gb_batch_add": (C.c_int, [C.c_void_p, C.POINTER(AggSpec), C.POINTER(Col), C.c_uint64,
                               C.POINTER(C.c_uint32)]),
    "gb_batch_set_option": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int64]),
    "gb_batch_run": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gb_batch_clear": (C.c_int, [C.c_void_p]),
    "gb_batch_size": (C.c_uint32, [C.c_void_p]),
    "gb_batch_result": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(Result)]),
    "gb_batch_result_device": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(Result)]),
    "gb_batch_slow_queries": (C.c_uint32, [C.c_void_p]),
    "gb_batch_kernel_launches": (C.c_uint64, [C.c_void_p]),
    "gb_batch_profile": (C.c_uint32, [C.c_void_p, C.POINTER(KernelStat), C.c_uint32]),
    "gb_batch_destroy": (None, [C.c_void_p]),
    "gb_agg_set_filters": (C.c_int, [C.c_void_p, C.POINTER(Filter), C.c_uint32]),
    "gb_agg_estimate_bytes": (C.c_int, [C.POINTER(AggSpec), C.c_uint64, C.POINTER(C.c_uint64)]),
    "gb_server_create": (C.c_int, [C.c_uint64, C.c_uint32, C.c_int32, C.POINTER(C.c_void_p)]),
    "gb_server_add_table": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.c_uint32, C.POINTER(Col), C.c_uint64,
                                      C.POINTER(C.c_uint32)]),
    "gb_server_submit": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint64, C.c_uint64, C.POINTER(AggSpec),
                                   C.POINTER(C.c_uint64)]),
    "gb_server_wait": (C.c_int, [C.c_void_p, C.c_uint64, C.c_int64]),
    "gb_server_result": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(Result)]),
    "gb_server_query_times": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                        C.POINTER(C.c_uint32)]),
    "gb_server_release": (C.c_int, [C.c_void_p, C.c_uint64]),
    "gb_server_set_lanes": (C.c_int, [C.c_void_p, C.c_uint32]),
    "gb_server_stats": (C.c_int, [C.c_void_p, C.POINTER(ServerStat)]),
    "gb_server_destroy": (None, [C.c_void_p]),
    "gb_hash_aggregate_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64), C.c_void_p]),
    "gb_pq_open": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]),
    "gb_pq_num_row_groups": (C.c_uint32, [C.c_void_p]),
    "gb_pq_num_rows": (C.c_uint64, [C.c_void_p]),
    "gb_pq_num_columns": (C.c_uint32, [C.c_void_p]),
    "gb_pq_column_info": (C.c_int, [C.c_void_p, C.c_uint32, C.c_char_p, C.c_uint32, C.POINTER(C.c_int32)]),
    "gb_pq_dict_sum": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int32, C.c_void_p,
                                 C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
    "gb_pq_row_group_might_match": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_int32), C.c_uint32,
                                              C.c_void_p, C.c_uint32, C.POINTER(C.c_int32)]),
    "gb_pq_upload": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gb_pq_close": (None, [C.c_void_p]),
    "gb_agg_ingest_parquet": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(C.c_int32),
                                        C.c_int32, C.c_void_p]),
    "gb_host_alloc": (C.c_int, [C.POINTER(C.c_void_p), C.c_size_t]),
    "gb_host_free": (C.c_int, [C.c_void_p]),
    "gb_device_alloc": (C.c_int, [C.POINTER(C.c_void_p), C.c_size_t]),
    "gb_device_free": (C.c_int, [C.c_void_p]),
    "gb_memcpy": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int32]),
    "gb_device_sync": (C.c_int, []),
}

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load the CUDA library (no fallback: raises if it cannot be loaded)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError("GB300 library not built (%s); run __graft_entry__.build()" % path)
        _build.build_lib()
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def declared_symbols():
    return sorted(_SIGS)


def check(status: int):
    if status != GB_OK:
        raise GbError(status, load().gb_last_error().decode())


def _arr_ptr(a):
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if hasattr(a, "data_ptr"):  # torch tensor
        return a.data_ptr()
    return a.ctypes.data


def _make_spec(col_types, group_cols, aggs, filters=(), nullable=(), est_groups=0):
    """gb_agg_spec for a query; returns (spec, arrays the spec points into)."""
    col_types = list(col_types)
    group_cols = list(group_cols)
    aggs = [(AGG_NAMES[k] if isinstance(k, str) else int(k), int(c)) for k, c in aggs]
    filters = list(filters)
    ct = (C.c_int32 * len(col_types))(*col_types)
    gc = (C.c_int32 * len(group_cols))(*group_cols)
    ag = (AggDesc * len(aggs))(*[AggDesc(k, c) for k, c in aggs])
    fl, fkeep = _filters(filters, col_types)
    mask = 0
    for c in nullable:
        mask |= 1 << int(c)
    spec = AggSpec(len(col_types), ct, len(group_cols), gc, len(aggs), ag,
                   len(filters), fl if filters else None, mask, int(est_groups))
    return spec, (ct, gc, ag, fl, fkeep)


def _result_bytes(r):
    """(rows, bytes) of a host result: validity words, fixed-width values,
    VARCHAR offsets and string bytes."""
    n = int(r.n_rows)
    nbytes = 0
    for c in range(r.n_cols):
        t = r.types[c]
        nbytes += (n + 63) // 64 * 8
        if t == VARCHAR:
            offs = np.frombuffer((C.c_char * ((n + 1) * 8)).from_address(r.offsets[c]), dtype=np.int64)
            nbytes += (n + 1) * 8 + int(offs[-1]) if n else 0
        else:
            nbytes += n * np.dtype(NP_TYPES[t]).itemsize
    return n, nbytes


def _read_result(r):
    """Host gb_result -> list of (values ndarray, valid bool ndarray)."""
    out = []
    n = int(r.n_rows)
    for c in range(r.n_cols):
        t = r.types[c]
        if t == VARCHAR:
            if n:
                offs = np.frombuffer((C.c_char * ((n + 1) * 8)).from_address(r.offsets[c]), dtype=np.int64).copy()
                nb = int(offs[-1])
                data = bytes((C.c_char * max(nb, 1)).from_address(r.data[c]))[:nb]
                vals = np.array([data[offs[i]:offs[i + 1]] for i in range(n)], dtype=object)
                vw = np.frombuffer((C.c_char * (((n + 63) // 64) * 8)).from_address(r.validity[c]),
                                   dtype=np.uint64)
                bits = np.unpackbits(vw.view(np.uint8), bitorder="little")[:n].astype(bool)
            else:
                vals = np.zeros(0, dtype=object)
                bits = np.zeros(0, dtype=bool)
            out.append((vals, bits))
            continue
        dt = np.dtype(NP_TYPES[t])
        if n:
            buf = (C.c_char * (n * dt.itemsize)).from_address(r.data[c])
            vals = np.frombuffer(buf, dtype=dt).copy()
            vw = np.frombuffer((C.c_char * (((n + 63) // 64) * 8)).from_address(r.validity[c]),
                               dtype=np.uint64)
            bits = np.unpackbits(vw.view(np.uint8), bitorder="little")[:n].astype(bool)
        else:
            vals = np.zeros(0, dtype=dt)
            bits = np.zeros(0, dtype=bool)
        out.append((vals, bits))
    return out


class GroupBy:
    """One GROUP BY handle (gb_agg) — the Python mirror of the operator.

    ``aggs``: list of (kind, col) with kind a name ('count_star', 'count',
    'sum', 'avg', 'min', 'max', 'count_distinct') or the gb_agg_kind code;
    col = -1 for COUNT(*).  ``filters``: list of (col, op, const) with op one of
    '==', '!=', '<', '<=', '>', '>='.
    """

    def __init__(self, col_types, group_cols, aggs, filters=(), nullable=(), est_groups=0, options=None):
        self.lib = load()
        self.col_types = list(col_types)
        self.group_cols = list(group_cols)
        spec, self._spec_keep = _make_spec(col_types, group_cols, aggs, filters, nullable, est_groups)
        h = C.c_void_p()
        check(self.lib.gb_agg_create(C.byref(spec), C.byref(h)))
        self.h = h
        self._keep = []
        for k, v in (options or {}).items():
            self.set_option(k, v)

    def set_topn(self, col_idx, ascending, limit):
        check(self.lib.gb_agg_set_topn(self.h, col_idx, 1 if ascending else 0, limit))

    def set_row_limit(self, limit):
        check(self.lib.gb_agg_set_row_limit(self.h, limit))

    def ingest(self, cols, nrows=None, validity=None, device=False, stream=None):
        """cols: numpy arrays (host) or torch CUDA tensors / int device
        pointers (device=True), one per input column."""
        n = len(self.col_types)
        arr = (Col * n)()
        keep = []
        for i, a in enumerate(cols):
            offs = None
            if self.col_types[i] == VARCHAR:
                # (offsets int64[n+1], bytes uint8) — numpy arrays or device tensors
                offs, a = a
                if not device:
                    offs = np.ascontiguousarray(offs, dtype=np.int64)
                    a = np.ascontiguousarray(a, dtype=np.uint8)
                    if len(a) == 0:
                        a = np.zeros(1, dtype=np.uint8)
                    keep += [offs, a]
            elif not device and isinstance(a, np.ndarray):
                a = np.ascontiguousarray(a, dtype=NP_TYPES[self.col_types[i]])
                keep.append(a)
            v = validity[i] if validity is not None else None
            if v is not None and not device and isinstance(v, np.ndarray):
                v = np.ascontiguousarray(v, dtype=np.uint64)
                keep.append(v)
            arr[i] = Col(_arr_ptr(a), _arr_ptr(v), _arr_ptr(offs))
        if nrows is None:
            c0 = cols[0]
            nrows = len(c0[0]) - 1 if self.col_types[0] == VARCHAR else len(c0)
        check(self.lib.gb_agg_ingest(self.h, arr, int(nrows), MEM_DEVICE if device else MEM_HOST,
                                     C.c_void_p(stream) if stream else None))

    def finalize(self, stream=None):
        check(self.lib.gb_agg_finalize(self.h, C.c_void_p(stream) if stream else None))

    def result(self):
        """Host copy of the result: list of (values ndarray, valid bool ndarray)."""
        r = Result()
        check(self.lib.gb_agg_result(self.h, C.byref(r)))
        return _read_result(r)

    def result_host_bytes(self):
        """gb_agg_result only (the library's device→host copy into its own
        pinned buffers, no Python conversion); returns (rows, bytes copied)."""
        r = Result()
        check(self.lib.gb_agg_result(self.h, C.byref(r)))
        return _result_bytes(r)

    def set_option(self, name, value):
        check(self.lib.gb_agg_set_option(self.h, name.encode(), int(value)))

    def set_filters(self, filters):
        """Replace the WHERE predicates (after create or reset)."""
        fl, _keep = _filters(filters, self.col_types)
        check(self.lib.gb_agg_set_filters(self.h, fl, len(filters)))

    def mode(self):
        return int(self.lib.gb_agg_get_mode(self.h))

    def set_profiling(self, on=True):
        check(self.lib.gb_agg_set_profiling(self.h, 1 if on else 0))

    def profile(self):
        """{kernel name: (launches, total ms)} measured with CUDA events."""
        arr = (KernelStat * 32)()
        n = self.lib.gb_agg_profile(self.h, arr, 32)
        return {arr[i].name.decode(): (int(arr[i].launches), float(arr[i].ms)) for i in range(min(n, 32))}

    def launches(self):
        return int(self.lib.gb_agg_kernel_launches(self.h))

    def row_groups_pruned(self):
        return int(self.lib.gb_agg_row_groups_pruned(self.h))

    def reset(self):
        check(self.lib.gb_agg_reset(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.gb_agg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Batch:
    """Many GROUP BY queries over device-resident tables run together
    (gb_batch): ``add`` takes a query's spec and its device columns (torch
    CUDA tensors or int device pointers; VARCHAR as (offsets, bytes)),
    ``run`` executes all of them, ``result(i)`` reads query i's result."""

    def __init__(self, options=None):
        self.lib = load()
        h = C.c_void_p()
        check(self.lib.gb_batch_create(C.byref(h)))
        self.h = h
        self._keep = []
        for k, v in (options or {}).items():
            self.set_option(k, v)

    def add(self, col_types, group_cols, aggs, cols, nrows, validity=None, filters=(), nullable=(), est_groups=0):
        spec, keep = _make_spec(col_types, group_cols, aggs, filters, nullable, est_groups)
        arr = (Col * len(col_types))()
        for i, a in enumerate(cols):
            offs = None
            if col_types[i] == VARCHAR:
                offs, a = a
            v = validity[i] if validity is not None else None
            arr[i] = Col(_arr_ptr(a), _arr_ptr(v), _arr_ptr(offs))
        q = C.c_uint32()
        check(self.lib.gb_batch_add(self.h, C.byref(spec), arr, int(nrows), C.byref(q)))
        self._keep.append((keep, cols, validity))
        return int(q.value)

    def set_option(self, name, value):
        check(self.lib.gb_batch_set_option(self.h, name.encode(), int(value)))

    def run(self, stream=None):
        check(self.lib.gb_batch_run(self.h, C.c_void_p(stream) if stream else None))

    def clear(self):
        check(self.lib.gb_batch_clear(self.h))
        self._keep = []

    def __len__(self):
        return int(self.lib.gb_batch_size(self.h))

    def result(self, q):
        r = Result()
        check(self.lib.gb_batch_result(self.h, int(q), C.byref(r)))
        return _read_result(r)

    def result_host_bytes(self, q):
        """gb_batch_result only (device→host copy of query q's result into
        the library's pinned buffers); returns (rows, bytes copied)."""
        r = Result()
        check(self.lib.gb_batch_result(self.h, int(q), C.byref(r)))
        return _result_bytes(r)

    def slow_queries(self):
        return int(self.lib.gb_batch_slow_queries(self.h))

    def launches(self):
        return int(self.lib.gb_batch_kernel_launches(self.h))

    def profile(self):
        """{kernel name: (launches, total ms)} of the profiled runs."""
        arr = (KernelStat * 8)()
        n = self.lib.gb_batch_profile(self.h, arr, 8)
        return {arr[i].name.decode(): (int(arr[i].launches), float(arr[i].ms)) for i in range(min(n, 8))}

    def close(self):
        if getattr(self, "h", None):
            self.lib.gb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def estimate_bytes(col_types, group_cols, aggs, nrows, filters=(), nullable=(), est_groups=0):
    """Device bytes a GROUP BY of nrows rows is expected to hold."""
    spec, keep = _make_spec(col_types, group_cols, aggs, filters, nullable, est_groups)
    out = C.c_uint64()
    check(load().gb_agg_estimate_bytes(C.byref(spec), int(nrows), C.byref(out)))
    return int(out.value)


class Server:
    """A served query stream over HBM-resident tables (gb_server).  mode 0 =
    continuous batching, 1 = one query at a time."""

    def __init__(self, budget_bytes, max_batch=256, mode=0, lanes=None):
        self.lib = load()
        h = C.c_void_p()
        check(self.lib.gb_server_create(int(budget_bytes), int(max_batch), int(mode), C.byref(h)))
        self.h = h
        self._keep = []
        self.tables = []
        if lanes is not None:
            check(self.lib.gb_server_set_lanes(self.h, int(lanes)))

    def add_table(self, col_types, cols, nrows, validity=None):
        """cols: torch CUDA tensors / device pointers (VARCHAR: (offsets, bytes))."""
        arr = (Col * len(col_types))()
        for i, a in enumerate(cols):
            offs = None
            if col_types[i] == VARCHAR:
                offs, a = a
            v = validity[i] if validity is not None else None
            arr[i] = Col(_arr_ptr(a), _arr_ptr(v), _arr_ptr(offs))
        ct = (C.c_int32 * len(col_types))(*col_types)
        tid = C.c_uint32()
        check(self.lib.gb_server_add_table(self.h, ct, len(col_types), arr, int(nrows), C.byref(tid)))
        self._keep.append((cols, validity))
        self.tables.append(list(col_types))
        return int(tid.value)

    def submit(self, table, row_begin, row_end, group_cols, aggs, filters=(), nullable=(), est_groups=0):
        spec, keep = _make_spec(self.tables[table], group_cols, aggs, filters, nullable, est_groups)
        t = C.c_uint64()
        check(self.lib.gb_server_submit(self.h, int(table), int(row_begin), int(row_end), C.byref(spec),
                                        C.byref(t)))
        return int(t.value)

    def wait(self, ticket, timeout_us=-1):
        """True when done (raises on a failed query), False on timeout."""
        st = self.lib.gb_server_wait(self.h, int(ticket), int(timeout_us))
        if st == GB_ERR_TIMEOUT:
            return False
        check(st)
        return True

    def result(self, ticket):
        r = Result()
        check(self.lib.gb_server_result(self.h, int(ticket), C.byref(r)))
        return _read_result(r)

    def times(self, ticket):
        qm, em, bs = C.c_double(), C.c_double(), C.c_uint32()
        check(self.lib.gb_server_query_times(self.h, int(ticket), C.byref(qm), C.byref(em), C.byref(bs)))
        return float(qm.value), float(em.value), int(bs.value)

    def release(self, ticket):
        check(self.lib.gb_server_release(self.h, int(ticket)))

    def stats(self):
        st = ServerStat()
        check(self.lib.gb_server_stats(self.h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in ServerStat._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.lib.gb_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def validity_words(valid_bool: np.ndarray) -> np.ndarray:
    """bool[n] → ValidityMask words (uint64, bit i%64 of word i/64)."""
    n = len(valid_bool)
    pad = np.zeros(((n + 63) // 64) * 64, dtype=bool)
    pad[:n] = valid_bool
    return np.packbits(pad, bitorder="little").view(np.uint64).copy()


class ParquetFile:
    """A Parquet file in host memory, parsed by the library (gb_pq_open)."""

    def __init__(self, data):
        self.lib = load()
        if isinstance(data, (bytes, bytearray)):
            self._buf = np.frombuffer(data, dtype=np.uint8)
        else:
            self._buf = np.ascontiguousarray(data, dtype=np.uint8)
        h = C.c_void_p()
        check(self.lib.gb_pq_open(self._buf.ctypes.data, len(self._buf), C.byref(h)))
        self.h = h

    @property
    def num_row_groups(self):
        return int(self.lib.gb_pq_num_row_groups(self.h))

    @property
    def num_rows(self):
        return int(self.lib.gb_pq_num_rows(self.h))

    def dict_sum(self, col, rg_begin=0, rg_end=None, device=False, stream=None):
        """(count, sum) of INT64 file column `col` through the dictionary
        histogram (gb_pq_dict_sum); raises GbError(GB_ERR_UNSUPPORTED) where
        the reference would take the fused path."""
        rg_end = self.num_row_groups if rg_end is None else rg_end
        n, sm = C.c_int64(), C.c_double()
        check(self.lib.gb_pq_dict_sum(self.h, int(col), int(rg_begin), int(rg_end), MEM_DEVICE if device else MEM_HOST,
                                      C.c_void_p(stream) if stream else None, C.byref(n), C.byref(sm)))
        return int(n.value), float(sm.value)

    def row_group_might_match(self, rg, col_map, filters):
        """Zone map of row group `rg`: False when its column statistics rule
        out the (col, op, const) filters (col = spec column, read from file
        column col_map[col])."""
        types = [t for _, t in self.columns()]
        fl, _keep = _filters(filters, [types[c] for c in col_map])
        cm = (C.c_int32 * len(col_map))(*col_map)
        m = C.c_int32()
        check(self.lib.gb_pq_row_group_might_match(self.h, int(rg), cm, len(col_map), C.cast(fl, C.c_void_p),
                                                   len(filters), C.byref(m)))
        return bool(m.value)

    def columns(self):
        out = []
        for i in range(int(self.lib.gb_pq_num_columns(self.h))):
            name = C.create_string_buffer(256)
            t = C.c_int32()
            check(self.lib.gb_pq_column_info(self.h, i, name, 256, C.byref(t)))
            out.append((name.value.decode(), int(t.value)))
        return out

    def upload(self, stream=None):
        check(self.lib.gb_pq_upload(self.h, C.c_void_p(stream) if stream else None))

    def close(self):
        if getattr(self, "h", None):
            self.lib.gb_pq_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ingest_parquet(g, pf, col_map, rg_begin=0, rg_end=None, device=False, stream=None):
    """Feed row groups of ParquetFile `pf` to GroupBy `g` (spec column c reads
    file column col_map[c])."""
    rg_end = pf.num_row_groups if rg_end is None else rg_end
    cm = (C.c_int32 * len(col_map))(*col_map)
    check(g.lib.gb_agg_ingest_parquet(g.h, pf.h, rg_begin, rg_end, cm, MEM_DEVICE if device else MEM_HOST,
                                      C.c_void_p(stream) if stream else None))


class PinnedBuffer:
    """Page-locked host buffer from gb_host_alloc, viewable as numpy."""

    def __init__(self, nbytes):
        self.lib = load()
        p = C.c_void_p()
        check(self.lib.gb_host_alloc(C.byref(p), int(nbytes)))
        self.ptr = p.value
        self.nbytes = int(nbytes)

    def view(self, dtype, count=None):
        dt = np.dtype(dtype)
        if count is None:
            count = self.nbytes // dt.itemsize
        buf = (C.c_char * (count * dt.itemsize)).from_address(self.ptr)
        return np.frombuffer(buf, dtype=dt)

    def close(self):
        if self.ptr:
            self.lib.gb_host_free(C.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
