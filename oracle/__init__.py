"""CPU oracle for the GB300 GROUP BY path — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this package, and only as the checker / the timed CPU restatement of the
reference.  The product library never imports it.

``run_query`` evaluates a GROUP BY with the reference's semantics through
the C restatement in ``gb_oracle.c`` (AggState with double accumulators,
typed MIN/MAX, SUM → (int64)double for BIGINT results, AVG = sum/count,
empty SUM → NULL), and returns the groups with, for DOUBLE SUM/AVG, a
Neumaier-compensated FP64 value per group for tolerance checks.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

SMALLINT, INTEGER, BIGINT, DOUBLE, VARCHAR = 1, 2, 3, 4, 5
COUNT_STAR, COUNT, SUM, AVG, MIN, MAX, COUNT_DISTINCT = 0, 1, 2, 3, 4, 5, 6
NP_TYPES = {SMALLINT: np.int16, INTEGER: np.int32, BIGINT: np.int64, DOUBLE: np.float64}
AGG_NAMES = {"count_star": COUNT_STAR, "count": COUNT, "sum": SUM, "avg": AVG, "min": MIN, "max": MAX,
             "count_distinct": COUNT_DISTINCT}
CMP_NAMES = {"==": 0, "=": 0, "!=": 1, "<>": 1, "<": 2, "<=": 3, ">": 4, ">=": 5, "in": 6, "like": 9,
             "not like": 10}

_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        import sys
        sys.path.insert(0, os.path.dirname(HERE))
        from slothdb_gb300 import build
        build.build_oracle()
    lib = C.CDLL(LIB_PATH)
    P = C.c_void_p
    lib.or_groupby.restype = C.c_int64
    lib.or_groupby.argtypes = [C.c_int64, P, P, P, C.c_int32, P, P, P, P, C.c_int32, C.c_int64, C.c_int64,
                               P, P, P, P, P, P]
    lib.or_groupby_str.restype = C.c_int64
    lib.or_groupby_str.argtypes = [C.c_int64, P, P, P, P, C.c_int32, P, P, P, P, C.c_int64, P, P, P, P, P, P]
    lib.or_filter.restype = None
    lib.or_filter.argtypes = [C.c_int64, C.c_int32, P, P, C.c_int32, C.c_int64, C.c_double, P]
    lib.or_rle_decode.restype = C.c_int64
    lib.or_rle_decode.argtypes = [P, C.c_int64, C.c_int32, P, C.c_int64]
    lib.or_filter_in.restype = None
    lib.or_filter_in.argtypes = [C.c_int64, C.c_int32, P, P, P, C.c_int64, P]
    lib.or_filter_str.restype = None
    lib.or_filter_str.argtypes = [C.c_int64, P, P, P, C.c_int32, P, C.c_int64, P]
    lib.or_snappy_decompress.restype = C.c_int64
    lib.or_snappy_decompress.argtypes = [P, C.c_int64, P, C.c_int64]
    _lib = lib
    return lib


def _p(a):
    return None if a is None else a.ctypes.data


def agg_out_type(kind, in_type):
    """Binder return type (src/binder/binder.cpp:1345-1391)."""
    if kind in (COUNT_STAR, COUNT, COUNT_DISTINCT):
        return BIGINT
    if kind == SUM:
        return DOUBLE if in_type == DOUBLE else BIGINT
    if kind == AVG:
        return DOUBLE
    return in_type


def filter_mask(n, col_types, cols, filters, nulls=None):
    lib = load()
    keep = np.ones(n, dtype=np.uint8)
    for col, op, const in filters:
        opc = CMP_NAMES[op] if isinstance(op, str) else int(op)
        t = col_types[col]
        nul = None
        if nulls is not None and nulls[col] is not None:
            nul = np.ascontiguousarray(nulls[col], dtype=np.uint8)
        if t == VARCHAR:
            # = / <> / LIKE '%x%' / NOT LIKE on the bytes (const: bytes)
            if opc in (0, 1):
                opc += 7
            offs = np.ascontiguousarray(cols[col][0], dtype=np.int64)
            data = np.ascontiguousarray(cols[col][1], dtype=np.uint8)
            lit = np.frombuffer(bytes(const), dtype=np.uint8) if len(const) else np.zeros(1, np.uint8)
            lib.or_filter_str(n, _p(offs), _p(data), _p(nul), opc, _p(lit), len(const), _p(keep))
            continue
        a = np.ascontiguousarray(cols[col], dtype=NP_TYPES[t])
        if opc == 6:
            members = np.ascontiguousarray(np.asarray(list(const), dtype=np.int64)) if len(const) else np.zeros(1,
                                                                                                          np.int64)
            lib.or_filter_in(n, t, _p(a), _p(nul), _p(members), len(const), _p(keep))
            continue
        if t == DOUBLE:
            lib.or_filter(n, t, _p(a), _p(nul), opc, 0, float(const), _p(keep))
        else:
            lib.or_filter(n, t, _p(a), _p(nul), opc, int(const), 0.0, _p(keep))
    return keep


def run_query(col_types, group_cols, aggs, cols, filters=(), nulls=None, nthreads=1, est_groups=0,
              str_cols=None, max_groups=None):
    """Evaluate SELECT keys, aggs FROM cols [WHERE filters] GROUP BY keys.

    cols: list of numpy arrays (VARCHAR columns: (offsets int64[n+1], bytes uint8)).
    nulls: optional list (per column) of bool arrays, True = NULL.
    max_groups: output capacity in groups (default: one per row); a result
    with more groups is recomputed with the capacity it needs.
    Returns dict(keys=[ndarray...], key_null=[bool ndarray...],
                 aggs=[(values, null bool, comp float64)...], out_types=[...]).
    """
    lib = load()
    n = len(cols[group_cols[0]][0]) - 1 if col_types[group_cols[0]] == VARCHAR else len(cols[group_cols[0]])
    aggs = [(AGG_NAMES[k] if isinstance(k, str) else int(k), int(c)) for k, c in aggs]
    keep = filter_mask(n, col_types, cols, filters, nulls) if filters else None
    na = len(aggs)
    kinds = np.array([k for k, _ in aggs], dtype=np.int32)
    in_types = np.array([col_types[c] if c >= 0 else 0 for _, c in aggs], dtype=np.int32)
    held = []
    data_ptrs = (C.c_void_p * na)()
    null_ptrs = (C.c_void_p * na)()
    for i, (k, c) in enumerate(aggs):
        if c >= 0:
            a = np.ascontiguousarray(cols[c], dtype=NP_TYPES[col_types[c]])
            held.append(a)
            data_ptrs[i] = a.ctypes.data
            if nulls is not None and nulls[c] is not None:
                m = np.ascontiguousarray(nulls[c], dtype=np.uint8)
                held.append(m)
                null_ptrs[i] = m.ctypes.data
    cap = (min(n, int(max_groups)) if max_groups else n) + 2
    out_i = np.zeros(na * cap, dtype=np.int64)
    out_d = np.zeros(na * cap, dtype=np.float64)
    out_null = np.zeros(na * cap, dtype=np.uint8)
    out_comp = np.zeros(na * cap, dtype=np.float64)
    out_key_null = np.zeros(cap, dtype=np.uint8)
    key_types = [col_types[g] for g in group_cols]

    if len(group_cols) == 1 and key_types[0] == VARCHAR:
        offs, data = cols[group_cols[0]]
        offs = np.ascontiguousarray(offs, dtype=np.int64)
        data = np.ascontiguousarray(data, dtype=np.uint8)
        kn = None
        if nulls is not None and nulls[group_cols[0]] is not None:
            kn = np.ascontiguousarray(nulls[group_cols[0]], dtype=np.uint8)
        out_rep = np.zeros(cap, dtype=np.int64)
        ng = lib.or_groupby_str(n, _p(offs), _p(data), _p(kn), _p(keep), na, _p(kinds), _p(in_types), data_ptrs,
                                null_ptrs, cap, _p(out_rep), _p(out_key_null), _p(out_i), _p(out_d),
                                _p(out_null), _p(out_comp))
        if ng < -1:
            return run_query(col_types, group_cols, aggs, cols, filters, nulls, nthreads, est_groups, str_cols,
                             max_groups=-ng - 2)
        if ng < 0:
            raise RuntimeError("oracle failed (%d)" % ng)
        reps = out_rep[:ng]
        strs = np.array([bytes(data[offs[r]:offs[r + 1]]) for r in reps], dtype=object)
        keys = [strs]
        key_null = [out_key_null[:ng].astype(bool)]
    elif (len(group_cols) == 2 and all(t in (SMALLINT, INTEGER) for t in key_types)
          and (nulls is None or all(nulls[g] is None for g in group_cols))):
        # two non-NULL 16/32-bit keys: one int64 key (a << 32 | b as 32 bits),
        # the same groups, through the multithreaded single-key loop
        a = np.asarray(cols[group_cols[0]]).astype(np.int64)
        b = np.asarray(cols[group_cols[1]]).astype(np.int64)
        packed = (a << 32) | (b & 0xFFFFFFFF)
        sub_types = list(col_types) + [BIGINT]
        sub = run_query(sub_types, [len(col_types)], [(k, c) for k, c in aggs], list(cols) + [packed],
                        filters=filters, nulls=(list(nulls) + [None]) if nulls is not None else None,
                        nthreads=nthreads, est_groups=est_groups, max_groups=max_groups)
        pk = sub["keys"][0]
        sub["keys"] = [(pk >> 32).astype(NP_TYPES[key_types[0]]),
                       (pk & 0xFFFFFFFF).astype(np.uint32).astype(np.int32).astype(NP_TYPES[key_types[1]])]
        sub["key_null"] = [np.zeros(len(pk), bool), np.zeros(len(pk), bool)]
        sub["out_types"] = list(key_types) + sub["out_types"][1:]
        return sub
    else:
        # group ids: single int key directly; composite keys via a dense id
        # over the (value, null) tuples (equality of the reference's
        # concatenated group key, physical_planner.cpp:6185-6206)
        kn_list = []
        for g in group_cols:
            if nulls is not None and nulls[g] is not None:
                kn_list.append(np.asarray(nulls[g], dtype=bool))
            else:
                kn_list.append(np.zeros(n, dtype=bool))
        if len(group_cols) == 1:
            packed = np.ascontiguousarray(cols[group_cols[0]], dtype=np.int64)
            kn = kn_list[0]
            packed = np.where(kn, 0, packed).astype(np.int64)
            knull = kn.astype(np.uint8)
            inv = None
        else:
            # a VARCHAR column of a pair key groups by its bytes: dense codes
            # per distinct string (the reference's concatenated group key,
            # physical_planner.cpp:6185-6206, compares the bytes)
            pair = []
            strings = {}
            for j, g in enumerate(group_cols):
                if col_types[g] == VARCHAR:
                    offs, data = cols[g]
                    code_of = {}
                    codes = np.empty(n, dtype=np.int64)
                    for r in range(n):
                        s_ = bytes(data[offs[r]:offs[r + 1]])
                        codes[r] = code_of.setdefault(s_, len(code_of))
                    strings[j] = np.array(list(code_of.keys()) + [b""], dtype=object)
                    pair.append(codes)
                else:
                    pair.append(cols[g])
            rec = np.empty(n, dtype=[("a", np.int64), ("na", np.bool_), ("b", np.int64), ("nb", np.bool_)])
            rec["a"] = np.where(kn_list[0], 0, pair[0])
            rec["na"] = kn_list[0]
            rec["b"] = np.where(kn_list[1], 0, pair[1])
            rec["nb"] = kn_list[1]
            uniq, inv = np.unique(rec, return_inverse=True)
            packed = inv.astype(np.int64).reshape(-1)
            knull = None
        out_keys = np.zeros(cap, dtype=np.int64)
        ng = lib.or_groupby(n, _p(packed), _p(knull), _p(keep), na, _p(kinds), _p(in_types), data_ptrs, null_ptrs,
                            int(nthreads), int(est_groups), cap, _p(out_keys), _p(out_key_null), _p(out_i),
                            _p(out_d), _p(out_null), _p(out_comp))
        if ng < -1:
            return run_query(col_types, group_cols, aggs, cols, filters, nulls, nthreads, est_groups, str_cols,
                             max_groups=-ng - 2)
        if ng < 0:
            raise RuntimeError("oracle failed (%d)" % ng)
        if len(group_cols) == 1:
            keys = [out_keys[:ng].astype(NP_TYPES[key_types[0]])]
            key_null = [out_key_null[:ng].astype(bool)]
        else:
            u = uniq[out_keys[:ng]]
            keys = []
            for j, f in enumerate(("a", "b")):
                if j in strings:
                    keys.append(strings[j][np.where(u["n" + f], len(strings[j]) - 1, u[f])])
                else:
                    keys.append(u[f].astype(NP_TYPES[key_types[j]]))
            key_null = [u["na"].astype(bool), u["nb"].astype(bool)]
    out_aggs = []
    out_types = list(key_types)
    for i, (k, c) in enumerate(aggs):
        ot = agg_out_type(k, in_types[i] if c >= 0 else 0)
        out_types.append(ot)
        sl = slice(i * cap, i * cap + ng)
        if ot == DOUBLE:
            vals = out_d[sl].copy()
        else:
            vals = out_i[sl].astype(NP_TYPES[ot])
        out_aggs.append((vals, out_null[sl].astype(bool), out_comp[sl].copy()))
    return dict(keys=keys, key_null=key_null, aggs=out_aggs, out_types=out_types, n_groups=int(ng))


def rle_decode(buf: bytes, bit_width: int, n: int) -> np.ndarray:
    lib = load()
    a = np.frombuffer(buf, dtype=np.uint8)
    out = np.zeros(max(n, 1), dtype=np.uint32)
    got = lib.or_rle_decode(_p(a), len(a), bit_width, _p(out), n)
    return out[:got]


def snappy_decompress(block: bytes, cap: int = 1 << 30) -> bytes:
    """A raw Snappy block decompressed by the oracle's restatement of the
    format (raises ValueError on a malformed block)."""
    lib = load()
    a = np.frombuffer(block, dtype=np.uint8) if block else np.zeros(1, np.uint8)
    # the preamble bounds the output
    want, sh, i = 0, 0, 0
    while i < len(block) and sh <= 28:
        want |= (block[i] & 0x7F) << sh
        i += 1
        if not block[i - 1] & 0x80:
            break
        sh += 7
    out = np.zeros(max(1, min(want, cap)), dtype=np.uint8)
    got = lib.or_snappy_decompress(_p(a), len(block), _p(out), min(want, cap))
    if got < 0:
        raise ValueError("malformed Snappy block")
    return out[:got].tobytes()
