"""A small Parquet writer for the test and benchmark inputs of the GROUP BY path.

Writes uncompressed files with DATA_PAGE (v1) pages, REQUIRED columns, and
per column either PLAIN values or a PLAIN dictionary page plus
RLE_DICTIONARY-encoded indices (RLE / bit-packed hybrid, fixed bit width).
BYTE_ARRAY (VARCHAR) columns are written dictionary-encoded, each value of
the dictionary page a 4-byte little-endian length followed by its bytes.
The thrift compact protocol encoder is the project's own; the RLE/bit-packed
hybrid encoder is ``pq_encode.c``.  Files written here are readable by any
Parquet reader (checked against pyarrow in the CPU tests where available).
"""
from __future__ import annotations

import ctypes as C
import os
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_ENC_LIB = os.path.join(HERE, "_build", "libpqenc.so")

# parquet.thrift enum values
T_INT32, T_INT64, T_DOUBLE, T_BYTE_ARRAY = 1, 2, 5, 6
ENC_PLAIN, ENC_RLE, ENC_BIT_PACKED, ENC_RLE_DICTIONARY = 0, 3, 4, 8
PAGE_DATA, PAGE_DICT = 0, 2
REQUIRED = 0
CONV_INT_16 = 16

# thrift compact types
CT_TRUE, CT_FALSE, CT_BYTE, CT_I16, CT_I32, CT_I64, CT_DOUBLE, CT_BINARY, CT_LIST, CT_SET, CT_MAP, CT_STRUCT = \
    1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12

_enc = None


def _encoder():
    global _enc
    if _enc is not None:
        return _enc
    src = os.path.join(HERE, "pq_encode.c")
    if not os.path.exists(_ENC_LIB) or os.path.getmtime(_ENC_LIB) < os.path.getmtime(src):
        os.makedirs(os.path.dirname(_ENC_LIB), exist_ok=True)
        tmp = _ENC_LIB + ".tmp"
        subprocess.run([os.environ.get("CC", "gcc"), "-O2", "-fPIC", "-shared", "-o", tmp, src], check=True)
        os.replace(tmp, _ENC_LIB)
    lib = C.CDLL(_ENC_LIB)
    lib.pq_rle_encode.restype = C.c_int64
    lib.pq_rle_encode.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p]
    lib.pq_snappy_compress.restype = C.c_int64
    lib.pq_snappy_compress.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p]
    lib.pq_zstd_compress.restype = C.c_int64
    lib.pq_zstd_compress.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p]
    _enc = lib
    return lib


def snappy_compress(data: bytes) -> bytes:
    """One raw Snappy block of `data` (the writer's SNAPPY pages)."""
    src = np.frombuffer(data, dtype=np.uint8) if data else np.zeros(1, np.uint8)
    cap = len(data) + len(data) // 6 + 64
    out = np.empty(cap, dtype=np.uint8)
    table = np.empty(1 << 14, dtype=np.int32)
    got = _encoder().pq_snappy_compress(src.ctypes.data, len(data), out.ctypes.data, cap, table.ctypes.data)
    if got < 0:
        raise RuntimeError("Snappy compress buffer overflow")
    return out[:got].tobytes()


def zstd_compress(data: bytes) -> bytes:
    """One ZSTD frame of `data` (the writer's ZSTD pages: greedy matches, raw
    literals, sequences coded with the format's predefined tables)."""
    src = np.frombuffer(data, dtype=np.uint8) if data else np.zeros(1, np.uint8)
    cap = len(data) + len(data) // 128 + 64
    out = np.empty(cap, dtype=np.uint8)
    table = np.empty(1 << 16, dtype=np.int32)
    got = _encoder().pq_zstd_compress(src.ctypes.data, len(data), out.ctypes.data, cap, table.ctypes.data)
    if got < 0:
        raise RuntimeError("ZSTD compress buffer overflow")
    return out[:got].tobytes()


def rle_hybrid(indices: np.ndarray, bit_width: int) -> bytes:
    """RLE / bit-packed hybrid encoding of `indices` (no bit-width byte)."""
    x = np.ascontiguousarray(indices, dtype=np.uint32)
    n = len(x)
    cap = n * 5 + 1024
    out = np.empty(cap, dtype=np.uint8)
    scratch = np.empty(n + 16, dtype=np.uint32)
    got = _encoder().pq_rle_encode(x.ctypes.data, n, bit_width, out.ctypes.data, cap, scratch.ctypes.data)
    if got < 0:
        raise RuntimeError("RLE encode buffer overflow")
    return out[:got].tobytes()


class TWriter:
    """Thrift compact protocol encoder (structs, lists, ints, binary, bool)."""

    def __init__(self):
        self.buf = bytearray()
        self.last = [0]

    def _varint(self, v):
        while v >= 0x80:
            self.buf.append((v & 0x7F) | 0x80)
            v >>= 7
        self.buf.append(v)

    @staticmethod
    def _zz(v):
        return (v << 1) ^ (v >> 63)

    def _field(self, fid, ctype):
        delta = fid - self.last[-1]
        if 0 < delta <= 15:
            self.buf.append((delta << 4) | ctype)
        else:
            self.buf.append(ctype)
            self._varint(self._zz(fid) & 0xFFFF)
        self.last[-1] = fid

    def i32(self, fid, v):
        self._field(fid, CT_I32)
        self._varint(self._zz(v) & 0xFFFFFFFFFFFFFFFF)

    def i64(self, fid, v):
        self._field(fid, CT_I64)
        self._varint(self._zz(v) & 0xFFFFFFFFFFFFFFFF)

    def i8(self, fid, v):
        self._field(fid, CT_BYTE)
        self.buf.append(v & 0xFF)

    def boolean(self, fid, v):
        self._field(fid, CT_TRUE if v else CT_FALSE)

    def binary(self, fid, b):
        if isinstance(b, str):
            b = b.encode()
        self._field(fid, CT_BINARY)
        self._varint(len(b))
        self.buf += b

    def begin_struct(self, fid):
        self._field(fid, CT_STRUCT)
        self.last.append(0)

    def end_struct(self):
        self.buf.append(0)
        self.last.pop()

    def begin_list(self, fid, elem_type, n):
        self._field(fid, CT_LIST)
        if n < 15:
            self.buf.append((n << 4) | elem_type)
        else:
            self.buf.append(0xF0 | elem_type)
            self._varint(n)

    def list_struct_begin(self):
        self.last.append(0)

    def list_struct_end(self):
        self.buf.append(0)
        self.last.pop()

    def list_i32(self, v):
        self._varint(self._zz(v) & 0xFFFFFFFFFFFFFFFF)

    def list_binary(self, b):
        if isinstance(b, str):
            b = b.encode()
        self._varint(len(b))
        self.buf += b

    def stop(self):
        self.buf.append(0)


CODEC_UNCOMPRESSED, CODEC_SNAPPY, CODEC_ZSTD = 0, 1, 6


def _page_header(ptype, size, num_values=None, encoding=None, dict_values=None, compressed_size=None):
    w = TWriter()
    w.i32(1, ptype)
    w.i32(2, size)
    w.i32(3, size if compressed_size is None else compressed_size)
    if ptype == PAGE_DATA:
        w.begin_struct(5)
        w.i32(1, num_values)
        w.i32(2, encoding)
        w.i32(3, ENC_RLE)
        w.i32(4, ENC_RLE)
        w.end_struct()
    else:
        w.begin_struct(7)
        w.i32(1, dict_values)
        w.i32(2, ENC_PLAIN)
        w.end_struct()
    w.stop()
    return bytes(w.buf)


class Column:
    """One REQUIRED column.  values: numpy array of the physical type, or for
    dictionary encoding `dictionary` (values; a list of bytes for BYTE_ARRAY)
    + `indices` (uint32).  shuffle_seed: each row group writes the dictionary
    in its own order (a permutation drawn from the seed and the row-group
    index) with the indices remapped, so the decoded values stay the same."""

    def __init__(self, name, ptype, values=None, dictionary=None, indices=None, int16=False, page_rows=None,
                 shuffle_seed=None):
        self.name = name
        self.page_rows = page_rows  # overrides the file-wide page size
        self.ptype = ptype
        self.values = values
        self.dictionary = dictionary
        self.indices = indices
        self.int16 = int16
        self.shuffle_seed = shuffle_seed

    @property
    def dict_encoded(self):
        return self.dictionary is not None

    def n(self):
        return len(self.indices) if self.dict_encoded else len(self.values)


def _np_dtype(ptype):
    return {T_INT32: "<i4", T_INT64: "<i8", T_DOUBLE: "<f8"}[ptype]


def _dict_payload(ptype, dictionary):
    if ptype == T_BYTE_ARRAY:
        return b"".join(struct.pack("<I", len(x)) + bytes(x) for x in dictionary)
    return np.ascontiguousarray(dictionary, dtype=_np_dtype(ptype)).tobytes()


def _stat_bytes(c, lo, hi):
    """min_value / max_value bytes of rows [lo, hi) of a numeric column (PLAIN
    encoding of the value), or None."""
    if c.ptype not in (T_INT32, T_INT64, T_DOUBLE) or hi <= lo:
        return None
    vals = np.asarray(c.dictionary)[c.indices[lo:hi]] if c.dict_encoded else np.asarray(c.values[lo:hi])
    vals = vals.astype(_np_dtype(c.ptype))
    return vals.min().tobytes(), vals.max().tobytes()


def write(columns, row_group_rows=1_000_000, page_rows=65_536, created_by="slothdb_gb300 writer", codec=None,
          stats=False):
    """Return the bytes of a Parquet file holding `columns` (equal lengths);
    codec "snappy" compresses every page (dictionary and data) as one raw
    Snappy block, codec "zstd" as one ZSTD frame; stats writes each numeric
    column chunk's min / max (Statistics min_value / max_value)."""
    assert codec in (None, "snappy", "zstd")

    def page(ptype, payload, **kw):
        if codec is None:
            return _page_header(ptype, len(payload), **kw), payload, len(payload)
        body = snappy_compress(payload) if codec == "snappy" else zstd_compress(payload)
        return _page_header(ptype, len(payload), compressed_size=len(body), **kw), body, len(payload)
    n = columns[0].n()
    for c in columns:
        assert c.n() == n
    parts = [b"PAR1"]
    pos = 4
    row_groups = []
    for rg0 in range(0, n, row_group_rows):
        rg1 = min(n, rg0 + row_group_rows)
        chunks = []
        rg_bytes = 0
        for c in columns:
            start = pos
            dict_off = None
            rg_dict, rg_idx = c.dictionary, c.indices
            if c.dict_encoded and c.shuffle_seed is not None:
                perm = np.random.default_rng([c.shuffle_seed, rg0]).permutation(len(c.dictionary))
                inv = np.empty_like(perm)
                inv[perm] = np.arange(len(perm))
                rg_dict = [c.dictionary[i] for i in perm] if c.ptype == T_BYTE_ARRAY else np.asarray(c.dictionary)[perm]
                rg_idx = np.zeros(len(c.indices), dtype=np.uint32)
                rg_idx[rg0:rg1] = inv[c.indices[rg0:rg1]]
            unc = 0
            if c.dict_encoded:
                hdr, body, raw = page(PAGE_DICT, _dict_payload(c.ptype, rg_dict), dict_values=len(rg_dict))
                dict_off = pos
                parts += [hdr, body]
                pos += len(hdr) + len(body)
                unc += len(hdr) + raw
                bw = max(1, int(len(c.dictionary) - 1).bit_length())
            data_off = pos
            prows = c.page_rows or page_rows
            for p0 in range(rg0, rg1, prows):
                p1 = min(rg1, p0 + prows)
                if c.dict_encoded:
                    payload = bytes([bw]) + rle_hybrid(rg_idx[p0:p1], bw)
                    enc = ENC_RLE_DICTIONARY
                else:
                    payload = np.ascontiguousarray(c.values[p0:p1], dtype=_np_dtype(c.ptype)).tobytes()
                    enc = ENC_PLAIN
                hdr, body, raw = page(PAGE_DATA, payload, num_values=p1 - p0, encoding=enc)
                parts += [hdr, body]
                pos += len(hdr) + len(body)
                unc += len(hdr) + raw
            size = pos - start
            rg_bytes += size
            chunks.append((c, start, dict_off, data_off, size, rg1 - rg0, unc,
                           _stat_bytes(c, rg0, rg1) if stats else None))
        row_groups.append((chunks, rg_bytes, rg1 - rg0))
    # footer
    w = TWriter()
    w.i32(1, 1)
    w.begin_list(2, CT_STRUCT, 1 + len(columns))
    w.list_struct_begin()
    w.binary(4, "schema")
    w.i32(5, len(columns))
    w.list_struct_end()
    for c in columns:
        w.list_struct_begin()
        w.i32(1, c.ptype)
        w.i32(3, REQUIRED)
        w.binary(4, c.name)
        if c.int16:
            w.i32(6, CONV_INT_16)
            w.begin_struct(10)       # LogicalType union
            w.begin_struct(10)       # INTEGER
            w.i8(1, 16)
            w.boolean(2, True)
            w.end_struct()
            w.end_struct()
        w.list_struct_end()
    w.i64(3, n)
    w.begin_list(4, CT_STRUCT, len(row_groups))
    for chunks, rg_bytes, rg_rows in row_groups:
        w.list_struct_begin()
        w.begin_list(1, CT_STRUCT, len(chunks))
        for c, start, dict_off, data_off, size, rows, unc, st in chunks:
            w.list_struct_begin()
            w.i64(2, start)
            w.begin_struct(3)
            w.i32(1, c.ptype)
            encs = [ENC_PLAIN, ENC_RLE] + ([ENC_RLE_DICTIONARY] if c.dict_encoded else [])
            w.begin_list(2, CT_I32, len(encs))
            for e in encs:
                w.list_i32(e)
            w.begin_list(3, CT_BINARY, 1)
            w.list_binary(c.name)
            w.i32(4, {None: CODEC_UNCOMPRESSED, "snappy": CODEC_SNAPPY, "zstd": CODEC_ZSTD}[codec])
            w.i64(5, rows)
            w.i64(6, unc)
            w.i64(7, size)
            w.i64(9, data_off)
            if dict_off is not None:
                w.i64(11, dict_off)
            if st is not None:
                w.begin_struct(12)  # Statistics
                w.binary(5, st[1])  # max_value
                w.binary(6, st[0])  # min_value
                w.end_struct()
            w.end_struct()
            w.list_struct_end()
        w.i64(2, rg_bytes)
        w.i64(3, rg_rows)
        w.list_struct_end()
    w.binary(6, created_by)
    if stats:
        # column_orders: TYPE_ORDER for every column, which makes readers
        # trust min_value / max_value
        w.begin_list(7, CT_STRUCT, len(columns))
        for _ in columns:
            w.list_struct_begin()
            w.begin_struct(1)
            w.end_struct()
            w.list_struct_end()
    w.stop()
    footer = bytes(w.buf)
    parts += [footer, struct.pack("<I", len(footer)), b"PAR1"]
    return b"".join(parts)


def filter_groupby_file(n_rows=200_000_000, seed=2, n_dict=65_536, row_group_rows=1_000_000, page_rows=65_536,
                        codec=None):
    """The fused decode + filter + aggregate workload's file: key INT32
    dictionary-encoded (n_dict entries uniform in [0, 2^31), RLE/bit-packed
    indices at bit width 16, run lengths geometric with mean 4, run value
    uniform), f INT16 (stored INT32, INT(16) annotation) uniform [0, 1000)
    PLAIN, v INT64 uniform [-10^9, 10^9] PLAIN.  Draw order: dictionary, run
    lengths, run values, f, v.  Returns (file bytes, key values, f, v)."""
    rng = np.random.default_rng(seed)
    dictionary = rng.integers(0, 2**31, n_dict, dtype=np.int64).astype(np.int32)
    m = n_rows // 4 + 1024
    lens = rng.geometric(0.25, m)
    while lens.sum() < n_rows:
        lens = np.concatenate([lens, rng.geometric(0.25, m)])
    vals = rng.integers(0, n_dict, len(lens), dtype=np.int64)
    idx = np.repeat(vals.astype(np.uint32), lens)[:n_rows]
    f = rng.integers(0, 1000, n_rows, dtype=np.int32)
    v = rng.integers(-10**9, 10**9 + 1, n_rows, dtype=np.int64)
    cols = [Column("key", T_INT32, dictionary=dictionary, indices=idx),
            Column("f", T_INT32, values=f, int16=True),
            Column("v", T_INT64, values=v)]
    data = write(cols, row_group_rows=row_group_rows, page_rows=page_rows, codec=codec)
    return data, dictionary[idx], f, v


def dict_int64_file(n_rows=200_000_000, seed=7, n_dict=65_536, row_group_rows=1_000_000, page_rows=65_536):
    """One INT64 column, dictionary-encoded: n_dict entries uniform in
    [-10^9, 10^9], indices in runs of geometric length (mean 4), run value
    uniform (the shape of the fused workload's key, as an INT64 measure for
    the ungrouped dictionary histogram).  Returns (file bytes, dictionary,
    indices)."""
    rng = np.random.default_rng(seed)
    dictionary = rng.integers(-10**9, 10**9 + 1, n_dict, dtype=np.int64)
    m = n_rows // 4 + 1024
    lens = rng.geometric(0.25, m)
    while lens.sum() < n_rows:
        lens = np.concatenate([lens, rng.geometric(0.25, m)])
    vals = rng.integers(0, n_dict, len(lens), dtype=np.int64)
    idx = np.repeat(vals.astype(np.uint32), lens)[:n_rows]
    data = write([Column("c", T_INT64, dictionary=dictionary, indices=idx)], row_group_rows=row_group_rows,
                 page_rows=page_rows)
    return data, dictionary, idx


def varchar_groupby_file(n_rows=200_000, seed=6, n_dict=3000, row_group_rows=50_000, page_rows=8192):
    """A file whose group key is VARCHAR, dictionary-encoded: n_dict strings
    of 8..32 characters over [a-z0-9] (each row group writes them in its own
    order), indices in runs of geometric length (mean 4); f INT16 (stored
    INT32) uniform [0, 1000) PLAIN; v INT64 uniform [-10^6, 10^6] PLAIN.
    Returns (file bytes, dictionary (list of bytes), indices, f, v)."""
    rng = np.random.default_rng(seed)
    alphabet = np.frombuffer(b"abcdefghijklmnopqrstuvwxyz0123456789", dtype=np.uint8)
    lens = rng.integers(8, 33, n_dict)
    dictionary = [alphabet[rng.integers(0, 36, n)].tobytes() for n in lens]
    runs = rng.geometric(0.25, n_rows // 4 + 64)
    while runs.sum() < n_rows:
        runs = np.concatenate([runs, rng.geometric(0.25, n_rows // 4 + 64)])
    vals = rng.integers(0, n_dict, len(runs), dtype=np.int64)
    idx = np.repeat(vals.astype(np.uint32), runs)[:n_rows]
    f = rng.integers(0, 1000, n_rows, dtype=np.int32)
    v = rng.integers(-10**6, 10**6 + 1, n_rows, dtype=np.int64)
    cols = [Column("name", T_BYTE_ARRAY, dictionary=dictionary, indices=idx, shuffle_seed=seed),
            Column("f", T_INT32, values=f, int16=True),
            Column("v", T_INT64, values=v)]
    data = write(cols, row_group_rows=row_group_rows, page_rows=page_rows)
    return data, dictionary, idx, f, v


def strings_of(dictionary, idx):
    """VARCHAR column (offsets int64[n + 1], bytes uint8) of dictionary[idx]."""
    lens = np.array([len(x) for x in dictionary], dtype=np.int64)
    offs = np.zeros(len(idx) + 1, dtype=np.int64)
    np.cumsum(lens[idx], out=offs[1:])
    blob = b"".join(dictionary[i] for i in idx.tolist())
    return offs, np.frombuffer(blob, dtype=np.uint8) if blob else np.zeros(1, np.uint8)
