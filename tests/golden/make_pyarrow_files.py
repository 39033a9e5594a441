"""Parquet files written by pyarrow (an independent writer) for the GPU
decoder's parity tests — regenerated by running this script from the
repository root:  python tests/golden/make_pyarrow_files.py

The GPU machine has no pyarrow, so the files themselves are committed (gzipped)
under tests/golden/; their logical columns are regenerated from the seeds by
`columns()` (numpy only), which the tests call to build the oracle's input.

Cases: OPTIONAL columns with NULLs in the key, the filter column and the
value columns, written as data page v1 and v2, with dictionary encoding on
every column (values falling back to PLAIN pages once the dictionary page
limit is reached), on no column, or on the key only, uncompressed or with
pyarrow's default SNAPPY codec; a dictionary-encoded VARCHAR key with NULL
keys (uncompressed and SNAPPY), also with PLAIN BYTE_ARRAY pages (no
dictionary, or pyarrow's fallback once the dictionary page limit is reached);
OPTIONAL columns without NULLs; an INT64 column whose dictionary falls back
to PLAIN pages.
"""
from __future__ import annotations

import gzip
import io
import os

import numpy as np

OUT = os.path.dirname(os.path.abspath(__file__))
N_ROWS = 24_000

CASES = {
    "pa_nulls_v1_dict": dict(version="1.0", dictionary=True),
    "pa_nulls_v2_dict": dict(version="2.0", dictionary=True),
    "pa_nulls_v1_plain": dict(version="1.0", dictionary=False),
    "pa_nulls_v2_keydict": dict(version="2.0", dictionary=["key"]),
    # pyarrow's default codec: SNAPPY pages (inflated on the GPU)
    "pa_nulls_v1_snappy": dict(version="1.0", dictionary=True, compression="snappy"),
    "pa_nulls_v2_snappy": dict(version="2.0", dictionary=["key"], compression="snappy"),
    # ZSTD pages (decoded on the GPU, one thread per page)
    "pa_nulls_v1_zstd": dict(version="1.0", dictionary=True, compression="zstd"),
    "pa_nulls_v2_zstd": dict(version="2.0", dictionary=["key"], compression="zstd"),
}


def columns(seed=31, n=N_ROWS):
    """key INT32, f INT16, v INT64, x DOUBLE and their NULL masks."""
    rng = np.random.default_rng(seed)
    key = rng.integers(0, 2000, n).astype(np.int32)
    f = rng.integers(0, 1000, n).astype(np.int16)
    v = rng.integers(-10**6, 10**6, n, dtype=np.int64)
    x = np.round(rng.normal(50, 10, n), 3)
    kn, fn, vn, xn = (rng.random(n) < p for p in (0.01, 0.05, 0.10, 0.07))
    vn[key == 7] = True  # a group whose values are all NULL
    return [key, f, v, x], [kn, fn, vn, xn]


def varchar_columns(seed=32, n=N_ROWS):
    """A VARCHAR key of 1500 distinct strings with NULL keys, and v INT64."""
    rng = np.random.default_rng(seed)
    pool = [("k%05d" % i).encode() * (1 + i % 3) for i in range(1500)]
    idx = rng.integers(0, len(pool), n)
    kn = rng.random(n) < 0.02
    v = rng.integers(0, 10**6, n, dtype=np.int64)
    vn = rng.random(n) < 0.1
    strs = [pool[i] for i in idx]
    offs = np.zeros(n + 1, dtype=np.int64)
    np.cumsum([len(s) for s in strs], out=offs[1:])
    blob = np.frombuffer(b"".join(strs), dtype=np.uint8)
    return strs, (offs, blob), v, kn, vn


def int64_column(seed=33, n=N_ROWS):
    """An INT64 column of 20,000 distinct values (its dictionary outgrows a
    16 KB dictionary page, so pyarrow falls back to PLAIN pages)."""
    rng = np.random.default_rng(seed)
    vals = rng.integers(-10**6, 10**6, 20_000, dtype=np.int64)
    return vals[rng.integers(0, len(vals), n)]


def load(name):
    """The committed file's bytes."""
    with gzip.open(os.path.join(OUT, name + ".parquet.gz"), "rb") as fh:
        return fh.read()


def _write(name, table, compression="none", **kw):
    import pyarrow.parquet as pq
    buf = io.BytesIO()
    pq.write_table(table, buf, compression=compression, **kw)
    with gzip.open(os.path.join(OUT, name + ".parquet.gz"), "wb", compresslevel=9) as fh:
        fh.write(buf.getvalue())
    print(name, len(buf.getvalue()), "bytes")


def main():
    import pyarrow as pa
    (key, f, v, x), (kn, fn, vn, xn) = columns()
    tbl = pa.table({"key": pa.array(key, pa.int32(), mask=kn), "f": pa.array(f, pa.int16(), mask=fn),
                    "v": pa.array(v, pa.int64(), mask=vn), "x": pa.array(x, pa.float64(), mask=xn)})
    for name, c in CASES.items():
        kw = dict(row_group_size=8_000, data_page_version=c["version"], data_page_size=8 * 1024,
                  use_dictionary=c["dictionary"])
        if c["dictionary"] is True:
            kw["dictionary_pagesize_limit"] = 16 * 1024  # v and x fall back to PLAIN pages
        _write(name, tbl, compression=c.get("compression", "none"), **kw)
    strs, _, v2, kn2, vn2 = varchar_columns()
    t2 = pa.table({"name": pa.array([s.decode() for s in strs], pa.string(), mask=kn2),
                   "v": pa.array(v2, pa.int64(), mask=vn2)})
    _write("pa_varchar_nulls", t2, row_group_size=8_000, data_page_size=4 * 1024)
    _write("pa_varchar_nulls_snappy", t2, compression="snappy", row_group_size=8_000, data_page_size=4 * 1024)
    # PLAIN BYTE_ARRAY data pages: no dictionary at all, and a dictionary
    # whose page limit is reached (pyarrow falls back to PLAIN pages)
    _write("pa_varchar_plain", t2, row_group_size=8_000, data_page_size=4 * 1024, use_dictionary=False)
    _write("pa_varchar_fallback_v2", t2, row_group_size=8_000, data_page_size=4 * 1024,
           dictionary_pagesize_limit=4 * 1024, data_page_version="2.0")
    _write("pa_varchar_fallback_snappy", t2, compression="snappy", row_group_size=8_000, data_page_size=4 * 1024,
           dictionary_pagesize_limit=4 * 1024)
    _write("pa_varchar_nulls_zstd", t2, compression="zstd", row_group_size=8_000, data_page_size=4 * 1024)
    _write("pa_varchar_fallback_zstd", t2, compression="zstd", row_group_size=8_000, data_page_size=4 * 1024,
           dictionary_pagesize_limit=4 * 1024, data_page_version="2.0")
    t3 = pa.table({"k": pa.array(np.arange(1000, dtype=np.int32) % 7), "v": pa.array(np.arange(1000, dtype=np.int64))})
    _write("pa_optional_nonnull", t3)
    t4 = pa.table({"c": pa.array(int64_column(), pa.int64())})
    _write("pa_int64_fallback", t4, row_group_size=8_000, data_page_size=8 * 1024,
           dictionary_pagesize_limit=16 * 1024)


if __name__ == "__main__":
    main()
