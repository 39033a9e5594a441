"""Parquet on the host: the project writer (checked against pyarrow when it is
installed), the oracle's RleDecoder restatement on the writer's encoding, and
the library's footer / page-header parser (no GPU needed)."""
import io

import numpy as np
import pytest

import oracle
from slothdb_gb300 import capi
from slothdb_gb300 import parquet as pq

pytestmark = pytest.mark.usefixtures("oracle_lib", "gblib")


@pytest.mark.parametrize("bw", [1, 2, 3, 5, 7, 8, 9, 13, 16, 17, 20, 24, 31, 32])
def test_rle_hybrid_roundtrip_through_oracle(bw):
    rng = np.random.default_rng(bw)
    n = 10_007  # not a multiple of 8 or 32: ragged tail
    hi = (1 << bw) - 1 if bw < 32 else 0xFFFFFFFF
    lens = rng.geometric(0.2, n)
    vals = rng.integers(0, hi, len(lens), dtype=np.uint64, endpoint=True).astype(np.uint32)
    x = np.repeat(vals, lens)[:n]
    x[100:180] = x[100]  # a long RLE run
    enc = pq.rle_hybrid(x, bw)
    dec = oracle.rle_decode(enc, bw, n)
    assert np.array_equal(dec, x)


def test_writer_matches_pyarrow():
    pa = pytest.importorskip("pyarrow.parquet")
    data, key, f, v = pq.filter_groupby_file(n_rows=250_000, row_group_rows=100_000, page_rows=16_384)
    t = pa.read_table(io.BytesIO(data))
    assert np.array_equal(t.column("key").to_numpy(), key)
    assert np.array_equal(t.column("f").to_numpy(), f)
    assert np.array_equal(t.column("v").to_numpy(), v)
    assert str(t.schema.field("f").type) == "int16"


def test_library_parses_footer_and_pages():
    data, key, f, v = pq.filter_groupby_file(n_rows=250_000, row_group_rows=100_000, page_rows=16_384)
    pf = capi.ParquetFile(data)
    assert pf.num_row_groups == 3
    assert pf.num_rows == 250_000
    assert pf.columns() == [("key", capi.INTEGER), ("f", capi.SMALLINT), ("v", capi.BIGINT)]
    pf.close()


@pytest.mark.parametrize("damage", ["magic", "footer_len", "truncated", "page_size"])
def test_malformed_files_are_rejected(damage):
    data, _, _, _ = pq.filter_groupby_file(n_rows=20_000, row_group_rows=10_000, page_rows=4096)
    b = bytearray(data)
    if damage == "magic":
        b[-1] = ord("X")
    elif damage == "footer_len":
        b[-8:-4] = (len(b) * 2).to_bytes(4, "little")
    elif damage == "truncated":
        b = b[: len(b) // 2] + b[-8:]
    elif damage == "page_size":
        # first data page header of column 'f' lies after the key chunk; grow its
        # compressed_page_size varint so the page runs past the chunk
        flen = int.from_bytes(b[-8:-4], "little")
        assert flen > 0
        i = 4
        # corrupt the dictionary page header's size field (first header in the file)
        b[i + 3] = 0x7F
    with pytest.raises(capi.GbError) as e:
        capi.ParquetFile(bytes(b))
    assert e.value.status in (6,)  # GB_ERR_CORRUPT


def test_varchar_dictionary_file_writer_and_parser():
    """BYTE_ARRAY dictionary-encoded key: pyarrow decodes the project writer's
    file (each row group with its own dictionary order) to the same strings,
    and the library's parser reports the column as VARCHAR."""
    data, d, idx, f, v = pq.varchar_groupby_file(n_rows=30_000, row_group_rows=8_000, page_rows=2048)
    pa = pytest.importorskip("pyarrow.parquet")
    t = pa.read_table(io.BytesIO(data))
    got = [x if isinstance(x, bytes) else x.encode() for x in t.column("name").to_pylist()]
    assert got == [d[i] for i in idx.tolist()]
    pf = capi.ParquetFile(data)
    assert pf.num_row_groups == 4
    assert pf.columns() == [("name", capi.VARCHAR), ("f", capi.SMALLINT), ("v", capi.BIGINT)]
    pf.close()
    offs, blob = pq.strings_of(d, idx[:5])
    assert [bytes(blob[offs[i]:offs[i + 1]]) for i in range(5)] == [d[i] for i in idx[:5].tolist()]


def test_varchar_dictionary_header_checked_on_open(monkeypatch):
    """A BYTE_ARRAY dictionary page declaring more values than its payload
    can hold (4 length bytes each) is rejected as corrupt by the parser."""
    real = pq._page_header

    def inflated(ptype, size, num_values=None, encoding=None, dict_values=None):
        if ptype == pq.PAGE_DICT:
            dict_values = size  # > size / 4
        return real(ptype, size, num_values=num_values, encoding=encoding, dict_values=dict_values)

    monkeypatch.setattr(pq, "_page_header", inflated)
    data, _, _, _, _ = pq.varchar_groupby_file(n_rows=5_000, row_group_rows=5_000, page_rows=2048)
    with pytest.raises(capi.GbError) as e:
        capi.ParquetFile(data)
    assert e.value.status == 6  # GB_ERR_CORRUPT


def test_snappy_oracle_matches_pyarrow():
    """The oracle's Snappy restatement decompresses blocks made by an
    independent Snappy (pyarrow's) and by the project writer's compressor,
    which pyarrow also decompresses; malformed blocks are refused."""
    pa = pytest.importorskip("pyarrow")
    rng = np.random.default_rng(7)
    blocks = [b"", b"x", b"abcabcabcabc" * 500, rng.integers(0, 256, 70_000, dtype=np.uint8).tobytes(),
              rng.integers(0, 3, 200_000, dtype=np.uint8).tobytes(),
              np.repeat(rng.integers(0, 1 << 20, 5000), 7).astype(np.int64).tobytes()]
    for data in blocks:
        assert oracle.snappy_decompress(pa.compress(data, codec="snappy", asbytes=True)) == data
        ours = pq.snappy_compress(data)
        assert oracle.snappy_decompress(ours) == data
        assert pa.decompress(ours, decompressed_size=len(data), codec="snappy", asbytes=True) == data
    good = pq.snappy_compress(b"hello hello hello hello")
    for bad in (good[:-1], good[:1] + b"\x0a\x00\x00", bytes([5, 0x06, 0xff, 0x00])):
        with pytest.raises(ValueError):
            oracle.snappy_decompress(bad)


def test_snappy_file_read_by_pyarrow_and_opened_by_the_gpu_parser():
    """SNAPPY column chunks from the writer are valid Parquet (pyarrow reads the
    same values) and the library's parser takes them (the pages are inflated
    on the GPU per batch); a GZIP file is refused on open."""
    pa = pytest.importorskip("pyarrow.parquet")
    _, key, f, v = pq.filter_groupby_file(n_rows=30_000, row_group_rows=10_000, page_rows=4096, n_dict=512)
    cols = [pq.Column("key", pq.T_INT32, values=key), pq.Column("f", pq.T_INT32, values=f, int16=True),
            pq.Column("v", pq.T_INT64, values=v)]
    data = pq.write(cols, row_group_rows=10_000, page_rows=4096, codec="snappy")
    plain = pq.write(cols, row_group_rows=10_000, page_rows=4096)
    assert len(data) < len(plain)
    t = pa.read_table(io.BytesIO(data))
    assert np.array_equal(t.column("key").to_numpy(), key) and np.array_equal(t.column("v").to_numpy(), v)
    pf = capi.ParquetFile(data)
    assert pf.num_rows == 30_000 and pf.columns() == [("key", capi.INTEGER), ("f", capi.SMALLINT), ("v", capi.BIGINT)]
    pf.close()
    import pyarrow as pa_
    buf = io.BytesIO()
    pa.write_table(pa_.table({"v": pa_.array(v)}), buf, compression="gzip")
    with pytest.raises(capi.GbError) as e:
        capi.ParquetFile(buf.getvalue())
    assert e.value.status == 3  # GB_ERR_UNSUPPORTED


def _zone_expect(op, v, mn, mx):
    """The reference's RowGroupMightMatch rules (parquet.cpp:3200-3240)."""
    return {"==": not (v < mn) and not (mx < v), ">": not (mx < v) and not (mx == v), ">=": not (mx < v),
            "<": not (v < mn) and not (mn == v), "<=": not (v < mn), "!=": not (mn == v and mx == v)}[op]


OPS = ["==", "!=", "<", "<=", ">", ">="]


def test_zone_maps_follow_the_reference_rules():
    """Row-group statistics written by the project writer (read back by
    pyarrow as the same min/max) rule row groups out exactly as the
    reference's zone-map check does, never ruling out one that has a passing
    row; SMALLINT columns carry none (as in the reference) and files without
    statistics rule nothing out."""
    pa = pytest.importorskip("pyarrow.parquet")
    n, rg = 40_000, 10_000
    rng = np.random.default_rng(11)
    k = np.sort(rng.integers(-1000, 1000, n)).astype(np.int32)
    x = np.sort(rng.normal(0, 3, n))
    v = np.arange(n, dtype=np.int64) * 3
    s16 = np.sort(rng.integers(0, 1000, n)).astype(np.int32)
    cols = [pq.Column("k", pq.T_INT32, values=k), pq.Column("x", pq.T_DOUBLE, values=x),
            pq.Column("v", pq.T_INT64, values=v), pq.Column("s", pq.T_INT32, values=s16, int16=True)]
    data = pq.write(cols, row_group_rows=rg, page_rows=4096, stats=True)
    md = pa.ParquetFile(io.BytesIO(data)).metadata
    pf = capi.ParquetFile(data)
    cm = [0, 1, 2, 3]
    consts = {0: [-1000, -509, -508, 0, 500, 999, 1000], 1: [-20.0, float(x[9_999]), 0.0, float(x[20_000]), 20.0],
              2: [0, 3 * 9_999, 3 * 10_000, 3 * 39_999, 10**9]}
    for g in range(4):
        lo, hi = g * rg, (g + 1) * rg
        for c, arr in ((0, k), (1, x), (2, v)):
            st = md.row_group(g).column(c).statistics
            assert st.min == arr[lo:hi].min() and st.max == arr[lo:hi].max()
            for const in consts[c]:
                for op in OPS:
                    got = pf.row_group_might_match(g, cm, [(c, op, const)])
                    assert got == _zone_expect(op, const, arr[lo:hi].min(), arr[lo:hi].max()), (g, c, op, const)
                    passing = {"==": arr[lo:hi] == const, "!=": arr[lo:hi] != const, "<": arr[lo:hi] < const,
                               "<=": arr[lo:hi] <= const, ">": arr[lo:hi] > const, ">=": arr[lo:hi] >= const}[op]
                    assert got or not passing.any()
        assert pf.row_group_might_match(g, cm, [(3, "<", -1)])       # SMALLINT: no statistics read
        assert pf.row_group_might_match(g, cm, [])
    # a conjunction is ruled out when any one filter is
    assert not pf.row_group_might_match(3, cm, [(1, ">", -100.0), (0, "<", 0)])
    pf.close()
    plain = capi.ParquetFile(pq.write(cols, row_group_rows=rg, page_rows=4096))
    assert all(plain.row_group_might_match(g, cm, [(0, "<", -5000)]) for g in range(4))
    plain.close()


def test_zone_maps_from_pyarrow_statistics():
    """Statistics written by pyarrow (an independent writer) drive the same
    decisions."""
    pa = pytest.importorskip("pyarrow")
    pq_ = pytest.importorskip("pyarrow.parquet")
    n = 30_000
    k = np.sort(np.random.default_rng(12).integers(-10**9, 10**9, n))
    t = pa.table({"k": pa.array(k, type=pa.int64()), "w": pa.array(np.arange(n, dtype=np.int32))})
    buf = io.BytesIO()
    pq_.write_table(t, buf, row_group_size=7_500, compression="none", use_dictionary=False,
                    write_statistics=True, data_page_version="1.0")
    data = buf.getvalue()
    pf = capi.ParquetFile(data)
    for g in range(4):
        lo, hi = g * 7_500, (g + 1) * 7_500
        for const in (int(k[0]) - 1, int(k[lo]), int(k[hi - 1]), 0, int(k[-1]) + 1):
            for op in OPS:
                assert pf.row_group_might_match(g, [0, 1], [(0, op, const)]) == \
                    _zone_expect(op, const, int(k[lo:hi].min()), int(k[lo:hi].max())), (g, op, const)
    pf.close()


def test_unsigned_columns():
    """Unsigned integers: uint8/uint16 columns (stored INT32) read as INTEGER;
    uint32/uint64 columns, whose values and statistics are ordered unsigned
    (values >= 2^31 would read negative), are refused by the GPU path, so a
    zone map can never rule out a row group on statistics read with the wrong
    sign."""
    pa = pytest.importorskip("pyarrow")
    pq_ = pytest.importorskip("pyarrow.parquet")
    n = 1000
    u32 = np.array([1, 0xFFFFFFFF] * (n // 2), dtype=np.uint32)
    t = pa.table({"a": pa.array(np.arange(n) % 200, type=pa.uint8()),
                  "b": pa.array(np.arange(n) * 60, type=pa.uint16()),
                  "c": pa.array(u32, type=pa.uint32()),
                  "d": pa.array(np.arange(n, dtype=np.uint64) << np.uint64(40), type=pa.uint64())})
    buf = io.BytesIO()
    pq_.write_table(t, buf, row_group_size=500, compression="none", write_statistics=True)
    pf = capi.ParquetFile(buf.getvalue())
    assert pf.columns() == [("a", capi.INTEGER), ("b", capi.INTEGER), ("c", 0), ("d", 0)]
    pf.close()


def test_optional_columns_parse():
    """pyarrow writes OPTIONAL columns (definition levels before the values,
    page v1 and v2): the footer and page parser accepts them; a page whose
    level length overruns the page is rejected."""
    pa = pytest.importorskip("pyarrow")
    pq_ = pytest.importorskip("pyarrow.parquet")
    n = 5000
    rng = np.random.default_rng(3)
    v = pa.array(rng.integers(0, 100, n), type=pa.int64(), mask=rng.random(n) < 0.2)
    for version in ("1.0", "2.0"):
        buf = io.BytesIO()
        pq_.write_table(pa.table({"k": pa.array(np.arange(n, dtype=np.int32) % 9), "v": v}), buf,
                        compression="none", data_page_version=version, row_group_size=2000)
        pf = capi.ParquetFile(buf.getvalue())
        assert pf.columns() == [("k", capi.INTEGER), ("v", capi.BIGINT)]
        assert pf.num_rows == n and pf.num_row_groups == 3
        pf.close()
    # page v1 of column v: overrun the 4-byte level length
    buf = io.BytesIO()
    pq_.write_table(pa.table({"v": v}), buf, compression="none", data_page_version="1.0", use_dictionary=False,
                    write_statistics=False)
    b = bytearray(buf.getvalue())
    md = pq_.ParquetFile(io.BytesIO(bytes(b))).metadata.row_group(0).column(0)
    start = md.data_page_offset
    # the page header is followed by the 4-byte level length (5000 levels at
    # bit width 1 take a little over 625 bytes)
    found = False
    for off in range(start + 4, start + 64):
        ln = int.from_bytes(b[off:off + 4], "little")
        if 625 <= ln <= 800:
            b[off:off + 4] = (1 << 30).to_bytes(4, "little")
            found = True
            break
    assert found
    with pytest.raises(capi.GbError):
        capi.ParquetFile(bytes(b))


def test_pyarrow_fixtures_match_their_columns():
    """The committed pyarrow files (tests/golden/*.parquet.gz) hold exactly
    the columns and NULLs that make_pyarrow_files.columns() regenerates."""
    pq_ = pytest.importorskip("pyarrow.parquet")
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_pyarrow_files as paf
    cols, nulls = paf.columns()
    for name in paf.CASES:
        t = pq_.read_table(io.BytesIO(paf.load(name)))
        for i, c in enumerate(["key", "f", "v", "x"]):
            col = t.column(c)
            assert np.array_equal(col.is_null().to_numpy(zero_copy_only=False), nulls[i])
            ok = ~nulls[i]
            assert np.array_equal(col.to_numpy(zero_copy_only=False)[ok].astype(cols[i].dtype), cols[i][ok])
        pf = capi.ParquetFile(paf.load(name))
        assert pf.columns() == [("key", capi.INTEGER), ("f", capi.SMALLINT), ("v", capi.BIGINT), ("x", capi.DOUBLE)]
        pf.close()
    strs, _, v, kn, vn = paf.varchar_columns()
    for name in ("pa_varchar_nulls", "pa_varchar_nulls_snappy", "pa_varchar_plain", "pa_varchar_fallback_v2",
                 "pa_varchar_fallback_snappy", "pa_varchar_nulls_zstd", "pa_varchar_fallback_zstd"):
        t = pq_.read_table(io.BytesIO(paf.load(name)))
        got = t.column("name").to_pylist()
        assert [None if n else s_.decode() for s_, n in zip(strs, kn)] == got
        assert np.array_equal(t.column("v").is_null().to_numpy(zero_copy_only=False), vn)
        pf = capi.ParquetFile(paf.load(name))
        assert pf.columns() == [("name", capi.VARCHAR), ("v", capi.BIGINT)]
        pf.close()
