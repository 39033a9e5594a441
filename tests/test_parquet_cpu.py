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


def test_snappy_file_read_by_pyarrow_and_refused_by_the_gpu_parser():
    """SNAPPY column chunks from the writer are valid Parquet (pyarrow reads the
    same values); the GPU path does not decompress pages yet and refuses the
    file on open."""
    pa = pytest.importorskip("pyarrow.parquet")
    _, key, f, v = pq.filter_groupby_file(n_rows=30_000, row_group_rows=10_000, page_rows=4096, n_dict=512)
    cols = [pq.Column("key", pq.T_INT32, values=key), pq.Column("f", pq.T_INT32, values=f, int16=True),
            pq.Column("v", pq.T_INT64, values=v)]
    data = pq.write(cols, row_group_rows=10_000, page_rows=4096, codec="snappy")
    plain = pq.write(cols, row_group_rows=10_000, page_rows=4096)
    assert len(data) < len(plain)
    t = pa.read_table(io.BytesIO(data))
    assert np.array_equal(t.column("key").to_numpy(), key) and np.array_equal(t.column("v").to_numpy(), v)
    with pytest.raises(capi.GbError) as e:
        capi.ParquetFile(data)
    assert e.value.status == 3  # GB_ERR_UNSUPPORTED
