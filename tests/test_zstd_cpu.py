"""The ZSTD page decoder (slothdb_gb300/csrc/gb_zstd.h, the same code the
GPU runs on one lane per page) built for the host and checked against
pyarrow's zstd on the same frames: compression levels from fast to high,
incompressible, constant, run-heavy, integer and text data, frames of
several blocks, the output capacity exactly the decoded size; damaged frames
are refused (or decode to some bytes) without reading or writing outside
their buffers."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def zs(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("zs") / "libzstd_host.so")
    p = subprocess.run([os.environ.get("CXX", "g++"), "-O2", "-shared", "-fPIC", "-I",
                        os.path.join(ROOT, "slothdb_gb300", "csrc"), os.path.join(ROOT, "tests", "cpp", "zstd_host.cpp"),
                        "-o", so], capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-2000:]
    lib = ctypes.CDLL(so)
    lib.zstd_host_decompress.restype = ctypes.c_longlong
    lib.zstd_host_decompress.argtypes = [ctypes.c_char_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_longlong]
    return lib


def _cases():
    rng = np.random.default_rng(0)
    return {
        "random bytes": rng.integers(0, 256, 300_000, dtype=np.uint8).tobytes(),
        "zeros": bytes(500_000),
        "int32 small range": rng.integers(0, 1000, 100_000, dtype=np.int32).tobytes(),
        "int64 wide": rng.integers(-10**9, 10**9, 70_000, dtype=np.int64).tobytes(),
        "uint16 runs": np.repeat(rng.integers(0, 65536, 30_000).astype(np.uint16),
                                 rng.geometric(0.25, 30_000)).tobytes(),
        "text": b"the quick brown fox jumps over the lazy dog " * 5000 + bytes(range(256)) * 50,
        "three bytes": b"abc",
        "empty": b"",
        "sorted int64": np.arange(200_000, dtype=np.int64).tobytes(),
        "8-letter alphabet": bytes(rng.choice(np.frombuffer(b"abcdefgh", np.uint8), 400_000)),
    }


@pytest.mark.parametrize("level", [-5, 1, 3, 9, 19])
def test_zstd_decoder_matches_pyarrow(zs, level):
    pa = pytest.importorskip("pyarrow")
    codec = pa.Codec("zstd", compression_level=level)
    for name, raw in _cases().items():
        c = codec.compress(raw, asbytes=True)
        out = ctypes.create_string_buffer(max(len(raw), 1))
        got = zs.zstd_host_decompress(c, len(c), out, len(raw))
        assert got == len(raw) and out.raw[:len(raw)] == raw, (name, level, got)


def test_zstd_damaged_frames(zs):
    pa = pytest.importorskip("pyarrow")
    rng = np.random.default_rng(1)
    raw = rng.integers(0, 1000, 50_000, dtype=np.int32).tobytes()
    c = bytearray(pa.Codec("zstd", compression_level=3).compress(raw, asbytes=True))
    out = ctypes.create_string_buffer(len(raw))
    bad = bytes(4) + bytes(c[4:])  # no frame magic
    assert zs.zstd_host_decompress(bad, len(bad), out, len(raw)) == -1
    assert zs.zstd_host_decompress(bytes(c[:len(c) // 2]), len(c) // 2, out, len(raw)) == -1  # truncated
    assert zs.zstd_host_decompress(bytes(c), len(c), out, len(raw) - 1) == -1  # output too small
    for _ in range(500):  # damaged bytes: any result, within the buffers
        m = bytearray(c)
        for _ in range(int(rng.integers(1, 4))):
            m[int(rng.integers(0, len(m)))] = int(rng.integers(0, 256))
        r = zs.zstd_host_decompress(bytes(m), len(m), out, len(raw))
        assert -1 <= r <= len(raw)


def test_writer_zstd_frames(zs):
    """The writer's ZSTD frames (slothdb_gb300/pq_encode.c) decode to the
    same bytes with pyarrow's zstd and with the page decoder."""
    pa = pytest.importorskip("pyarrow")
    from slothdb_gb300 import parquet as pq
    for name, raw in _cases().items():
        c = pq.zstd_compress(raw)
        if raw:
            assert pa.decompress(c, decompressed_size=len(raw), codec="zstd", asbytes=True) == raw, name
        out = ctypes.create_string_buffer(max(len(raw), 1))
        assert zs.zstd_host_decompress(c, len(c), out, len(raw)) == len(raw), name
        assert out.raw[:len(raw)] == raw, name


def test_writer_zstd_file_read_by_pyarrow():
    """A ZSTD Parquet file from the writer: pyarrow reads the same values,
    and the library's parser opens it."""
    pq_ = pytest.importorskip("pyarrow.parquet")
    import io
    from slothdb_gb300 import capi
    from slothdb_gb300 import parquet as pq
    _, key, f, v = pq.filter_groupby_file(n_rows=30_000, row_group_rows=10_000, page_rows=4096, n_dict=512)
    cols = [pq.Column("key", pq.T_INT32, values=key), pq.Column("f", pq.T_INT32, values=f, int16=True),
            pq.Column("v", pq.T_INT64, values=v)]
    data = pq.write(cols, row_group_rows=10_000, page_rows=4096, codec="zstd")
    t = pq_.read_table(io.BytesIO(data))
    assert np.array_equal(t.column("key").to_numpy(), key) and np.array_equal(t.column("v").to_numpy(), v)
    assert np.array_equal(t.column("f").to_numpy(), f.astype(np.int16))
    pf = capi.ParquetFile(data)
    assert pf.num_rows == 30_000
    pf.close()
