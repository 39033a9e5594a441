"""GPU parity of the Parquet path: pages decoded on the GPU (dictionary
RLE/bit-unpack + gather, PLAIN loads), filtered and aggregated, against the
oracle on the same logical columns.  Integer results bit-exact."""
import numpy as np
import pytest

import oracle
from slothdb_gb300 import capi
from slothdb_gb300 import parquet as pq
from slothdb_gb300.capi import BIGINT, DOUBLE, INTEGER, SMALLINT
from util import compare, gpu_to_dict

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("oracle_lib", "gblib")]


def run_pq(data, col_types, col_map, group_cols, aggs, filters=(), est_groups=0, device=False, batches=1,
           mode=0, nullable=(), pruned=None):
    pf = capi.ParquetFile(data)
    if device:
        pf.upload()
    g = capi.GroupBy(col_types, group_cols, aggs, filters=filters, est_groups=est_groups,
                     options={"mode": mode} if mode else None, nullable=nullable)
    try:
        nrg = pf.num_row_groups
        step = max(1, (nrg + batches - 1) // batches)
        for b in range(0, nrg, step):
            capi.ingest_parquet(g, pf, col_map, b, min(nrg, b + step), device=device)
        if pruned is not None:
            pruned.append(g.row_groups_pruned())
        g.finalize()
        res = g.result()
    finally:
        g.close()
        pf.close()
    out_types = [col_types[c] for c in group_cols] + [
        oracle.agg_out_type(oracle.AGG_NAMES[k], col_types[c] if c >= 0 else 0) for k, c in aggs]
    return gpu_to_dict(res, len(group_cols), out_types)


def test_filter_groupby_file_2m_rows():
    """The fused decode + filter + aggregate shape: SELECT key, SUM(v),
    COUNT(*) WHERE f < 100 GROUP BY key (10% selectivity)."""
    data, key, f, v = pq.filter_groupby_file(n_rows=2_000_000, row_group_rows=200_000, page_rows=16_384)
    aggs = [("sum", 2), ("count_star", -1)]
    types = [INTEGER, SMALLINT, BIGINT]
    orc = oracle.run_query(types, [0], aggs, [key, f.astype(np.int16), v], filters=[(1, "<", 100)])
    for device, batches in [(False, 1), (True, 3)]:
        gpu = run_pq(data, types, [0, 1, 2], [0], aggs, filters=[(1, "<", 100)], est_groups=65_536,
                     device=device, batches=batches)
        compare(gpu, orc)


def test_no_filter_and_radix_mode():
    data, key, f, v = pq.filter_groupby_file(n_rows=600_000, row_group_rows=100_000, page_rows=32_768, n_dict=4096)
    aggs = [("count_star", -1), ("sum", 2), ("min", 2), ("max", 2)]
    types = [INTEGER, SMALLINT, BIGINT]
    orc = oracle.run_query(types, [0], aggs, [key, f.astype(np.int16), v])
    compare(run_pq(data, types, [0, 1, 2], [0], aggs), orc)
    compare(run_pq(data, types, [0, 1, 2], [0], aggs, mode=2), orc)


@pytest.mark.parametrize("n_dict", [1, 2, 3, 100, 255, 256, 257, 70_000, 1 << 20])
def test_dictionary_bit_widths(n_dict):
    """bit widths 1..20, RLE and bit-packed runs, ragged page tails."""
    rng = np.random.default_rng(n_dict)
    n = 150_007
    dictionary = rng.integers(-(2**31), 2**31 - 1, n_dict, dtype=np.int64).astype(np.int32)
    lens = rng.geometric(0.1, n)
    idx = np.repeat(rng.integers(0, n_dict, len(lens)).astype(np.uint32), lens)[:n]
    v = rng.integers(-1000, 1000, n, dtype=np.int64)
    cols = [pq.Column("k", pq.T_INT32, dictionary=dictionary, indices=idx),
            pq.Column("v", pq.T_INT64, values=v, page_rows=10_000)]  # pages not aligned with k's
    data = pq.write(cols, row_group_rows=50_000, page_rows=7_001)
    aggs = [("count_star", -1), ("sum", 1)]
    orc = oracle.run_query([INTEGER, BIGINT], [0], aggs, [dictionary[idx], v])
    compare(run_pq(data, [INTEGER, BIGINT], [0, 1], [0], aggs), orc)


def test_int64_dictionary_and_double_plain():
    rng = np.random.default_rng(77)
    n = 200_000
    dictionary = rng.integers(-(2**62), 2**62, 5000, dtype=np.int64)
    idx = rng.integers(0, 5000, n).astype(np.uint32)
    x = rng.normal(0, 1e3, n)
    cols = [pq.Column("k", pq.T_INT64, dictionary=dictionary, indices=idx),
            pq.Column("x", pq.T_DOUBLE, values=x)]
    data = pq.write(cols, row_group_rows=64_000, page_rows=9_000)
    aggs = [("count_star", -1), ("sum", 1), ("min", 1), ("max", 1), ("avg", 1)]
    orc = oracle.run_query([BIGINT, DOUBLE], [0], aggs, [dictionary[idx], x], filters=[(1, ">", -500.0)])
    gpu = run_pq(data, [BIGINT, DOUBLE], [0, 1], [0], aggs, filters=[(1, ">", -500.0)])
    compare(gpu, orc)


def test_plain_key_column_and_column_map():
    rng = np.random.default_rng(5)
    n = 100_000
    a = rng.integers(0, 1000, n, dtype=np.int32)
    b = rng.integers(0, 50, n, dtype=np.int64)
    cols = [pq.Column("a", pq.T_INT32, values=a), pq.Column("b", pq.T_INT64, values=b)]
    data = pq.write(cols, row_group_rows=30_000, page_rows=5_000)
    # spec column 0 <- file column 1 (b), spec column 1 <- file column 0 (a)
    aggs = [("count_star", -1), ("sum", 1)]
    orc = oracle.run_query([BIGINT, INTEGER], [0], aggs, [b, a])
    compare(run_pq(data, [BIGINT, INTEGER], [1, 0], [0], aggs), orc)


def test_varchar_dictionary_key():
    """A dictionary-encoded BYTE_ARRAY key (each row group with its own
    dictionary order): dictionary strings encoded once per batch into the
    handle's string dictionary, data pages gathering string ids; host and
    resident files, one or several batches, with a filter."""
    data, d, idx, f, v = pq.varchar_groupby_file(n_rows=300_000, row_group_rows=60_000, page_rows=8192)
    names = pq.strings_of(d, idx)
    types = [capi.VARCHAR, SMALLINT, BIGINT]
    aggs = [("count_star", -1), ("sum", 2), ("max", 1)]
    for filters in ([], [(1, "<", 500)]):
        orc = oracle.run_query(types, [0], aggs, [names, f.astype(np.int16), v], filters=filters)
        for device, batches in [(False, 1), (True, 1), (False, 3), (True, 5)]:
            gpu = run_pq(data, types, [0, 1, 2], [0], aggs, filters=filters, est_groups=3000, device=device,
                         batches=batches)
            compare(gpu, orc)


import os  # noqa: E402
import sys  # noqa: E402

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_pyarrow_files as paf  # noqa: E402


@pytest.mark.parametrize("name", sorted(paf.CASES))
def test_pyarrow_files_with_nulls(name):
    """Files written by pyarrow (an independent writer: OPTIONAL columns with
    definition levels, data page v1 and v2, its own page splits, dictionary
    fallback to PLAIN pages, SNAPPY and ZSTD pages; committed under
    tests/golden/) through the GPU
    decoder: NULLs in the key, the filter column and the value columns,
    against the oracle on the same logical columns."""
    data = paf.load(name)
    (key, f, v, x), nulls = paf.columns()
    types = [INTEGER, SMALLINT, BIGINT, DOUBLE]
    aggs = [("count_star", -1), ("count", 2), ("sum", 2), ("min", 2), ("max", 3), ("sum", 3), ("avg", 3)]
    for filters in ([], [(1, "<", 500)], [(1, "in", [3, 5, 800])]):
        orc = oracle.run_query(types, [0], aggs, [key, f, v, x], filters=filters, nulls=nulls)
        for device in (False, True):
            gpu = run_pq(data, types, [0, 1, 2, 3], [0], aggs, filters=filters, est_groups=2000, device=device,
                         nullable=[0, 1, 2, 3])
            compare(gpu, orc)


@pytest.mark.parametrize("name", ["pa_varchar_nulls", "pa_varchar_nulls_snappy", "pa_varchar_plain",
                                  "pa_varchar_fallback_v2", "pa_varchar_fallback_snappy",
                                  "pa_varchar_nulls_zstd", "pa_varchar_fallback_zstd"])
def test_pyarrow_varchar_key_with_nulls(name):
    """A pyarrow-written VARCHAR key with NULL keys (one NULL group) and a
    nullable value column; a LIKE and an equality on the key; dictionary
    pages, PLAIN BYTE_ARRAY pages (no dictionary, or pyarrow's fallback to
    PLAIN once the dictionary page limit is reached: both encodings in one
    chunk), data page v1 and v2, uncompressed and SNAPPY."""
    data = paf.load(name)
    _, names, v, kn, vn = paf.varchar_columns()
    types = [capi.VARCHAR, BIGINT]
    aggs = [("count_star", -1), ("count", 1), ("sum", 1)]
    for filters in ([], [(0, "like", b"k001")], [(0, "==", b"k00042")]):
        orc = oracle.run_query(types, [0], aggs, [names, v], filters=filters, nulls=[kn, vn])
        for device in (False, True):
            gpu = run_pq(data, types, [0, 1], [0], aggs, filters=filters, est_groups=1500, device=device,
                         nullable=[0, 1])
            compare(gpu, orc)


def test_optional_column_must_be_declared_nullable():
    pf = capi.ParquetFile(paf.load("pa_optional_nonnull"))
    g = capi.GroupBy([INTEGER, BIGINT], [0], [("sum", 1)])
    try:
        with pytest.raises(capi.GbError) as e:
            capi.ingest_parquet(g, pf, [0, 1])
        assert "nullable" in str(e.value)
    finally:
        g.close()
        pf.close()
    # declared nullable, the same file aggregates (no NULLs in it)
    k = np.arange(1000, dtype=np.int32) % 7
    v = np.arange(1000, dtype=np.int64)
    orc = oracle.run_query([INTEGER, BIGINT], [0], [("sum", 1)], [k, v])
    compare(run_pq(paf.load("pa_optional_nonnull"), [INTEGER, BIGINT], [0, 1], [0], [("sum", 1)], nullable=[0, 1]),
            orc)


def test_parquet_in_list_and_key_string_predicates():
    """IN on integer Parquet columns in the fused scan, and string
    predicates on a dictionary-encoded VARCHAR key, tested once per
    dictionary entry (a dictionary match table)."""
    data, key, f, v = pq.filter_groupby_file(n_rows=400_000, row_group_rows=100_000, page_rows=16_384, n_dict=2048)
    types = [INTEGER, SMALLINT, BIGINT]
    aggs = [("sum", 2), ("count_star", -1)]
    members = [int(x) for x in np.unique(key)[:40]] + [5, 6]
    for filters in ([(1, "in", [1, 2, 3, 500, 999])], [(0, "in", members), (1, "<", 700)]):
        orc = oracle.run_query(types, [0], aggs, [key, f.astype(np.int16), v], filters=filters)
        for device in (False, True):
            compare(run_pq(data, types, [0, 1, 2], [0], aggs, filters=filters, est_groups=2048, device=device), orc)
    data, d, idx, f, v = pq.varchar_groupby_file(n_rows=200_000, row_group_rows=50_000, page_rows=8192)
    names = pq.strings_of(d, idx)
    types = [capi.VARCHAR, SMALLINT, BIGINT]
    aggs = [("count_star", -1), ("sum", 2)]
    for filters in ([(0, "like", b"ab")], [(0, "not like", b"a"), (1, "<", 500)], [(0, "=", d[3])],
                    [(0, "!=", d[3]), (0, "like", b"")]):
        orc = oracle.run_query(types, [0], aggs, [names, f.astype(np.int16), v], filters=filters)
        for device in (False, True):
            compare(run_pq(data, types, [0, 1, 2], [0], aggs, filters=filters, est_groups=3000, device=device), orc)


def test_parquet_int_varchar_pair_key():
    """(SMALLINT, VARCHAR) pair key from a Parquet file: the dictionary
    strings become ids once per batch, packed beside the integer key."""
    data, d, idx, f, v = pq.varchar_groupby_file(n_rows=150_000, row_group_rows=50_000, page_rows=8192, n_dict=300)
    names = pq.strings_of(d, idx)
    types = [capi.VARCHAR, SMALLINT, BIGINT]
    aggs = [("count_star", -1), ("sum", 2)]
    orc = oracle.run_query(types, [1, 0], aggs, [names, f.astype(np.int16), v], filters=[(1, "<", 20)])
    for device in (False, True):
        compare(run_pq(data, types, [0, 1, 2], [1, 0], aggs, filters=[(1, "<", 20)], est_groups=6000, device=device),
                orc)


@pytest.mark.parametrize("codec", ["snappy", "zstd"])
@pytest.mark.parametrize("device", [False, True])
def test_compressed_pages_from_the_project_writer(device, codec):
    """SNAPPY or ZSTD column chunks (dictionary and data pages) decompressed
    on the GPU per batch and decoded from the image, against the oracle;
    several batches, with a filter that the zone maps do not prune."""
    _, key, f, v = pq.filter_groupby_file(n_rows=300_000, row_group_rows=50_000, page_rows=8192, n_dict=4096)
    cols = [pq.Column("key", pq.T_INT32, values=key), pq.Column("f", pq.T_INT32, values=f, int16=True),
            pq.Column("v", pq.T_INT64, values=v)]
    data = pq.write(cols, row_group_rows=50_000, page_rows=8192, codec=codec)
    types = [INTEGER, SMALLINT, BIGINT]
    aggs = [("sum", 2), ("count_star", -1), ("max", 2)]
    for filters, batches in (([], 1), ([(1, "<", 300)], 3)):
        orc = oracle.run_query(types, [0], aggs, [key, f.astype(np.int16), v], filters=filters)
        compare(run_pq(data, types, [0, 1, 2], [0], aggs, filters=filters, est_groups=4096, device=device,
                       batches=batches), orc)


def test_snappy_byte_patterns():
    """SNAPPY pages whose blocks exercise every element shape of the
    inflate: incompressible values (literals longer than a round, copied by
    the whole warp), constant and short-period runs (overlapping copies of
    up to 64 bytes, sources inside the same round), small values in runs
    (short literals followed by copies of them), pages whose block ends
    inside a round; the decoded values against the oracle bit for bit
    (magnitudes below 2^44: every group's SUM stays below 2^53, where the
    reference's double accumulator is exact)."""
    rng = np.random.default_rng(31)
    seg = 24_576
    v = np.concatenate([
        rng.integers(-2**44, 2**44, seg, dtype=np.int64),                           # incompressible
        np.zeros(seg, dtype=np.int64),                                               # one long run
        np.tile(np.array([7, -3, 2**40], dtype=np.int64), seg // 3),                 # period 24 bytes
        np.repeat(rng.integers(0, 256, seg // 4, dtype=np.int64), 4),                # short runs
        rng.integers(0, 4, seg, dtype=np.int64),                                     # tiny alphabet
        np.repeat(rng.integers(-2**44, 2**44, seg // 64, dtype=np.int64), 64),       # long runs of random words
        rng.integers(-1000, 1000, 5_000, dtype=np.int64),                            # a ragged tail
    ])
    n = len(v)
    key = (np.arange(n) % 97).astype(np.int32)
    cols = [pq.Column("key", pq.T_INT32, values=key), pq.Column("v", pq.T_INT64, values=v)]
    for page_rows in (8192, 3000):
        data = pq.write(cols, row_group_rows=40_000, page_rows=page_rows, codec="snappy")
        types = [INTEGER, BIGINT]
        aggs = [("sum", 1), ("min", 1), ("max", 1), ("count_star", -1)]
        orc = oracle.run_query(types, [0], aggs, [key, v])
        compare(run_pq(data, types, [0, 1], [0], aggs, est_groups=97, device=True), orc)


def test_corrupt_snappy_block_is_reported():
    """A page whose Snappy block is damaged (a copy reaching before the
    start of the output) is reported as a corrupt file, not decoded."""
    zeros = np.zeros(20_000, dtype=np.int64)
    data = bytearray(pq.write([pq.Column("v", pq.T_INT64, values=zeros)], row_group_rows=20_000, page_rows=20_000,
                              codec="snappy"))
    # the page's block: a varint length, a literal, then copies with a 2-byte
    # offset (tag ..10); its first copy's offset is raised past its position
    blk = pq.snappy_compress(zeros.tobytes())
    at = bytes(data).index(blk)
    j = 0
    while blk[j] & 0x80:
        j += 1
    j += 1  # past the length varint
    assert blk[j] & 3 == 0  # the literal
    j += 1 + (blk[j] >> 2) + 1
    assert blk[j] & 3 == 2  # the first copy
    data[at + j + 1], data[at + j + 2] = 0xff, 0x7f
    pf = capi.ParquetFile(bytes(data))
    g = capi.GroupBy([BIGINT], [0], [("count_star", -1)])
    try:
        with pytest.raises(capi.GbError) as e:
            capi.ingest_parquet(g, pf, [0])
        assert e.value.status == 6  # GB_ERR_CORRUPT
    finally:
        g.close()
        pf.close()


def test_corrupt_zstd_page_is_reported():
    """A ZSTD page whose frame is damaged (its magic number zeroed) is
    reported as a corrupt file, not decoded."""
    data = bytearray(paf.load("pa_nulls_v1_zstd"))
    at = bytes(data).index(b"\x28\xb5\x2f\xfd", 4)  # the first frame
    data[at:at + 4] = bytes(4)
    pf = capi.ParquetFile(bytes(data))
    g = capi.GroupBy([INTEGER, SMALLINT, BIGINT, DOUBLE], [0], [("count_star", -1)], nullable=[0, 1, 2, 3])
    try:
        with pytest.raises(capi.GbError) as e:
            capi.ingest_parquet(g, pf, [0, 1, 2, 3])
        assert e.value.status == 6  # GB_ERR_CORRUPT
    finally:
        g.close()
        pf.close()


@pytest.mark.parametrize("key", ["int", "varchar"])
def test_zone_map_pruning_against_the_oracle(key):
    """Row groups whose statistics rule out the WHERE clause are skipped
    (none, some, all of them) and the result still equals the oracle's over
    the whole file; a numeric and a dictionary-encoded VARCHAR key (whose
    dictionaries of skipped row groups are not encoded), one or several
    batches, host and resident files."""
    n, rg = 240_000, 40_000
    rng = np.random.default_rng(41)
    f = (np.arange(n) // rg * 100 + rng.integers(0, 100, n)).astype(np.int32)  # row group g: [100g, 100g + 100)
    v = rng.integers(-10**6, 10**6, n, dtype=np.int64)
    idx = rng.integers(0, 1500, n).astype(np.uint32)
    if key == "int":
        d = rng.integers(-(2**31), 2**31 - 1, 1500, dtype=np.int64).astype(np.int32)
        kcol = pq.Column("k", pq.T_INT32, dictionary=d, indices=idx)
        types, kvals = [INTEGER, INTEGER, BIGINT], d[idx]
    else:
        d = [b"name-%05d" % i * (1 + i % 3) for i in range(1500)]
        kcol = pq.Column("k", pq.T_BYTE_ARRAY, dictionary=d, indices=idx, shuffle_seed=3)
        types, kvals = [capi.VARCHAR, INTEGER, BIGINT], pq.strings_of(d, idx)
    # f is an INTEGER column: the reference reads no statistics for SMALLINT
    data = pq.write([kcol, pq.Column("f", pq.T_INT32, values=f), pq.Column("v", pq.T_INT64, values=v)],
                    row_group_rows=rg, page_rows=8192, stats=True)
    aggs = [("count_star", -1), ("sum", 2), ("max", 2)]
    for filters, n_pruned in (([(1, "<", 1000)], 0), ([(1, "<", 250)], 3), ([(1, ">=", 300), (1, "<", 420)], 4),
                              ([(1, ">", 5000)], 6)):
        orc = oracle.run_query(types, [0], aggs, [kvals, f, v], filters=filters)
        for device, batches in ((False, 1), (True, 1), (False, 4), (True, 6)):
            got = []
            gpu = run_pq(data, types, [0, 1, 2], [0], aggs, filters=filters, est_groups=1500, device=device,
                         batches=batches, pruned=got)
            assert got == [n_pruned], (filters, device, batches, got)
            compare(gpu, orc)


def _exact(vals):
    return int(np.asarray(vals, dtype=np.int64).astype(object).sum())


def _near(got, vals):
    """(count, sum) equal to the values' count and exact sum rounded once."""
    cnt, sm = got
    ex = _exact(vals)
    return cnt == len(vals) and abs(sm - ex) <= abs(ex) * 2.0 ** -52

def test_dictionary_histogram_sum():
    """Ungrouped SUM / COUNT of an INT64 dictionary column through the
    dictionary histogram (no decode), host and resident files, a row-group
    range, a dictionary that falls back to PLAIN pages (pyarrow), OPTIONAL
    without NULLs; the shapes the reference leaves to its fused path (NULLs,
    no dictionary, not INT64) are GB_ERR_UNSUPPORTED."""
    rng = np.random.default_rng(91)
    n = 300_007
    d = rng.integers(-10**12, 10**12, 5000, dtype=np.int64)
    lens = rng.geometric(0.2, n)
    idx = np.repeat(rng.integers(0, len(d), len(lens)).astype(np.uint32), lens)[:n]
    plain = rng.integers(0, 10**6, n, dtype=np.int64)
    data = pq.write([pq.Column("k", pq.T_INT32, values=(idx % 97).astype(np.int32)),
                     pq.Column("c", pq.T_INT64, dictionary=d, indices=idx),
                     pq.Column("p", pq.T_INT64, values=plain)], row_group_rows=50_000, page_rows=7_001)
    vals = d[idx]
    pf = capi.ParquetFile(data)
    try:
        pf.upload()
        for device in (False, True):
            assert _near(pf.dict_sum(1, device=device), vals)
            assert _near(pf.dict_sum(1, 2, 4, device=device), vals[100_000:200_000])
        assert pf.dict_sum(1, 3, 3) == (0, 0.0)
        for col in (0, 2):  # INT32; INT64 without a dictionary
            with pytest.raises(capi.GbError) as e:
                pf.dict_sum(col)
            assert e.value.status == capi.GB_ERR_UNSUPPORTED
    finally:
        pf.close()
    for name, col, expect in (("pa_optional_nonnull", 1, np.arange(1000, dtype=np.int64)),
                              ("pa_int64_fallback", 0, paf.int64_column())):
        pf = capi.ParquetFile(paf.load(name))
        try:
            assert _near(pf.dict_sum(col), expect)
        finally:
            pf.close()
    pf = capi.ParquetFile(paf.load("pa_nulls_v1_dict"))  # v holds NULLs
    try:
        with pytest.raises(capi.GbError) as e:
            pf.dict_sum(2)
        assert e.value.status == capi.GB_ERR_UNSUPPORTED
    finally:
        pf.close()
