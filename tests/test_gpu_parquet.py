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
           mode=0):
    pf = capi.ParquetFile(data)
    if device:
        pf.upload()
    g = capi.GroupBy(col_types, group_cols, aggs, filters=filters, est_groups=est_groups,
                     options={"mode": mode} if mode else None)
    try:
        nrg = pf.num_row_groups
        step = max(1, (nrg + batches - 1) // batches)
        for b in range(0, nrg, step):
            capi.ingest_parquet(g, pf, col_map, b, min(nrg, b + step), device=device)
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
