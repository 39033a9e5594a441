"""GPU parity of COUNT(DISTINCT col) against the oracle's per-group value
sets (src/execution/int_group_agg.cpp:89-92, 154-270): counts bit-exact for
every key shape, NULL values never counted, NULL keys their own group, the
pair sets grown across ingests and the HBM table spilling underneath."""
import numpy as np
import pytest

from slothdb_gb300 import capi, datagen
from slothdb_gb300.capi import BIGINT, DOUBLE, INTEGER, SMALLINT, VARCHAR
from test_gpu_groupby import check, run_gpu

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("oracle_lib", "gblib")]

HASH, RADIX = 1, 2
DAGGS = [("count_distinct", 1), ("count_star", -1), ("sum", 1)]


@pytest.mark.parametrize("device", [False, True])
def test_int_key_with_nulls(device):
    n = 400_000
    rng = np.random.default_rng(31)
    k = rng.integers(0, 2000, n, dtype=np.int32)
    v = rng.integers(0, 500, n, dtype=np.int64)
    vn = rng.random(n) < 0.1
    kn = rng.random(n) < 0.01
    # a group whose values are all NULL counts 0 distinct values
    k[:40] = 7777
    kn[:40] = False
    vn[:40] = True
    check([INTEGER, BIGINT], [0], DAGGS, [k, v], nulls=[kn, vn], device=device)


def test_bigint_key_marker_pair_and_null_key():
    """INT64_MIN keys (the table's empty key) with INT64_MIN values (the pair
    set's empty marker) and NULL keys of a BIGINT key (twin sets)."""
    lo = np.iinfo(np.int64).min
    n = 100_000
    rng = np.random.default_rng(32)
    k = rng.integers(-50, 50, n, dtype=np.int64)
    v = rng.integers(-20, 20, n, dtype=np.int64)
    k[:1000:2] = lo
    v[:300] = lo
    v[300:600] = np.iinfo(np.int64).max
    kn = rng.random(n) < 0.05
    kn[:1000:2] = False
    # no SUM: the extreme values put it beyond 2^53, where the reference's
    # double accumulation is not exact
    check([BIGINT, BIGINT], [0], [("count_distinct", 1), ("count_star", -1), ("max", 1)], [k, v],
          nulls=[kn, None], chunks=16_384)


def test_composite_and_varchar_keys():
    a, b, s, m = datagen.composite(300_000, 20_000, seed=33)
    check([INTEGER, SMALLINT, BIGINT, INTEGER], [0, 1], [("count_distinct", 3), ("count_star", -1)], [a, b, s, m])
    (offs, data), s, m = datagen.varchar_table(60_000, 3000, seed=34)
    m = (m % 97).astype(np.int32)
    check([VARCHAR, BIGINT, INTEGER], [0], [("count_distinct", 2), ("max", 1)], [(offs, data), s, m])


def test_two_distinct_columns_filters_and_growth():
    """Two pair sets; a WHERE clause; 12 ingests grow the sets (rehash of
    what they hold) while a 16-group estimate makes the table spill."""
    n = 600_000
    rng = np.random.default_rng(35)
    k = rng.integers(0, 40_000, n, dtype=np.int64)
    x = rng.integers(-30_000, 30_000, n, dtype=np.int16)
    y = rng.integers(0, 10**9, n, dtype=np.int32)
    f = rng.integers(0, 100, n, dtype=np.int16)
    aggs = [("count_distinct", 1), ("count_distinct", 2), ("count_distinct", 1), ("sum", 2)]
    check([BIGINT, SMALLINT, INTEGER, SMALLINT], [0], aggs, [k, x, y, f], filters=[(3, "<", 70)], est_groups=16,
          chunks=50_000)


def test_all_distinct_single_group_and_topn():
    n = 200_000
    rng = np.random.default_rng(36)
    v = rng.permutation(n).astype(np.int64) - 10**12
    check([INTEGER, BIGINT], [0], [("count_distinct", 1)], [np.zeros(n, np.int32), v])
    k = rng.integers(0, 5000, n, dtype=np.int32)
    w = rng.integers(0, 64, n, dtype=np.int64)
    import oracle
    aggs = [("count_distinct", 1), ("count_star", -1)]
    gpu = run_gpu([INTEGER, BIGINT], [0], aggs, [k, w], topn=(1, False, 10))
    orc = oracle.run_query([INTEGER, BIGINT], [0], aggs, [k, w])
    d = orc["aggs"][0][0]
    order = np.lexsort((orc["keys"][0], -d))[:10]
    assert np.array_equal(gpu["aggs"][0][0], d[order])
    assert np.array_equal(gpu["keys"][0], orc["keys"][0][order])


def test_reset_reuses_pair_sets():
    k, v = datagen.plain(300_000, seed=37)
    aggs = [("count_distinct", 1), ("count_star", -1)]
    g = capi.GroupBy([INTEGER, BIGINT], [0], aggs)
    try:
        outs = []
        for n in (300_000, 120_000, 300_000):
            g.ingest([k[:n], v[:n]])
            g.finalize()
            outs.append(g.result())
            g.reset()
    finally:
        g.close()
    o0, o2 = (np.argsort(o[0][0]) for o in (outs[0], outs[2]))
    for c in range(3):
        assert np.array_equal(outs[0][c][0][o0], outs[2][c][0][o2])
    assert int(outs[1][2][0].sum()) == 120_000


@pytest.mark.parametrize("key_type", [INTEGER, SMALLINT])
def test_narrow_pair_sets(key_type):
    """A non-NULL 16/32-bit key with 16/32-bit distinct columns packs each
    pair into one 8-byte slot: negative keys and values, the pair equal to
    the empty marker (key -1, value -1), two distinct columns (one of them
    nullable), a WHERE clause, and 12 ingests that grow the sets (rehash of
    the 8-byte slots) while the table spills."""
    n = 600_000
    rng = np.random.default_rng(41 + key_type)
    k = rng.integers(-25_000, 25_000, n).astype(np.int16 if key_type == SMALLINT else np.int32)
    if key_type == INTEGER:
        k[-2:] = [-(2**31), 2**31 - 1]
    k[:5000] = -1
    x = rng.integers(-1000, 1000, n).astype(np.int32)
    x[:2500] = -1  # the marker pair
    x[-3:] = [-(2**31), 2**31 - 1, 0]
    y = rng.integers(-30_000, 30_000, n).astype(np.int16)
    yn = rng.random(n) < 0.05
    f = rng.integers(0, 100, n).astype(np.int16)
    aggs = [("count_distinct", 1), ("count_distinct", 2), ("count_star", -1), ("sum", 1)]
    types = [key_type, INTEGER, SMALLINT, SMALLINT]
    check(types, [0], aggs, [k, x, y, f], nulls=[None, None, yn, None], est_groups=16, chunks=49_984)
    check(types, [0], aggs, [k, x, y, f], nulls=[None, None, yn, None], filters=[(3, "<", 70)])


def test_narrow_pair_sets_reset_and_resident():
    """The 8-byte pair sets emptied by reset (same results on the same
    rows) and fed from device-resident columns."""
    rng = np.random.default_rng(44)
    n = 300_000
    k = rng.integers(0, 7000, n).astype(np.int32)
    v = rng.integers(-50, 50, n).astype(np.int32)
    aggs = [("count_distinct", 1), ("count_star", -1)]
    check([INTEGER, INTEGER], [0], aggs, [k, v], device=True)
    g = capi.GroupBy([INTEGER, INTEGER], [0], aggs)
    try:
        outs = []
        for m in (n, 100_000, n):
            g.ingest([k[:m], v[:m]])
            g.finalize()
            outs.append(g.result())
            g.reset()
    finally:
        g.close()
    o0, o2 = (np.argsort(o[0][0]) for o in (outs[0], outs[2]))
    for c in range(3):
        assert np.array_equal(outs[0][c][0][o0], outs[2][c][0][o2])


def test_rejections():
    with pytest.raises(capi.GbError):
        capi.GroupBy([INTEGER, DOUBLE], [0], [("count_distinct", 1)])
    with pytest.raises(capi.GbError):
        capi.GroupBy([INTEGER, BIGINT, BIGINT, BIGINT], [0],
                     [("count_distinct", 1), ("count_distinct", 2), ("count_distinct", 3)])
    with pytest.raises(capi.GbError):
        capi.GroupBy([BIGINT, BIGINT], [0], [("count_distinct", 1)], options={"mode": RADIX})


def test_batch_with_count_distinct():
    """COUNT(DISTINCT) queries in a batch (generic tiles, pair sets emptied
    by the batch's init): 8-byte sets (INTEGER key and value), 16-byte sets
    with NULL keys (a nullable BIGINT key: twin sets), a VARCHAR key, next to
    a plain query; every result against the oracle, on the first run and on
    the graph's replay."""
    import torch
    import oracle
    from util import compare, gpu_to_dict
    rng = np.random.default_rng(61)
    n = 250_000
    k1 = rng.integers(-3000, 3000, n).astype(np.int32)
    v1 = rng.integers(-500, 500, n).astype(np.int32)
    k2 = rng.integers(0, 9000, n).astype(np.int64)
    v2 = rng.integers(0, 10**9, n).astype(np.int64)
    kn2 = rng.random(n) < 0.03
    (offs, data), s3, m3 = datagen.varchar_table(80_000, 2000, seed=62)
    m3 = (m3 % 300).astype(np.int32)
    qs = [
        ([INTEGER, INTEGER], [0], [("count_distinct", 1), ("count_star", -1)], [k1, v1], None, 6000),
        ([BIGINT, BIGINT], [0], [("count_distinct", 1), ("sum", 1)], [k2, v2], [kn2, None], 9000),
        ([VARCHAR, BIGINT, INTEGER], [0], [("count_distinct", 2), ("max", 1)], [(offs, data), s3, m3], None, 2000),
        ([INTEGER, INTEGER], [0], [("count_star", -1), ("sum", 1)], [k1, v1], None, 6000),
    ]

    def dev(c):
        if isinstance(c, tuple):
            return (torch.from_numpy(c[0]).cuda(), torch.from_numpy(c[1]).cuda())
        return torch.from_numpy(np.ascontiguousarray(c)).cuda()

    b = capi.Batch()
    try:
        for types, gcols, aggs, cols, nulls, est in qs:
            d = [dev(c) for c in cols]
            vd = None
            nullable = ()
            if nulls is not None:
                vd = [torch.from_numpy(capi.validity_words(~m).view(np.int64)).cuda() if m is not None else None
                      for m in nulls]
                nullable = [i for i, m in enumerate(nulls) if m is not None]
            rows = len(cols[-1])
            b.add(types, gcols, aggs, d, rows, validity=vd, nullable=nullable, est_groups=est)
        torch.cuda.synchronize()
        for _ in range(2):  # the first run and the graph's replay
            b.run()
            for i, (types, gcols, aggs, cols, nulls, est) in enumerate(qs):
                orc = oracle.run_query(types, gcols, aggs, cols, nulls=nulls)
                out_types = [types[c] for c in gcols] + [
                    oracle.agg_out_type(oracle.AGG_NAMES[kd], types[c] if c >= 0 else 0) for kd, c in aggs]
                compare(gpu_to_dict(b.result(i), len(gcols), out_types), orc)
    finally:
        b.close()
