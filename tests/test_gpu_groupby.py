"""GPU parity: the CUDA GROUP BY (through the C ABI) against the oracle on
identical seeded inputs.  Integer results bit-exact; DOUBLE SUM/AVG within
1e-12 relative error of the FP64 compensated sum."""
import numpy as np
import pytest

import oracle
from slothdb_gb300 import capi, datagen
from slothdb_gb300.capi import BIGINT, DOUBLE, INTEGER, SMALLINT
from util import compare, gpu_to_dict

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("oracle_lib", "gblib")]

REL_TOL = 1e-12


def run_gpu(col_types, group_cols, aggs, cols, filters=(), nulls=None, est_groups=0, device=False,
            chunks=None, topn=None, mode=0, options=None):
    nullable = [i for i, m in enumerate(nulls or []) if m is not None]
    opts = dict({"mode": mode} if mode else {}, **(options or {}))
    g = capi.GroupBy(col_types, group_cols, aggs, filters=filters, nullable=nullable, est_groups=est_groups,
                     options=opts or None)
    if mode == 2:
        assert g.mode() == 1
    try:
        if topn:
            g.set_topn(*topn)
        n = (len(cols[0][0]) - 1) if col_types[0] == capi.VARCHAR else len(cols[0])
        validity = None
        if nulls is not None:
            validity = [capi.validity_words(~m) if m is not None else None for m in nulls]
        bounds = [(0, n)] if not chunks else [(i, min(n, i + chunks)) for i in range(0, max(n, 1), chunks)]
        for lo, hi in bounds:
            if hi <= lo and n > 0:
                continue
            part = [_slice(c, t, lo, hi) for c, t in zip(cols, col_types)]
            vpart = None
            if validity is not None:
                assert lo % 64 == 0
                vpart = [v[lo // 64:(hi + 63) // 64] if v is not None else None for v in validity]
            if device:
                import torch
                tens = [(torch.from_numpy(p[0]).cuda(), torch.from_numpy(p[1]).cuda()) if t == capi.VARCHAR
                        else torch.from_numpy(np.ascontiguousarray(p)).cuda() for p, t in zip(part, col_types)]
                vt = None
                if vpart is not None:
                    vt = [torch.from_numpy(v.view(np.int64)).cuda() if v is not None else None for v in vpart]
                torch.cuda.synchronize()
                g.ingest(tens, nrows=hi - lo, validity=vt, device=True)
                torch.cuda.synchronize()
            else:
                g.ingest(part, nrows=hi - lo, validity=vpart)
        g.finalize()
        res = g.result()
        launches = g.launches()
    finally:
        g.close()
    n_keys = len(group_cols)
    out_types = [col_types[c] for c in group_cols] + [oracle.agg_out_type(oracle.AGG_NAMES[k] if isinstance(k, str)
                                                                          else k, col_types[c] if c >= 0 else 0)
                                                      for k, c in aggs]
    d = gpu_to_dict(res, n_keys, out_types)
    d["launches"] = launches
    return d


def _slice(c, t, lo, hi):
    if t == capi.VARCHAR:
        offs, data = c
        o = offs[lo:hi + 1]
        return (np.ascontiguousarray(o - o[0]), np.ascontiguousarray(data[o[0]:o[-1]]) if o[-1] > o[0]
                else np.zeros(1, np.uint8))
    return c[lo:hi]


def check(col_types, group_cols, aggs, cols, **kw):
    nulls = kw.get("nulls")
    filters = kw.get("filters", ())
    orc = oracle.run_query(col_types, group_cols, aggs, cols, filters=filters, nulls=nulls)
    gpu = run_gpu(col_types, group_cols, aggs, cols, **kw)
    assert gpu["launches"] > 0
    return compare(gpu, orc, rel_tol=REL_TOL), gpu, orc


PLAIN_AGGS = [("count_star", -1), ("sum", 1), ("min", 1), ("max", 1)]
HASH, RADIX = 1, 2


@pytest.mark.parametrize("mode", [HASH, RADIX])
def test_plain_workload_1m_host_and_device(mode):
    k, v = datagen.plain(1_000_000, seed=0)
    check([INTEGER, BIGINT], [0], PLAIN_AGGS, [k, v], mode=mode)
    check([INTEGER, BIGINT], [0], PLAIN_AGGS, [k, v], device=True, mode=mode)


@pytest.mark.parametrize("mode", [HASH, RADIX])
@pytest.mark.parametrize("n", [0, 1, 31, 32, 33, 2047, 2048, 2049, 122_880 + 7])
def test_ragged_sizes(n, mode):
    k, v = datagen.plain(max(n, 1), seed=11, n_keys=97)
    k, v = k[:n], v[:n]
    if n == 0:
        gpu = run_gpu([INTEGER, BIGINT], [0], PLAIN_AGGS, [k, v], mode=mode)
        assert len(gpu["keys"][0]) == 0
        return
    check([INTEGER, BIGINT], [0], PLAIN_AGGS, [k, v], mode=mode)


@pytest.mark.parametrize("mode", [HASH, RADIX])
def test_all_distinct_and_single_group(mode):
    n = 300_000
    rng = np.random.default_rng(3)
    k = rng.permutation(n).astype(np.int64) * 7919 - 10**12
    v = rng.integers(-10**9, 10**9, n, dtype=np.int64)
    check([BIGINT, BIGINT], [0], PLAIN_AGGS, [k, v], est_groups=n, mode=mode)
    check([BIGINT, BIGINT], [0], PLAIN_AGGS, [np.full(n, 42, np.int64), v], mode=mode)


def test_table_growth_from_tiny_estimate():
    """500K distinct keys into a table sized for 16 groups: spill records,
    rehash and replay must lose nothing."""
    n = 1_500_000
    rng = np.random.default_rng(4)
    k = rng.integers(0, 500_000, n, dtype=np.int64)
    v = rng.integers(0, 10**6, n, dtype=np.int64)
    check([BIGINT, BIGINT], [0], PLAIN_AGGS, [k, v], est_groups=16)


def test_radix_partition_growth_over_many_chunks():
    """The first chunk sizes the partitions; later chunks overflow them, so
    the overflow list, partition regrowth and drain must keep every row."""
    n = 1_500_000
    rng = np.random.default_rng(14)
    k = rng.integers(0, 400_000, n, dtype=np.int64)
    v = rng.integers(0, 10**6, n, dtype=np.int64)
    check([BIGINT, BIGINT], [0], PLAIN_AGGS, [k, v], est_groups=16, chunks=65536, mode=RADIX)


@pytest.mark.parametrize("mode", [HASH, RADIX])
def test_zipf_double_sum_avg_tolerance(mode):
    k, x = datagen.zipf(2_000_000, seed=1, n_values=400_000)
    err, gpu, orc = check([BIGINT, DOUBLE], [0], [("count_star", -1), ("sum", 1), ("avg", 1)], [k, x],
                          est_groups=400_000, mode=mode)
    assert err <= REL_TOL


@pytest.mark.parametrize("pre", [0, 1])
@pytest.mark.parametrize("vtype", [DOUBLE, BIGINT])
def test_radix_partition_pass_with_and_without_precombine(vtype, pre):
    """The per-partition pass folds repeated tail keys with the warp
    pre-combine and tuple by tuple (DOUBLE SUM words fold in L2, BIGINT SUM
    words in shared memory); a WHERE clause takes the generic partition pass."""
    k, x = datagen.zipf(2_000_000, seed=5, n_values=400_000)
    if vtype == BIGINT:
        # per-group sums stay below 2^53, where the reference's double
        # accumulation is exact
        x = np.random.default_rng(5).integers(-10**6, 10**6, len(k), dtype=np.int64)
    aggs = [("count_star", -1), ("sum", 1), ("avg", 1)]
    opts = {"radix_precombine": pre}
    err, _, _ = check([BIGINT, vtype], [0], aggs, [k, x], est_groups=400_000, mode=RADIX, options=opts)
    assert err <= REL_TOL
    err, _, _ = check([BIGINT, vtype], [0], aggs, [k, x], est_groups=400_000, mode=RADIX, options=opts,
                      filters=[(1, ">", 0)], device=True)
    assert err <= REL_TOL


@pytest.mark.parametrize("vtype", [DOUBLE, BIGINT])
def test_radix_hot_table_full_key_range(vtype):
    """The specialised partition pass on Zipf ranks mapped to keys across the
    whole int64 range: INT64_MIN (also the hot table's empty marker) and
    INT64_MAX among the hottest keys."""
    rng = np.random.default_rng(21)
    n = 1_500_000
    ranks = np.minimum(rng.zipf(1.2, n), 300_000) - 1
    vals = rng.integers(np.iinfo(np.int64).min, np.iinfo(np.int64).max, 300_000, dtype=np.int64)
    vals[:4] = [np.iinfo(np.int64).min, np.iinfo(np.int64).max, -1, 0]
    k = vals[ranks]
    x = rng.normal(50, 10, n) if vtype == DOUBLE else rng.integers(-10**6, 10**6, n, dtype=np.int64)
    aggs = [("count_star", -1), ("sum", 1)]
    err, _, _ = check([BIGINT, vtype], [0], aggs, [k, x], est_groups=300_000, mode=RADIX, device=True)
    assert err <= REL_TOL


@pytest.mark.parametrize("vtype", [DOUBLE, BIGINT])
def test_radix_predicate_on_the_value_column(vtype):
    """The specialised partition pass with one compare on the value column
    (the served Zipf shape), and a radix handle whose predicates are
    replaced after reset: none, on the value column, on another column
    (the generic pass) and back, each against the oracle."""
    import torch
    k, x = datagen.zipf(1_500_000, seed=8, n_values=300_000)
    if vtype == BIGINT:
        x = np.random.default_rng(8).integers(-10**6, 10**6, len(k), dtype=np.int64)
    f = np.random.default_rng(9).integers(0, 1000, len(k)).astype(np.int32)
    thr = 95.0 if vtype == DOUBLE else 0
    aggs = [("count_star", -1), ("sum", 1), ("avg", 1)]
    types = [BIGINT, vtype, INTEGER]
    for op in ("<", ">=", "!="):
        err, _, _ = check(types, [0], aggs, [k, x, f], est_groups=300_000, mode=RADIX, filters=[(1, op, thr)],
                          device=True)
        assert err <= REL_TOL
    dk, dx, df = (torch.from_numpy(a).cuda() for a in (k, x, f))
    g = capi.GroupBy(types, [0], aggs, est_groups=300_000, options={"mode": RADIX})
    try:
        for filters in ([], [(1, "<", thr)], [(2, "<", 300)], [(1, ">", thr)], []):
            g.reset()
            g.set_filters(filters)
            g.ingest([dk, dx, df], nrows=len(k), device=True)
            g.finalize()
            gpu = gpu_to_dict(g.result(), 1, [BIGINT, BIGINT, vtype if vtype == DOUBLE else BIGINT, DOUBLE])
            orc = oracle.run_query(types, [0], aggs, [k, x, f], filters=filters)
            assert compare(gpu, orc, rel_tol=REL_TOL) <= REL_TOL
    finally:
        g.close()


@pytest.mark.parametrize("n_keys", [1, 700])
def test_radix_specialised_pass_all_keys_hot(n_keys):
    """The specialised partition pass (one BIGINT key, one DOUBLE SUM) when
    every key lands in the hot table: no row is partitioned, so the
    per-partition pass runs on empty partitions and the result comes from
    the hot emit alone (with and without a TopN on it)."""
    rng = np.random.default_rng(23)
    n = 1_000_000
    k = rng.integers(0, n_keys, n).astype(np.int64) * 1_000_003 - 5
    x = rng.normal(50, 10, n)
    aggs = [("count_star", -1), ("sum", 1)]
    err, _, _ = check([BIGINT, DOUBLE], [0], aggs, [k, x], est_groups=2_000_000, mode=RADIX, device=True)
    assert err <= REL_TOL
    gpu = run_gpu([BIGINT, DOUBLE], [0], aggs, [k, x], topn=(1, False, 5), est_groups=2_000_000, mode=RADIX,
                  device=True)
    orc = oracle.run_query([BIGINT, DOUBLE], [0], aggs, [k, x])
    order = np.lexsort((orc["keys"][0], -orc["aggs"][0][0]))[:5]
    assert np.array_equal(gpu["keys"][0], orc["keys"][0][order])
    assert np.array_equal(gpu["aggs"][0][0], orc["aggs"][0][0][order])


@pytest.mark.parametrize("mode", [HASH, RADIX])
def test_zipf_topn_count_desc(mode):
    k, x = datagen.zipf(2_000_000, seed=1, n_values=400_000)
    aggs = [("count_star", -1), ("sum", 1), ("avg", 1)]
    gpu = run_gpu([BIGINT, DOUBLE], [0], aggs, [k, x], topn=(1, False, 10), est_groups=400_000, mode=mode)
    orc = oracle.run_query([BIGINT, DOUBLE], [0], aggs, [k, x])
    cnt = orc["aggs"][0][0]
    order = np.lexsort((orc["keys"][0], -cnt))[:10]
    assert np.array_equal(gpu["keys"][0], orc["keys"][0][order])
    assert np.array_equal(gpu["aggs"][0][0], cnt[order])
    ref_sum = orc["aggs"][1][2][order]
    assert np.max(np.abs(gpu["aggs"][1][0] - ref_sum) / np.abs(ref_sum)) <= REL_TOL


def test_topn_ties_key_ascending_and_asc_order():
    # the reference's ORDER BY cnt DESC, dept tie case (test_aggregation.cpp:196-212) on int keys
    k = np.array([7, 7, 3, 3, 9], dtype=np.int32)
    v = np.arange(5, dtype=np.int64)
    gpu = run_gpu([INTEGER, BIGINT], [0], [("count_star", -1)], [k, v], topn=(1, False, 3))
    assert gpu["keys"][0].tolist() == [3, 7, 9]
    assert gpu["aggs"][0][0].tolist() == [2, 2, 1]
    gpu = run_gpu([INTEGER, BIGINT], [0], [("sum", 1)], [k, v], topn=(1, True, 2))
    assert gpu["keys"][0].tolist() == [7, 9]


def _expected_topn(orc, col, asc, K):
    """Rows of the oracle's result in TopN order: the order column's value
    (NULL first ascending, last descending), then the key ascending."""
    n = orc["n_groups"]
    vals, nul, _ = orc["aggs"][col - 1]
    keys = orc["keys"][0].astype(np.int64)
    big = 1 << 64

    def code(i):
        prim = 0 if nul[i] else (int(vals[i]) + (1 << 63))
        return (prim if asc else (big - 1 - prim), int(keys[i]))
    return sorted(range(n), key=code)[:K]


@pytest.mark.parametrize("small", [0, 1])
def test_topn_limits_orders_and_nulls(small):
    """TopN for K from 1 to 64 (warp-register lists up to 32, the
    shared-memory select beyond, and with the small path switched off) on
    COUNT DESC with many ties, MIN ASC with NULL results, and a result with
    fewer groups than K that holds a NULL order value and the key INT64_MAX."""
    rng = np.random.default_rng(12)
    n = 400_000
    k = rng.integers(0, 30_000, n).astype(np.int64)
    v = rng.integers(-1000, 1000, n, dtype=np.int64)
    vn = rng.random(n) < 0.3
    vn[k % 97 == 0] = True  # groups whose values are all NULL
    aggs = [("count_star", -1), ("min", 1)]
    orc = oracle.run_query([BIGINT, BIGINT], [0], aggs, [k, v], nulls=[None, vn])
    for K in (1, 5, 10, 32, 33, 64):
        for col, asc in ((1, False), (2, True), (2, False)):
            gpu = run_gpu([BIGINT, BIGINT], [0], aggs, [k, v], nulls=[None, vn], topn=(col, asc, K),
                          options={"topn_small": small})
            want = _expected_topn(orc, col, asc, K)
            assert gpu["keys"][0].astype(np.int64).tolist() == orc["keys"][0][want].astype(np.int64).tolist(), (K, col)
    kk = np.array([np.iinfo(np.int64).max, 3, 3, 5], dtype=np.int64)
    vv = np.array([1, 2, 3, 4], dtype=np.int64)
    vnn = np.array([True, False, False, False])
    orc = oracle.run_query([BIGINT, BIGINT], [0], aggs, [kk, vv], nulls=[None, vnn])
    for K in (3, 10):
        gpu = run_gpu([BIGINT, BIGINT], [0], aggs, [kk, vv], nulls=[None, vnn], topn=(2, False, K),
                      options={"topn_small": small})
        want = _expected_topn(orc, 2, False, K)
        assert gpu["keys"][0].astype(np.int64).tolist() == orc["keys"][0][want].astype(np.int64).tolist()


def test_nulls_in_keys_and_values():
    n = 200_000
    rng = np.random.default_rng(6)
    k = rng.integers(0, 1000, n, dtype=np.int32)
    v = rng.integers(-10**6, 10**6, n, dtype=np.int64)
    kn = rng.random(n) < 0.01
    vn = rng.random(n) < 0.2
    # a group whose values are all NULL (SUM/MIN/MAX → NULL)
    k[:50] = 5000
    vn[:50] = True
    kn[:50] = False
    check([INTEGER, BIGINT], [0], [("count_star", -1), ("count", 1), ("sum", 1), ("avg", 1), ("min", 1), ("max", 1)],
          [k, v], nulls=[kn, vn], chunks=65536)


@pytest.mark.parametrize("mode", [HASH, RADIX])
def test_composite_int32_int16_key_batched_shape(mode):
    a, b, s, m = datagen.composite(400_000, 50_000, seed=3)
    check([INTEGER, SMALLINT, BIGINT, INTEGER], [0, 1], [("count_star", -1), ("sum", 2), ("max", 3)], [a, b, s, m],
          mode=mode)


def test_composite_with_nulls_and_wide_pair():
    n = 100_000
    rng = np.random.default_rng(8)
    a = rng.integers(-50, 50, n, dtype=np.int32)
    b = rng.integers(-3, 3, n, dtype=np.int16)
    an = rng.random(n) < 0.05
    bn = rng.random(n) < 0.05
    s = rng.integers(0, 100, n, dtype=np.int64)
    check([INTEGER, SMALLINT, BIGINT], [0, 1], [("count_star", -1), ("sum", 2)], [a, b, s], nulls=[an, bn, None])
    c = rng.integers(-(2**31), 2**31 - 1, n, dtype=np.int32)
    d = rng.integers(-5, 5, n, dtype=np.int32)
    check([INTEGER, INTEGER, BIGINT], [0, 1], [("count_star", -1), ("min", 2)], [c, d, s])


@pytest.mark.parametrize("mode", [HASH, RADIX])
def test_filters_int_and_double(mode):
    n = 500_000
    rng = np.random.default_rng(9)
    k = rng.integers(0, 5000, n, dtype=np.int32)
    f = rng.integers(0, 1000, n, dtype=np.int16)
    v = rng.integers(-10**9, 10**9 + 1, n, dtype=np.int64)
    x = rng.normal(0, 1, n)
    check([INTEGER, SMALLINT, BIGINT, DOUBLE], [0], [("sum", 2), ("count_star", -1)], [k, f, v, x],
          filters=[(1, "<", 100)], mode=mode)
    check([INTEGER, SMALLINT, BIGINT, DOUBLE], [0], [("sum", 2), ("min", 3), ("max", 3)], [k, f, v, x],
          filters=[(3, ">=", 0.5), (1, "!=", 7)], mode=mode)


@pytest.mark.parametrize("mode", [HASH, RADIX])
def test_special_key_values_and_smallint(mode):
    k = np.array([np.iinfo(np.int64).min, 0, -1, np.iinfo(np.int64).max, np.iinfo(np.int64).min, -1], dtype=np.int64)
    v = np.arange(6, dtype=np.int64)
    check([BIGINT, BIGINT], [0], PLAIN_AGGS, [k, v], mode=mode)
    ks = np.array([-32768, 32767, 0, -32768], dtype=np.int16)
    vd = np.array([-1.5, 2.25, -0.0, 7.0])
    check([SMALLINT, DOUBLE], [0], [("min", 1), ("max", 1), ("sum", 1), ("count", 1)], [ks, vd], mode=mode)


def test_radix_null_keys_and_mode_rejection():
    n = 100_000
    rng = np.random.default_rng(15)
    k = rng.integers(0, 20_000, n, dtype=np.int64)
    kn = rng.random(n) < 0.02
    v = rng.integers(0, 100, n, dtype=np.int64)
    check([BIGINT, BIGINT], [0], PLAIN_AGGS, [k, v], nulls=[kn, None], mode=RADIX)
    with pytest.raises(capi.GbError):
        capi.GroupBy([BIGINT, BIGINT], [0], PLAIN_AGGS, nullable=[1], options={"mode": RADIX})


def test_many_chunks_accumulate():
    k, v = datagen.plain(100_000, seed=12)
    check([INTEGER, BIGINT], [0], PLAIN_AGGS, [k, v], chunks=2048)


def test_engine_hash_aggregate_known_answer(gblib):
    import ctypes as C
    keys = np.array([1, 2, 1, 2, 1], dtype=np.int32)
    vals = np.array([10, 20, 30, 40, 50], dtype=np.int32)
    ok = np.zeros(8, np.int32)
    os_ = np.zeros(8, np.int64)
    oc = np.zeros(8, np.int64)
    n = C.c_uint64()
    capi.check(gblib.gb_engine_hash_aggregate(keys.ctypes.data, vals.ctypes.data, 5, ok.ctypes.data,
                                              os_.ctypes.data, oc.ctypes.data, 8, C.byref(n)))
    got = {int(ok[i]): (int(os_[i]), int(oc[i])) for i in range(n.value)}
    assert got == {1: (90, 3), 2: (60, 2)}


def test_reset_reuses_handle():
    k, v = datagen.plain(50_000, seed=13)
    g = capi.GroupBy([INTEGER, BIGINT], [0], PLAIN_AGGS)
    try:
        outs = []
        for _ in range(2):
            g.ingest([k, v])
            g.finalize()
            outs.append(g.result())
            g.reset()
        o0, o1 = (np.argsort(o[0][0]) for o in outs)
        for c in range(5):
            assert np.array_equal(outs[0][c][0][o0], outs[1][c][0][o1])
    finally:
        g.close()


VARCHAR = capi.VARCHAR


@pytest.mark.parametrize("device", [False, True])
def test_varchar_key_batched_shape(device):
    """VARCHAR key of length 8..32 over [a-z0-9]: COUNT(*), SUM(INT64), MAX(INT32)."""
    (offs, data), s, m = datagen.varchar_table(300_000, 20_000, seed=31)
    check([VARCHAR, BIGINT, INTEGER], [0], [("count_star", -1), ("sum", 1), ("max", 2)], [(offs, data), s, m],
          device=device, est_groups=1000)


def test_varchar_nulls_empty_and_long_strings():
    rng = np.random.default_rng(32)
    pool = [b"", b"a", b"ab", b"x" * 12, b"x" * 13, b"prefix-shared-1", b"prefix-shared-2",
            bytes(rng.integers(0, 256, 300, dtype=np.uint8))]
    n = 50_000
    pick = rng.integers(0, len(pool), n)
    strs = [pool[i] for i in pick]
    lens = np.array([len(x) for x in strs], dtype=np.int64)
    offs = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(lens, out=offs[1:])
    data = np.frombuffer(b"".join(strs), dtype=np.uint8)
    kn = rng.random(n) < 0.05
    v = rng.integers(0, 100, n, dtype=np.int64)
    check([VARCHAR, BIGINT], [0], [("count_star", -1), ("sum", 1)], [(offs, data), v], nulls=[kn, None],
          chunks=8192)


def test_varchar_dictionary_growth():
    """100K distinct strings into a dictionary sized for 16: retries + rehash."""
    (offs, data), s, m = datagen.varchar_table(400_000, 100_000, seed=33)
    check([VARCHAR, BIGINT, INTEGER], [0], [("count_star", -1), ("sum", 1)], [(offs, data), s, m], est_groups=16)


@pytest.mark.parametrize("form", ["in", "str_eq", "str_ne", "like", "not_like", "like_empty", "in_and_like"])
@pytest.mark.parametrize("device", [False, True])
def test_in_list_and_varchar_predicates(form, device):
    """The IN-list and VARCHAR predicate forms of the scan filter (=, <>,
    LIKE '%x%', NOT LIKE) on a non-key VARCHAR column, and on a VARCHAR key."""
    (offs, data), s, m = datagen.varchar_table(120_000, 4000, seed=9)
    rng = np.random.default_rng(9)
    k = rng.integers(0, 300, len(s)).astype(np.int32)
    lit = bytes(data[offs[17]:offs[18]])
    filters = {"in": [(0, "in", [3, 7, 11, 299, 1000, 7, -4])], "str_eq": [(1, "=", lit)],
               "str_ne": [(1, "!=", lit)], "like": [(1, "like", b"ab")], "not_like": [(1, "not like", b"a")],
               "like_empty": [(1, "like", b"")], "in_and_like": [(0, "in", [5, 6]), (1, "like", b"z")]}[form]
    types = [INTEGER, capi.VARCHAR, BIGINT, INTEGER]
    aggs = [("count_star", -1), ("sum", 2), ("max", 3)]
    check(types, [0], aggs, [k, (offs, data), s, m], filters=filters, device=device)
    # the same predicates with the VARCHAR column as the group key
    check(types, [1], aggs, [k, (offs, data), s, m], filters=filters, device=device)


def test_in_list_radix_and_nulls():
    """IN on the radix path (generic partition pass) and NULLs in the IN
    column (a NULL row never passes)."""
    k, x = datagen.zipf(1_000_000, seed=5, n_values=300_000)
    rng = np.random.default_rng(10)
    tag = rng.integers(0, 50, len(k)).astype(np.int16)
    tn = rng.random(len(k)) < 0.05
    aggs = [("count_star", -1), ("sum", 1)]
    check([BIGINT, DOUBLE, SMALLINT], [0], aggs, [k, x, tag], filters=[(2, "in", [1, 2, 3, 40])],
          est_groups=300_000, mode=RADIX, nulls=[None, None, tn])
    check([BIGINT, DOUBLE, SMALLINT], [0], aggs, [k, x, tag], filters=[(2, "in", [])], mode=HASH)


@pytest.mark.parametrize("other", [INTEGER, SMALLINT])
@pytest.mark.parametrize("order", ["int_str", "str_int"])
@pytest.mark.parametrize("device", [False, True])
def test_int_varchar_pair_key(other, order, device):
    """(INTEGER or SMALLINT, VARCHAR) pair keys: the string becomes a 32-bit
    dictionary id packed beside the integer; NULL strings form their own
    groups, and with a SMALLINT partner NULL integers too."""
    (offs, data), s, m = datagen.varchar_table(150_000, 2000, seed=13)
    rng = np.random.default_rng(13)
    k = rng.integers(-60, 60, len(s)).astype(np.int32 if other == INTEGER else np.int16)
    sn = rng.random(len(s)) < 0.02
    kn = (rng.random(len(s)) < 0.03) if other == SMALLINT else None
    groups = [0, 1] if order == "int_str" else [1, 0]
    types = [other, capi.VARCHAR, BIGINT, INTEGER]
    aggs = [("count_star", -1), ("sum", 2), ("max", 3)]
    check(types, groups, aggs, [k, (offs, data), s, m], nulls=[kn, sn, None, None], device=device,
          filters=[(1, "not like", b"q")])


def test_int_varchar_pair_key_radix():
    (offs, data), s, m = datagen.varchar_table(400_000, 150_000, seed=14)
    k = np.random.default_rng(14).integers(0, 8, len(s)).astype(np.int16)
    check([SMALLINT, capi.VARCHAR, BIGINT, INTEGER], [0, 1], [("count_star", -1), ("sum", 2)],
          [k, (offs, data), s, m], est_groups=1_200_000, mode=RADIX)
