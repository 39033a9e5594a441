"""GPU parity of the single-query fast ingest (integer plans compiled into
registers, narrow shared states, spill records) and of the interpreted
k_ingest it replaces for such plans (option fast_ingest = 0), against the
oracle on the same seeded inputs.  Integer results bit-exact."""
import numpy as np
import pytest

from slothdb_gb300 import capi, datagen
from slothdb_gb300.capi import BIGINT, DOUBLE, INTEGER, SMALLINT
from test_gpu_groupby import HASH, check

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("oracle_lib", "gblib")]

I64 = np.iinfo(np.int64)


def _opts(fast, **kw):
    return dict({"fast_ingest": fast}, **kw)


@pytest.mark.parametrize("fast", [0, 1])
def test_four_ops_with_nulls(fast):
    """COUNT(*), SUM, MIN, MAX and COUNT over a nullable BIGINT column and a
    SMALLINT column (32-bit shared MIN/MAX words), negative values."""
    rng = np.random.default_rng(51)
    n = 700_000
    k = rng.integers(0, 3000, n).astype(np.int32)
    v = rng.integers(-10**12, 10**12, n, dtype=np.int64)
    s = rng.integers(-30000, 30000, n).astype(np.int16)
    vn = rng.random(n) < 0.2
    vn[k == 5] = True  # a group whose values are all NULL
    aggs = [("count_star", -1), ("min", 1), ("max", 1), ("count", 1), ("max", 2)]
    check([INTEGER, BIGINT, SMALLINT], [0], aggs, [k, v, s], nulls=[None, vn, None], est_groups=3000,
          mode=HASH, options=_opts(fast))
    check([INTEGER, BIGINT, SMALLINT], [0], [("count_star", -1), ("min", 2), ("max", 2), ("sum", 2)], [k, v, s],
          est_groups=3000, mode=HASH, options=_opts(fast), device=True)


@pytest.mark.parametrize("fast", [0, 1])
def test_two_predicates_integer_and_double(fast):
    rng = np.random.default_rng(52)
    n = 500_000
    k = rng.integers(0, 1024, n).astype(np.int32)
    f = rng.integers(0, 1000, n).astype(np.int16)
    x = rng.normal(0, 1, n)
    v = rng.integers(0, 10**6, n, dtype=np.int64)
    for filters in ([(1, "<", 300), (2, ">=", -0.25)], [(1, "!=", 7)], [(2, "<", -9.0)]):
        check([INTEGER, SMALLINT, DOUBLE, BIGINT], [0], [("count_star", -1), ("sum", 3), ("max", 3)],
              [k, f, x, v], filters=filters, est_groups=1024, mode=HASH, options=_opts(fast))


@pytest.mark.parametrize("fast", [0, 1])
def test_packed_pair_key_with_null_keys(fast):
    rng = np.random.default_rng(53)
    n = 400_000
    a = rng.integers(-500, 500, n).astype(np.int32)
    b = rng.integers(0, 64, n).astype(np.int16)
    v = rng.integers(0, 10**6, n, dtype=np.int64)
    an, bn = rng.random(n) < 0.02, rng.random(n) < 0.03
    check([INTEGER, SMALLINT, BIGINT], [0, 1], [("count_star", -1), ("sum", 2), ("min", 2)], [a, b, v],
          nulls=[an, bn, None], est_groups=64_000, mode=HASH, options=_opts(fast))


@pytest.mark.parametrize("fast", [0, 1])
def test_spill_records_and_growth(fast):
    """500K distinct keys into a table sized for 16 groups: keys that find no
    slot become spill records, the table grows and the records merge."""
    rng = np.random.default_rng(54)
    n = 1_500_000
    k = rng.integers(0, 500_000, n, dtype=np.int64)
    v = rng.integers(-10**6, 10**6, n, dtype=np.int64)
    check([BIGINT, BIGINT], [0], [("count_star", -1), ("sum", 1), ("max", 1)], [k, v], est_groups=16, mode=HASH,
          options=_opts(fast), chunks=400_000)


@pytest.mark.parametrize("fast", [0, 1])
def test_groups_beyond_the_shared_table(fast):
    """Estimated groups above the shared table: rows fold straight into the
    HBM table (and with the pre-combine forced on, after the warp match)."""
    rng = np.random.default_rng(55)
    n = 1_000_000
    k = rng.integers(0, 200_000, n).astype(np.int32)
    v = rng.integers(0, 10**6, n, dtype=np.int64)
    for pre in (0, 1):
        check([INTEGER, BIGINT], [0], [("count_star", -1), ("sum", 1)], [k, v], est_groups=200_000, mode=HASH,
              options=_opts(fast, precombine=pre), device=True)


@pytest.mark.parametrize("fast", [0, 1])
def test_out_of_band_keys(fast):
    """INT64_MIN (the table's empty marker) and NULL keys fold into their own
    slots; INT64_MAX and 0 stay ordinary keys."""
    rng = np.random.default_rng(56)
    n = 300_000
    k = rng.choice(np.array([I64.min, I64.max, 0, -1, 17], dtype=np.int64), n)
    v = rng.integers(-1000, 1000, n, dtype=np.int64)
    kn = rng.random(n) < 0.1
    check([BIGINT, BIGINT], [0], [("count_star", -1), ("sum", 1), ("min", 1), ("max", 1)], [k, v],
          nulls=[kn, None], mode=HASH, options=_opts(fast))


@pytest.mark.parametrize("fast", [0, 1])
def test_varchar_key(fast):
    (offs, data), s, m = datagen.varchar_table(300_000, 5000, seed=57)
    check([capi.VARCHAR, BIGINT, INTEGER], [0], [("count_star", -1), ("sum", 1), ("max", 2)], [(offs, data), s, m],
          est_groups=5000, mode=HASH, options=_opts(fast))


def test_config1_shape_takes_the_fast_kernel():
    """The 1M-row plain shape runs k_ingest_fast by default and k_ingest when
    the option is off (the kernel names in the profile)."""
    k, v = datagen.plain(1_000_000, seed=0)
    for fast, name in ((1, "k_ingest_fast"), (0, "k_ingest")):
        g = capi.GroupBy([INTEGER, BIGINT], [0], [("count_star", -1), ("sum", 1), ("min", 1), ("max", 1)],
                         est_groups=1024, options={"fast_ingest": fast})
        try:
            g.set_profiling(True)
            g.ingest([k, v], nrows=len(k))
            g.finalize()
            prof = g.profile()
        finally:
            g.close()
        assert name in prof and prof[name][0] >= 1, prof
        assert ("k_ingest_fast" in prof) == bool(fast)
