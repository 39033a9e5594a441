"""The oracle pinned to the reference engine itself.

oracle/ref.mk compiles SlothDB from its own sources (no build system of its
own is run) and oracle/ref_harness.cpp runs SQL through Connection::Query on
tables loaded with Connection::CreateTable + Append, or on a Parquet file
through the reference's own reader.  Each test runs the same seeded query
through the reference and through the oracle: group sets and every integer
column equal, DOUBLE SUM/AVG of both within 1e-12 relative of the oracle's
compensated FP64 sum.  The shapes are the benchmark configurations at sizes
the reference finishes in seconds.  Skipped where the reference's sources
are absent (the fixtures they produced are committed under tests/golden/).
"""
import os
import tempfile

import numpy as np
import pytest

import oracle
from oracle import reference
from slothdb_gb300 import datagen
from util import REL_TOL_F64, rel_err

SMALLINT, INTEGER, BIGINT, DOUBLE, VARCHAR = 1, 2, 3, 4, 5

pytestmark = pytest.mark.skipif(reference.reference_source() is None, reason="reference sources not present")


@pytest.fixture(scope="module", autouse=True)
def built(oracle_lib):
    reference.build()


def _key_tuples(keys):
    return list(zip(*[[bytes(x) if isinstance(x, (bytes, np.bytes_)) else int(x) for x in k] for k in keys]))


def check(sql, types, groups, aggs, cols, filters=(), nulls=None, ref_file=None):
    """Reference vs oracle on one query; returns (groups, max DOUBLE rel err
    of the reference, of the oracle)."""
    if ref_file is not None:
        ref, _ = reference.query(sql.format(file=ref_file))
    else:
        ref, _ = reference.query(sql, types, cols, nulls=nulls)
    orc = oracle.run_query(types, groups, aggs, cols, filters=filters, nulls=nulls)
    nk = len(groups)
    rkeys = _key_tuples([ref[i][1] for i in range(nk)])
    okeys = _key_tuples(orc["keys"])
    assert len(rkeys) == len(okeys), "group count: reference %d oracle %d" % (len(rkeys), len(okeys))
    assert len(set(rkeys)) == len(rkeys)
    pos = {k: i for i, k in enumerate(okeys)}
    assert set(rkeys) == set(okeys), "group sets differ"
    perm = np.array([pos[k] for k in rkeys], dtype=np.int64)
    worst_ref = worst_orc = 0.0
    for a, (kind, c) in enumerate(aggs):
        t, rv, rnull = ref[nk + a]
        ov, onull, ocomp = (x[perm] if len(perm) else x for x in orc["aggs"][a])
        assert np.array_equal(rnull, onull), "agg %d: NULL flags differ" % a
        ot = orc["out_types"][nk + a]
        m = ~rnull
        if ot == DOUBLE:
            exact = np.where(ocomp != 0.0, ocomp, ov)
            er = rel_err(rv[m], exact[m])
            eo = rel_err(ov[m], exact[m])
            worst_ref = max(worst_ref, float(er.max()) if er.size else 0.0)
            worst_orc = max(worst_orc, float(eo.max()) if eo.size else 0.0)
        else:
            bad = np.nonzero(rv[m].astype(np.int64) != ov[m].astype(np.int64))[0]
            assert bad.size == 0, "agg %d: %d integer mismatches (ref %r oracle %r)" % (
                a, bad.size, rv[m][bad[0]], ov[m][bad[0]])
    assert worst_ref <= REL_TOL_F64, "reference DOUBLE rel err %.3e" % worst_ref
    assert worst_orc <= REL_TOL_F64, "oracle DOUBLE rel err %.3e" % worst_orc
    return len(rkeys), worst_ref, worst_orc


def test_plain_groupby_1m_rows():
    """1,000,000 rows, 1,024 INT32 keys; COUNT/SUM/MIN/MAX(INT64), bit-exact."""
    k, v = datagen.plain(1_000_000, seed=0)
    ng, _, _ = check("SELECT c0, COUNT(*), SUM(c1), MIN(c1), MAX(c1) FROM t GROUP BY c0", [INTEGER, BIGINT], [0],
                     [("count_star", -1), ("sum", 1), ("min", 1), ("max", 1)], [k, v])
    assert ng == 1024


def test_zipf_groupby_2m_rows():
    """The radix workload's shape at 2M rows (Zipf(1.1) over 400K keys in
    [0, 2^40), DOUBLE ~ N(100, 25)): COUNT bit-exact, SUM/AVG within 1e-12."""
    k, x = datagen.zipf(2_000_000, seed=1, n_values=400_000)
    ng, er, eo = check("SELECT c0, COUNT(*), SUM(c1), AVG(c1) FROM t GROUP BY c0", [BIGINT, DOUBLE], [0],
                       [("count_star", -1), ("sum", 1), ("avg", 1)], [k, x])
    assert ng > 100_000


def test_parquet_filter_groupby_pyarrow_file():
    """The fused Parquet workload's shape written by pyarrow (an independent
    writer: dictionary-encoded INT32 key, INT16 filter column stored INT32,
    PLAIN INT64), read by the reference's own Parquet reader with WHERE f <
    100, against the oracle on the decoded columns."""
    pa = pytest.importorskip("pyarrow")
    pq = pytest.importorskip("pyarrow.parquet")
    from slothdb_gb300 import parquet as gpq
    _, key, f, v = gpq.filter_groupby_file(n_rows=400_000, seed=2, n_dict=65_536, row_group_rows=100_000,
                                           page_rows=16_384)
    tbl = pa.table({"key": pa.array(key, pa.int32()), "f": pa.array(f.astype(np.int16), pa.int16()),
                    "v": pa.array(v, pa.int64())})
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "t.parquet")
        pq.write_table(tbl, path, row_group_size=100_000, compression="NONE", use_dictionary=["key"])
        check("SELECT \"key\", SUM(v), COUNT(*) FROM '{file}' WHERE f < 100 GROUP BY \"key\"",
              [INTEGER, SMALLINT, BIGINT], [0], [("sum", 2), ("count_star", -1)], [key, f.astype(np.int16), v],
              filters=[(1, "<", 100)], ref_file=path)


def test_parquet_filter_groupby_project_writer_file():
    """The same query on the project writer's file (RLE/bit-packed hybrid at
    bit width 16, runs of mean length 4, 1 data page per 16K rows)."""
    from slothdb_gb300 import parquet as gpq
    data, key, f, v = gpq.filter_groupby_file(n_rows=400_000, seed=2, n_dict=65_536, row_group_rows=100_000,
                                              page_rows=16_384)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "t.parquet")
        with open(path, "wb") as fh:
            fh.write(data)
        check("SELECT \"key\", SUM(v), COUNT(*) FROM '{file}' WHERE f < 100 GROUP BY \"key\"",
              [INTEGER, SMALLINT, BIGINT], [0], [("sum", 2), ("count_star", -1)], [key, f.astype(np.int16), v],
              filters=[(1, "<", 100)], ref_file=path)


@pytest.mark.parametrize("codec", ["snappy", "zstd"])
def test_parquet_compressed_pages(codec):
    """The fused workload's shape with SNAPPY or ZSTD pages, written by
    pyarrow and by the project writer (its own compressors), read by the
    reference's Parquet reader (its vendored snappy and zstd) with WHERE f <
    100, against the oracle on the decoded columns."""
    pa = pytest.importorskip("pyarrow")
    pq = pytest.importorskip("pyarrow.parquet")
    from slothdb_gb300 import parquet as gpq
    _, key, f, v = gpq.filter_groupby_file(n_rows=300_000, seed=2, n_dict=65_536, row_group_rows=100_000,
                                           page_rows=16_384)
    cols = [gpq.Column("key", gpq.T_INT32, values=key), gpq.Column("f", gpq.T_INT32, values=f, int16=True),
            gpq.Column("v", gpq.T_INT64, values=v)]
    ours = gpq.write(cols, row_group_rows=100_000, page_rows=16_384, codec=codec)
    tbl = pa.table({"key": pa.array(key, pa.int32()), "f": pa.array(f.astype(np.int16), pa.int16()),
                    "v": pa.array(v, pa.int64())})
    with tempfile.TemporaryDirectory() as d:
        for name in ("pyarrow", "project"):
            path = os.path.join(d, name + ".parquet")
            if name == "pyarrow":
                pq.write_table(tbl, path, row_group_size=100_000, compression=codec.upper(), use_dictionary=["key"])
            else:
                with open(path, "wb") as fh:
                    fh.write(ours)
            check("SELECT \"key\", SUM(v), COUNT(*) FROM '{file}' WHERE f < 100 GROUP BY \"key\"",
                  [INTEGER, SMALLINT, BIGINT], [0], [("sum", 2), ("count_star", -1)], [key, f.astype(np.int16), v],
                  filters=[(1, "<", 100)], ref_file=path)


def test_parquet_optional_columns_with_nulls():
    """pyarrow OPTIONAL columns with NULL values (definition levels), read by
    the reference's own Parquet reader, against the oracle with the same
    NULLs: COUNT(col) skips them, SUM/MIN/MAX of an all-NULL group are NULL."""
    pa = pytest.importorskip("pyarrow")
    pq = pytest.importorskip("pyarrow.parquet")
    rng = np.random.default_rng(33)
    n = 300_000
    key = rng.integers(0, 3000, n).astype(np.int32)
    v = rng.integers(-10**6, 10**6, n, dtype=np.int64)
    x = rng.normal(20, 4, n)
    vn = rng.random(n) < 0.15
    vn[key == 11] = True
    xn = rng.random(n) < 0.05
    tbl = pa.table({"key": pa.array(key, pa.int32()), "v": pa.array(v, pa.int64(), mask=vn),
                    "x": pa.array(x, pa.float64(), mask=xn)})
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "t.parquet")
        pq.write_table(tbl, path, row_group_size=100_000, compression="NONE", data_page_size=64 * 1024)
        check("SELECT \"key\", COUNT(*), COUNT(v), SUM(v), MIN(v), MAX(v), SUM(x), AVG(x) FROM '{file}' GROUP BY \"key\"",
              [INTEGER, BIGINT, DOUBLE], [0],
              [("count_star", -1), ("count", 1), ("sum", 1), ("min", 1), ("max", 1), ("sum", 2), ("avg", 2)],
              [key, v, x], nulls=[None, vn, xn], ref_file=path)


def test_composite_key_500k_rows():
    """(INT32, SMALLINT) key, COUNT/SUM(INT64)/MAX(INT32) — the batched
    workload's composite shape."""
    a, b, s, m = datagen.composite(500_000, 100_000, seed=3)
    check("SELECT c0, c1, COUNT(*), SUM(c2), MAX(c3) FROM t GROUP BY c0, c1", [INTEGER, SMALLINT, BIGINT, INTEGER],
          [0, 1], [("count_star", -1), ("sum", 2), ("max", 3)], [a, b, s, m])


def test_varchar_key_100k_rows():
    """VARCHAR key of 8..32 chars over [a-z0-9] — the batched workload's
    string shape."""
    (offs, data), s, m = datagen.varchar_table(100_000, 20_000, seed=4)
    check("SELECT c0, COUNT(*), SUM(c1), MAX(c2) FROM t GROUP BY c0", [VARCHAR, BIGINT, INTEGER], [0],
          [("count_star", -1), ("sum", 1), ("max", 2)], [(offs, data), s, m])


@pytest.mark.parametrize("op", ["=", "!=", "<", "<=", ">", ">="])
def test_scan_filter_ops(op):
    """Every comparison of the scan filter on an INTEGER and a DOUBLE column.
    (The DOUBLE values have mean 5: a zero-mean sum cancels, and relative
    error against its exact value is then not a meaningful bar — the
    reference's own sums of N(0, 1) values miss 1e-12 relative.)"""
    rng = np.random.default_rng(11)
    n = 200_000
    k = rng.integers(0, 500, n).astype(np.int32)
    f = rng.integers(0, 100, n).astype(np.int32)
    x = rng.normal(5, 1, n)
    sql = "SELECT c0, COUNT(*), SUM(c2), MIN(c1) FROM t WHERE c1 %s 37 AND c2 %s 5.25 GROUP BY c0" % (op, op)
    check(sql, [INTEGER, INTEGER, DOUBLE], [0], [("count_star", -1), ("sum", 2), ("min", 1)], [k, f, x],
          filters=[(1, op, 37), (2, op, 5.25)])


@pytest.mark.parametrize("form", ["in", "str_eq", "str_ne", "like", "not_like", "like_empty", "in_empty_str"])
def test_scan_filter_in_and_varchar_forms(form):
    """The other SimplePredicate forms (physical_planner.cpp:110-135,
    396-496): an integer IN list, VARCHAR = / <> a literal, LIKE '%x%' and
    NOT LIKE '%x%' (LIKE '%%' matches every string)."""
    (offs, data), s_, m = datagen.varchar_table(60_000, 3000, seed=8)
    rng = np.random.default_rng(8)
    k = rng.integers(0, 300, len(s_)).astype(np.int32)
    strs = [bytes(data[offs[i]:offs[i + 1]]) for i in range(len(s_))]
    lit = strs[17]
    cases = {
        "in": ("c0 IN (3, 7, 11, 299, 1000, 7)", [(0, "in", [3, 7, 11, 299, 1000, 7])]),
        "str_eq": ("c1 = '%s'" % lit.decode(), [(1, "=", lit)]),
        "str_ne": ("c1 <> '%s'" % lit.decode(), [(1, "!=", lit)]),
        "like": ("c1 LIKE '%ab%'", [(1, "like", b"ab")]),
        "not_like": ("c1 NOT LIKE '%a%'", [(1, "not like", b"a")]),
        "like_empty": ("c1 LIKE '%%'", [(1, "like", b"")]),
        "in_empty_str": ("c0 IN (5) AND c1 LIKE '%z%'", [(0, "in", [5]), (1, "like", b"z")]),
    }
    where, filters = cases[form]
    check("SELECT c0, COUNT(*), SUM(c2), MAX(c3) FROM t WHERE %s GROUP BY c0" % where,
          [INTEGER, VARCHAR, BIGINT, INTEGER], [0], [("count_star", -1), ("sum", 2), ("max", 3)],
          [k, (offs, data), s_, m], filters=filters)


@pytest.mark.parametrize("order", ["int_str", "str_int"])
def test_int_varchar_pair_key(order):
    """An (INTEGER, VARCHAR) pair key — the shape of RadixCount2ColIntStr
    (radix_count_agg.cpp:767-1358) — in both column orders."""
    (offs, data), s_, m = datagen.varchar_table(80_000, 600, seed=12)
    rng = np.random.default_rng(12)
    k = rng.integers(0, 40, len(s_)).astype(np.int32)
    if order == "int_str":
        sql, groups = "SELECT c0, c1, COUNT(*), SUM(c2), MAX(c3) FROM t GROUP BY c0, c1", [0, 1]
    else:
        sql, groups = "SELECT c1, c0, COUNT(*), SUM(c2), MAX(c3) FROM t GROUP BY c1, c0", [1, 0]
    check(sql, [INTEGER, VARCHAR, BIGINT, INTEGER], groups, [("count_star", -1), ("sum", 2), ("max", 3)],
          [k, (offs, data), s_, m])


def test_nullable_values_and_empty_sums():
    """NULLs in the value columns: COUNT(col) skips them, SUM/AVG/MIN/MAX of
    a group whose values are all NULL are NULL (agg_emit_helpers.cpp).
    One 2,048-row chunk: the reference's in-memory column storage keeps a
    validity mask of one vector's size (src/storage/column_data.cpp:41-44
    writes bit count_ + i into a VECTOR_SIZE-bit mask), so an in-memory table
    with NULLs past row 2,048 corrupts its heap; NULLs at larger sizes are
    pinned through Parquet files instead."""
    rng = np.random.default_rng(12)
    n = 2048
    k = rng.integers(0, 200, n).astype(np.int32)
    v = rng.integers(-1000, 1000, n).astype(np.int64)
    x = rng.normal(5, 2, n)
    vnull = rng.random(n) < 0.3
    vnull[k < 10] = True  # groups whose values are all NULL
    xnull = rng.random(n) < 0.1
    check("SELECT c0, COUNT(*), COUNT(c1), SUM(c1), MIN(c1), MAX(c1), SUM(c2), AVG(c2), MAX(c2) FROM t GROUP BY c0",
          [INTEGER, BIGINT, DOUBLE], [0],
          [("count_star", -1), ("count", 1), ("sum", 1), ("min", 1), ("max", 1), ("sum", 2), ("avg", 2), ("max", 2)],
          [k, v, x], nulls=[None, vnull, xnull])


def test_count_distinct():
    """COUNT(DISTINCT) of integer columns under a composite key and a filter."""
    a, b, s, m = datagen.composite(200_000, 2000, seed=5)
    check("SELECT c0, c1, COUNT(DISTINCT c2), COUNT(DISTINCT c3), COUNT(*) FROM t WHERE c2 >= 500 GROUP BY c0, c1",
          [INTEGER, SMALLINT, BIGINT, INTEGER], [0, 1],
          [("count_distinct", 2), ("count_distinct", 3), ("count_star", -1)],
          [a, b, s % 997, (m % 300).astype(np.int32)], filters=[(2, ">=", 500)])


def test_golden_fixtures_are_reference_results():
    """Every committed golden fixture was made by the reference engine, and
    its DOUBLE values sit within 1e-12 of the compensated sums stored beside
    them."""
    gdir = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    names = [n for n in os.listdir(gdir) if n.endswith(".npz")]
    assert names
    for n in names:
        z = np.load(os.path.join(gdir, n), allow_pickle=True)
        assert str(z["source"]) == "reference", n
        a = 0
        while "agg%d" % a in z:
            comp = z["agg%d_comp" % a]
            m = (comp != 0.0) & ~z["agg%d_null" % a]
            if m.any():
                assert rel_err(z["agg%d" % a][m], comp[m]).max() <= REL_TOL_F64, n
            a += 1


def test_dictionary_histogram_sum_and_count():
    """The reference's ungrouped SUM / COUNT over INT64 dictionary columns
    (its dictionary-histogram fast path, one aggregate per query) equal the
    values' count and sum: a project-writer file and a pyarrow file whose
    dictionary falls back to PLAIN pages."""
    import sys
    from slothdb_gb300 import parquet as gpq
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_pyarrow_files as paf
    rng = np.random.default_rng(92)
    d = rng.integers(-10**6, 10**6, 3000, dtype=np.int64)
    idx = rng.integers(0, len(d), 120_000).astype(np.uint32)
    files = [(gpq.write([gpq.Column("c", gpq.T_INT64, dictionary=d, indices=idx)], row_group_rows=40_000,
                        page_rows=9_000), d[idx]),
             (paf.load("pa_int64_fallback"), paf.int64_column())]
    with tempfile.TemporaryDirectory() as tmp:
        for i, (data, vals) in enumerate(files):
            path = os.path.join(tmp, "f%d.parquet" % i)
            with open(path, "wb") as fh:
                fh.write(data)
            s, _ = reference.query("SELECT SUM(c) FROM '%s'" % path)
            n, _ = reference.query("SELECT COUNT(c) FROM '%s'" % path)
            assert int(s[0][1][0]) == int(vals.astype(object).sum())
            assert int(n[0][1][0]) == len(vals)
