"""Regenerate the golden GROUP BY fixtures (tests/golden/*.npz).

The fixtures are the REFERENCE ENGINE's own results: oracle/ref.mk builds
SlothDB from its sources and oracle/ref_harness.cpp runs each case's SQL
through Connection::Query (in-memory tables loaded with
Connection::CreateTable + Append; the Parquet case reads the file with the
reference's own reader).  Beside each DOUBLE SUM/AVG column the fixture
keeps the oracle's FP64 compensated sum (``agg<i>_comp``), the tolerance
reference for floating-point results.  Inputs are not stored: they are
regenerated from the seeds by slothdb_gb300.datagen / parquet, and
tests/test_golden.py checks that the oracle and the GPU path both reproduce
the stored results (integers exactly, DOUBLE within 1e-12).

Run from the repository root (needs the reference's sources):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import reference  # noqa: E402
from slothdb_gb300 import datagen  # noqa: E402
from slothdb_gb300 import parquet as pq  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

INTEGER, SMALLINT, BIGINT, DOUBLE, VARCHAR = 2, 1, 3, 4, 5


def cases():
    """name -> (col_types, group_cols, aggs, filters, columns)."""
    out = {}
    k, v = datagen.plain(100_000, seed=0)
    out["plain_100k"] = ([INTEGER, BIGINT], [0], [("count_star", -1), ("sum", 1), ("min", 1), ("max", 1)], [],
                         [k, v])
    k, x = datagen.zipf(20_000, seed=1, n_values=50_000)
    out["zipf_20k"] = ([BIGINT, DOUBLE], [0], [("count_star", -1), ("sum", 1), ("avg", 1)], [], [k, x])
    _, key, f, v = pq.filter_groupby_file(n_rows=200_000, seed=2, n_dict=4096, row_group_rows=50_000, page_rows=8192)
    out["parquet_filter_200k"] = ([INTEGER, SMALLINT, BIGINT], [0], [("sum", 2), ("count_star", -1)], [(1, "<", 100)],
                                  [key, f.astype(np.int16), v])
    a, b, s, m = datagen.composite(60_000, 3000, seed=3)
    out["composite_60k"] = ([INTEGER, SMALLINT, BIGINT, INTEGER], [0, 1], [("count_star", -1), ("sum", 2), ("max", 3)],
                            [], [a, b, s, m])
    (offs, data), s, m = datagen.varchar_table(40_000, 2000, seed=4)
    out["varchar_40k"] = ([VARCHAR, BIGINT, INTEGER], [0], [("count_star", -1), ("sum", 1), ("max", 2)], [],
                          [(offs, data), s, m])
    a, b, s, m = datagen.composite(50_000, 400, seed=5)
    out["distinct_50k"] = ([INTEGER, SMALLINT, BIGINT, INTEGER], [0, 1], [("count_distinct", 2), ("count_distinct", 3),
                                                                          ("count_star", -1)], [(2, ">=", 500)],
                           [a, b, s % 997, (m % 300).astype(np.int32)])
    return out


# each case as the reference's SQL over table t (columns c0, c1, ...); the
# Parquet case reads its file (column names key, f, v)
SQL = {
    "plain_100k": "SELECT c0, COUNT(*), SUM(c1), MIN(c1), MAX(c1) FROM t GROUP BY c0",
    "zipf_20k": "SELECT c0, COUNT(*), SUM(c1), AVG(c1) FROM t GROUP BY c0",
    "parquet_filter_200k": "SELECT \"key\", SUM(v), COUNT(*) FROM '{file}' WHERE f < 100 GROUP BY \"key\"",
    "composite_60k": "SELECT c0, c1, COUNT(*), SUM(c2), MAX(c3) FROM t GROUP BY c0, c1",
    "varchar_40k": "SELECT c0, COUNT(*), SUM(c1), MAX(c2) FROM t GROUP BY c0",
    "distinct_50k": "SELECT c0, c1, COUNT(DISTINCT c2), COUNT(DISTINCT c3), COUNT(*) FROM t WHERE c2 >= 500 "
                    "GROUP BY c0, c1",
}


def parquet_case_file():
    """The Parquet case's file bytes (the project writer's file)."""
    data, _, _, _ = pq.filter_groupby_file(n_rows=200_000, seed=2, n_dict=4096, row_group_rows=50_000,
                                           page_rows=8192)
    return data


def reference_result(name, types, groups, aggs, filters, cols):
    """The reference engine's result for one case, in the oracle's result
    shape; DOUBLE SUM/AVG carry the oracle's compensated sums beside it."""
    import tempfile
    orc = oracle.run_query(types, groups, aggs, cols, filters=filters)
    if name.startswith("parquet"):
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "case.parquet")
            with open(path, "wb") as f:
                f.write(parquet_case_file())
            ref, _ = reference.query(SQL[name].format(file=path))
    else:
        ref, _ = reference.query(SQL[name], types, cols)
    nk = len(groups)
    keys, key_null = [], []
    for i in range(nk):
        t, vals, null = ref[i]
        if types[groups[i]] == VARCHAR:
            keys.append(vals)
        else:
            keys.append(vals.astype(oracle.NP_TYPES[types[groups[i]]]))
        key_null.append(null)
    # the oracle's compensated sums, matched to the reference's rows by key
    comp_of = {}
    okeys = list(zip(*[[bytes(x) if isinstance(x, (bytes, np.bytes_)) else int(x) for x in k]
                       for k in orc["keys"]]))
    for a in range(len(aggs)):
        comp_of[a] = dict(zip(okeys, orc["aggs"][a][2]))
    rkeys = list(zip(*[[bytes(x) if isinstance(x, (bytes, np.bytes_)) else int(x) for x in k] for k in keys]))
    out_aggs = []
    for a, (kind, c) in enumerate(aggs):
        t, vals, null = ref[nk + a]
        ot = oracle.agg_out_type(oracle.AGG_NAMES[kind], types[c] if c >= 0 else 0)
        vals = vals.astype(np.float64) if ot == DOUBLE else vals.astype(oracle.NP_TYPES[ot])
        comp = np.array([comp_of[a].get(k, 0.0) for k in rkeys], dtype=np.float64)
        out_aggs.append((vals, null, comp))
    return dict(keys=keys, key_null=key_null, aggs=out_aggs)


def canonical(res, n_keys):
    """Oracle result → rows sorted by key (NULL keys first)."""
    keys = res["keys"]
    order = np.lexsort([np.array([str(x) for x in keys[i]]) if keys[i].dtype == object else keys[i]
                        for i in reversed(range(n_keys))])
    out = {}
    for i in range(n_keys):
        col = keys[i][order]
        out["key%d" % i] = np.array([bytes(x) for x in col], dtype=object) if col.dtype == object else col
        out["key%d_null" % i] = res["key_null"][i][order]
    for a, (vals, nulls, comp) in enumerate(res["aggs"]):
        out["agg%d" % a] = vals[order]
        out["agg%d_null" % a] = nulls[order]
        out["agg%d_comp" % a] = comp[order]
    return out


def main():
    oracle.load()
    if reference.build() is None:
        raise SystemExit("the reference's sources are needed to regenerate the fixtures")
    for name, (types, groups, aggs, filters, cols) in cases().items():
        res = reference_result(name, types, groups, aggs, filters, cols)
        fx = canonical(res, len(groups))
        fx["source"] = np.array("reference")
        np.savez_compressed(os.path.join(OUT, name + ".npz"), allow_pickle=True, **fx)
        print(name, len(res["keys"][0]), "groups (reference)")


if __name__ == "__main__":
    main()
