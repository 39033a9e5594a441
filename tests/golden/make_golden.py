"""Regenerate the golden GROUP BY fixtures (tests/golden/*.npz).

The reference (SlothDB) is not buildable in this project (its GROUP BY lives
inside the whole engine), so the fixtures are the oracle's results — the
oracle is pinned to the reference's own known answers in test_oracle.py —
on small seeded inputs of every workload shape.  Inputs are not stored: they
are regenerated from the seeds by slothdb_gb300.datagen / parquet, and
tests/test_golden.py checks that the oracle and the GPU path both reproduce
the stored results (integers exactly, DOUBLE within 1e-12).

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
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
    for name, (types, groups, aggs, filters, cols) in cases().items():
        res = oracle.run_query(types, groups, aggs, cols, filters=filters)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), allow_pickle=True, **canonical(res, len(groups)))
        print(name, len(res["keys"][0]), "groups")


if __name__ == "__main__":
    main()
