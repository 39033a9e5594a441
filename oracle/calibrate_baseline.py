"""How fast the oracle port runs against the reference engine itself on the
same inputs and host — TEST INFRASTRUCTURE ONLY.

The GPU host has neither the reference's sources nor an x86 build of it, so
the benchmark's CPU baseline there is the oracle port (oracle/gb_oracle.c)
run at the reference's own thread counts.  This script, run where the
reference builds (oracle/ref.mk), times both on the workload shapes and
prints one row per shape: reference ms (``Connection::Query`` around the
materialised result, median of 3), port ms at 1 thread and at every host
thread (median of 3), and the ratio reference / port.  A ratio above 1 means
the port is faster than the reference, so a GPU/port speed-up understates
the GPU/reference speed-up by that factor.

    python oracle/calibrate_baseline.py
"""
from __future__ import annotations

import json
import os
import statistics
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from oracle import reference  # noqa: E402
from slothdb_gb300 import datagen  # noqa: E402


def _port_ms(types, group_cols, aggs, cols, threads, filters=()):
    ts = []
    for _ in range(3):
        t = time.perf_counter()
        oracle.run_query(types, group_cols, aggs, cols, filters=filters, nthreads=threads)
        ts.append((time.perf_counter() - t) * 1e3)
    return statistics.median(ts)


def shapes():
    k, v = datagen.plain(1_000_000, seed=0)
    yield ("plain 1M rows, 1,024 INT32 keys, COUNT/SUM/MIN/MAX",
           "SELECT c0, COUNT(*), SUM(c1), MIN(c1), MAX(c1) FROM t GROUP BY c0",
           [2, 3], [0], [("count_star", -1), ("sum", 1), ("min", 1), ("max", 1)], [k, v])
    for rows, nv in ((2_000_000, 400_000), (10_000_000, 2_000_000)):
        k, x = datagen.zipf(rows, seed=1, n_values=nv)
        yield ("Zipf(1.1) %dM rows over %dK INT64 keys, COUNT/SUM/AVG(DOUBLE)" % (rows // 10**6, nv // 1000),
               "SELECT c0, COUNT(*), SUM(c1), AVG(c1) FROM t GROUP BY c0",
               [3, 4], [0], [("count_star", -1), ("sum", 1), ("avg", 1)], [k, x])
    a, b, s, m = datagen.composite(1_000_000, 100_000, seed=3)
    yield ("(INT32, SMALLINT) key 1M rows, 100K groups, COUNT/SUM/MAX",
           "SELECT c0, c1, COUNT(*), SUM(c2), MAX(c3) FROM t GROUP BY c0, c1",
           [2, 1, 3, 2], [0, 1], [("count_star", -1), ("sum", 2), ("max", 3)], [a, b, s, m])
    (offs, data), s, m = datagen.varchar_table(200_000, 10_000, seed=4)
    yield ("VARCHAR key 200K rows, 10K strings, COUNT/SUM/MAX",
           "SELECT c0, COUNT(*), SUM(c1), MAX(c2) FROM t GROUP BY c0",
           [5, 3, 2], [0], [("count_star", -1), ("sum", 1), ("max", 2)], [(offs, data), s, m])


def main():
    if reference.build() is None or not reference.available():
        print("reference sources not found: nothing to calibrate")
        return
    rows = []
    threads = os.cpu_count() or 1
    for name, sql, types, gc, aggs, cols in shapes():
        _, ref_ms = reference.query(sql, types, cols, repeat=3)
        p1 = _port_ms(types, gc, aggs, cols, 1)
        pn = _port_ms(types, gc, aggs, cols, threads)
        rows.append({"shape": name, "reference_ms": round(ref_ms, 2), "port_1t_ms": round(p1, 2),
                     "port_%dt_ms" % threads: round(pn, 2), "reference_over_port_1t": round(ref_ms / p1, 2)})
        print(json.dumps(rows[-1]), flush=True)


if __name__ == "__main__":
    main()
