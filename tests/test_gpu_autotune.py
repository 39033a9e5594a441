"""The autotuner on the GPU: candidates run, the winner lands in the cache,
and a handle built with the tuned options returns the oracle's result."""
import numpy as np
import pytest

import oracle
from slothdb_gb300 import autotune, capi, datagen
from util import compare, gpu_to_dict

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("oracle_lib", "gblib")]


def test_tune_groupby_and_apply(tmp_path):
    import torch
    k, x = datagen.zipf(1_000_000, seed=4, n_values=300_000)
    dk, dx = torch.from_numpy(k).cuda(), torch.from_numpy(x).cuda()
    aggs = [("count_star", -1), ("sum", 1), ("avg", 1)]
    types = [capi.BIGINT, capi.DOUBLE]
    cache = autotune.TuneCache(str(tmp_path / "tune.json"))
    cands = [{"mode": 1, "smem_slots": 0, "tile_rows": 8192, "ctas_per_sm": 2},
             {"mode": 1, "smem_slots": 4096, "tile_rows": 32768, "ctas_per_sm": 2},
             {"mode": 2, "radix_bits": 8}, {"mode": 2, "radix_bits": 10}]
    best, ms = autotune.tune_groupby(types, [0], aggs, [dk, dx], len(k), est_groups=1 << 18, cache=cache,
                                     candidates=cands, reps=1)
    assert best in cands and ms > 0
    again = autotune.TuneCache(str(tmp_path / "tune.json"))
    opts = autotune.tuned_groupby_options(types, [0], aggs, len(k), est_groups=1 << 18, cache=again)
    assert opts == best
    g = capi.GroupBy(types, [0], aggs, est_groups=1 << 18, options={"mode": opts["mode"]})
    try:
        for name, v in opts.items():
            if name != "mode":
                g.set_option(name, v)
        g.ingest([dk, dx], nrows=len(k), device=True)
        g.finalize()
        res = g.result()
    finally:
        g.close()
    orc = oracle.run_query(types, [0], aggs, [k, x])
    compare(gpu_to_dict(res, 1, [capi.BIGINT, capi.BIGINT, capi.DOUBLE, capi.DOUBLE]), orc)


def test_tune_batch(tmp_path):
    shapes = datagen.batch_shapes(n_tables=6, seed=12, rows_exp=(4.0, 5.5), groups_exp=(1.0, 4.5))
    tables = []
    import torch
    for sh in shapes:
        tables.append(datagen.batch_table_device(sh))
    torch.cuda.synchronize()

    def make(opts):
        b = capi.Batch(opts)
        for sh, cols in zip(shapes, tables):
            q = datagen.BATCH_COMPOSITE if sh["kind"] == "composite" else datagen.BATCH_VARCHAR
            b.add(q["col_types"], q["group_cols"], q["aggs"], cols, sh["rows"], est_groups=sh["groups"])
        return b

    cache = autotune.TuneCache(str(tmp_path / "tune.json"))
    cands = [{"tile_rows": 8192, "smem_slots": 4096, "order": 0}, {"tile_rows": 65536, "smem_slots": 2048, "order": 1}]
    best, ms = autotune.tune_batch(make, "t6", sum(s["rows"] for s in shapes), len(shapes), cache=cache,
                                   candidates=cands, reps=1)
    assert best in cands and ms > 0
    # the tuned batch and a default batch agree query by query
    b1, b2 = make(best), make({})
    try:
        b1.run()
        b2.run()
        for i in range(len(shapes)):
            r1, r2 = b1.result(i), b2.result(i)
            assert len(r1[0][0]) == len(r2[0][0])
            assert sorted(map(repr, zip(*[c[0] for c in r1]))) == sorted(map(repr, zip(*[c[0] for c in r2])))
    finally:
        b1.close()
        b2.close()
