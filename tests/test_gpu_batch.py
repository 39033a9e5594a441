"""GPU parity of the batched path: many independent GROUP BY queries
(composite (INT32, INT16) keys and VARCHAR keys; COUNT(*), SUM(INT64),
MAX(INT32)) executed together through gb_batch, each result checked against
the oracle and against the same query run alone.  Bit-exact."""
import numpy as np
import pytest

import oracle
from slothdb_gb300 import capi, datagen
from util import as_expected, compare, gpu_to_dict

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("oracle_lib", "gblib")]

COMP = datagen.BATCH_COMPOSITE
STR = datagen.BATCH_VARCHAR


def _q(shape):
    return COMP if shape["kind"] == "composite" else STR


def _out_types(q):
    return [q["col_types"][c] for c in q["group_cols"]] + [
        oracle.agg_out_type(oracle.AGG_NAMES[k], q["col_types"][c] if c >= 0 else 0) for k, c in q["aggs"]]


def _to_device(cols, col_types):
    import torch
    out = []
    for c, t in zip(cols, col_types):
        if t == capi.VARCHAR:
            offs, data = c
            data = data if len(data) else np.zeros(1, np.uint8)
            out.append((torch.from_numpy(np.ascontiguousarray(offs)).cuda(),
                        torch.from_numpy(np.ascontiguousarray(data)).cuda()))
        else:
            out.append(torch.from_numpy(np.ascontiguousarray(c)).cuda())
    torch.cuda.synchronize()
    return out


def _orc(shape, cols, nulls=None):
    q = _q(shape)
    return oracle.run_query(q["col_types"], q["group_cols"], q["aggs"], cols, nulls=nulls)


def _gpu(res, shape):
    q = _q(shape)
    return gpu_to_dict(res, len(q["group_cols"]), _out_types(q))


def _build(shapes, est=None, options=None):
    b = capi.Batch(options)
    host, dev = [], []
    for i, sh in enumerate(shapes):
        q = _q(sh)
        cols = datagen.batch_table_host(sh)
        d = _to_device(cols, q["col_types"])
        host.append(cols)
        dev.append(d)
        e = sh["groups"] if est is None else est[i]
        assert b.add(q["col_types"], q["group_cols"], q["aggs"], d, sh["rows"], est_groups=e) == i
    return b, host, dev


def test_batch_mixed_queries_match_oracle_and_replay():
    shapes = datagen.batch_shapes(n_tables=24, seed=7, rows_exp=(3.0, 5.3), groups_exp=(1.0, 4.5))
    b, host, dev = _build(shapes)
    try:
        assert len(b) == 24
        b.run()
        first = []
        for i, sh in enumerate(shapes):
            r = b.result(i)
            first.append(r)
            compare(_gpu(r, sh), _orc(sh, host[i]))
        assert b.launches() > 0
        # replay of the captured graph: same results
        b.run()
        assert b.slow_queries() == 0
        for i, sh in enumerate(shapes):
            compare(_gpu(b.result(i), sh), as_expected(_gpu(first[i], sh)), rel_tol=0.0)
    finally:
        b.close()


@pytest.mark.parametrize("options", [{"graph": 0}, {"smem_slots": 0, "precombine": 0},
                                     {"ctas_per_sm": 1, "smem_slots": 512}, {"fast": 0}, {"order": 1},
                                     {"fast": 0, "precombine": 0}, {"profiling": 1}, {"precombine": 2}])
def test_batch_options(options):
    shapes = datagen.batch_shapes(n_tables=10, seed=8, rows_exp=(3.0, 5.0), groups_exp=(1.0, 4.0))
    b, host, _ = _build(shapes, options=options)
    try:
        for _ in range(2):
            b.run()
            for i, sh in enumerate(shapes):
                compare(_gpu(b.result(i), sh), _orc(sh, host[i]))
        if options.get("profiling"):
            prof = b.profile()
            assert prof["k_batch_ingest"][0] == 2 and prof["k_batch_ingest"][1] > 0
    finally:
        b.close()


def test_batch_result_same_as_alone():
    """Each query's batched result equals the same query run on its own."""
    shapes = datagen.batch_shapes(n_tables=8, seed=9, rows_exp=(4.0, 5.5), groups_exp=(2.0, 4.5))
    b, host, dev = _build(shapes)
    try:
        b.run()
        for i, sh in enumerate(shapes):
            q = _q(sh)
            g = capi.GroupBy(q["col_types"], q["group_cols"], q["aggs"], est_groups=sh["groups"])
            try:
                g.ingest(dev[i], nrows=sh["rows"], device=True)
                g.finalize()
                alone = g.result()
            finally:
                g.close()
            compare(_gpu(b.result(i), sh), as_expected(_gpu(alone, sh)), rel_tol=0.0)
    finally:
        b.close()


def test_batch_underestimated_groups_take_the_slow_path():
    """est_groups far below the real count: the batched table overflows, the
    query re-runs on its own handle, and the next run fits in the batch."""
    shapes = [dict(kind="composite", rows=200_000, groups=60_000, seed=11),
              dict(kind="varchar", rows=150_000, groups=40_000, seed=12),
              dict(kind="composite", rows=5_000, groups=100, seed=13)]
    b, host, _ = _build(shapes, est=[16, 16, 100])
    try:
        b.run()
        assert b.slow_queries() >= 2
        for i, sh in enumerate(shapes):
            compare(_gpu(b.result(i), sh), _orc(sh, host[i]))
        b.run()
        assert b.slow_queries() == 0
        for i, sh in enumerate(shapes):
            compare(_gpu(b.result(i), sh), _orc(sh, host[i]))
    finally:
        b.close()


def test_batch_empty_tiny_and_nullable():
    import torch
    rng = np.random.default_rng(21)
    b = capi.Batch()
    try:
        # empty table
        e = [torch.zeros(1, dtype=torch.int32, device="cuda"), torch.zeros(1, dtype=torch.int16, device="cuda"),
             torch.zeros(1, dtype=torch.int64, device="cuda"), torch.zeros(1, dtype=torch.int32, device="cuda")]
        b.add(COMP["col_types"], COMP["group_cols"], COMP["aggs"], e, 0, est_groups=10)
        # one row
        one = datagen.batch_table_host(dict(kind="varchar", rows=1, groups=1, seed=5))
        b.add(STR["col_types"], STR["group_cols"], STR["aggs"], _to_device(one, STR["col_types"]), 1, est_groups=1)
        # nullable key and value columns
        n = 70_001
        a = rng.integers(0, 300, n, dtype=np.int32)
        kb = rng.integers(0, 64, n, dtype=np.int16)
        s = rng.integers(0, 10**6, n, dtype=np.int64)
        m = rng.integers(-(2**31), 2**31 - 1, n, dtype=np.int32)
        an = rng.random(n) < 0.05
        mn = rng.random(n) < 0.3
        va = capi.validity_words(~an)
        vm = capi.validity_words(~mn)
        d = _to_device([a, kb, s, m], COMP["col_types"])
        vd = [torch.from_numpy(va.view(np.int64)).cuda(), None, None, torch.from_numpy(vm.view(np.int64)).cuda()]
        b.add(COMP["col_types"], COMP["group_cols"], COMP["aggs"], d, n, validity=vd, nullable=[0, 3],
              est_groups=20_000)
        torch.cuda.synchronize()
        b.run()
        r0 = b.result(0)
        assert len(r0[0][0]) == 0
        compare(_gpu(b.result(1), dict(kind="varchar")), _orc(dict(kind="varchar"), one))
        orc = oracle.run_query(COMP["col_types"], COMP["group_cols"], COMP["aggs"], [a, kb, s, m],
                               nulls=[an, None, None, mn])
        compare(_gpu(b.result(2), dict(kind="composite")), orc)
    finally:
        b.close()


def test_batch_filters_int_and_double():
    """WHERE predicates on the fast path (integer and DOUBLE columns, with
    and without NULLs) and on the generic path (a DOUBLE SUM)."""
    import torch
    rng = np.random.default_rng(31)
    b = capi.Batch()
    checks = []
    try:
        for i, (kind, flt) in enumerate([("composite", [(2, "<", 300_000)]),
                                          ("composite", [(3, ">=", 0), (2, "!=", 5)]),
                                          ("varchar", [(1, "<", 500_000)]),
                                          ("composite", [(2, "<", -1)])]):   # selects nothing
            sh = dict(kind=kind, rows=120_000 + 17 * i, groups=3000 + 1000 * i, seed=40 + i)
            q = _q(sh)
            cols = datagen.batch_table_host(sh)
            b.add(q["col_types"], q["group_cols"], q["aggs"], _to_device(cols, q["col_types"]), sh["rows"],
                  filters=flt, est_groups=sh["groups"])
            checks.append((sh, oracle.run_query(q["col_types"], q["group_cols"], q["aggs"], cols, filters=flt)))
        # DOUBLE filter + nullable filter column on the fast path
        n = 90_001
        k = rng.integers(0, 700, n, dtype=np.int32)
        x = rng.normal(100, 25, n)
        v = rng.integers(-1000, 1000, n, dtype=np.int64)
        xn = rng.random(n) < 0.1
        types = [capi.INTEGER, capi.DOUBLE, capi.BIGINT]
        aggs = [("count_star", -1), ("sum", 2), ("min", 2)]
        d = _to_device([k, x, v], types)
        vx = torch.from_numpy(capi.validity_words(~xn).view(np.int64)).cuda()
        b.add(types, [0], aggs, d, n, validity=[None, vx, None], nullable=[1], filters=[(1, ">", 104.5)],
              est_groups=700)
        orc_fast = oracle.run_query(types, [0], aggs, [k, x, v], filters=[(1, ">", 104.5)], nulls=[None, xn, None])
        # generic path: SUM of a DOUBLE
        aggs_g = [("count_star", -1), ("sum", 1)]
        b.add(types, [0], aggs_g, d, n, filters=[(2, "<", 0)], est_groups=700)
        orc_gen = oracle.run_query(types, [0], aggs_g, [k, x, v], filters=[(2, "<", 0)])
        torch.cuda.synchronize()
        b.run()
        for i, (sh, orc) in enumerate(checks):
            compare(_gpu(b.result(i), sh), orc)
        nb = len(checks)
        compare(gpu_to_dict(b.result(nb), 1, [capi.INTEGER, capi.BIGINT, capi.BIGINT, capi.BIGINT]), orc_fast)
        compare(gpu_to_dict(b.result(nb + 1), 1, [capi.INTEGER, capi.BIGINT, capi.DOUBLE]), orc_gen)
    finally:
        b.close()


def test_batch_clear_reuses_handles_with_new_filters():
    """gb_batch_clear keeps the queries' handles; the next adds of the same
    shape reuse them with new predicates and still match the oracle."""
    shapes = [dict(kind="composite", rows=50_000 + i * 1000, groups=2000, seed=80 + i) for i in range(3)] + \
             [dict(kind="varchar", rows=40_000, groups=900, seed=90)]
    host = [datagen.batch_table_host(sh) for sh in shapes]
    dev = [_to_device(c, _q(sh)["col_types"]) for c, sh in zip(host, shapes)]
    b = capi.Batch()
    try:
        for rnd, thr in enumerate([300_000, 800_000, 50_000]):
            if rnd:
                b.clear()
            for sh, d in zip(shapes, dev):
                q = _q(sh)
                fcol = 2 if sh["kind"] == "composite" else 1
                b.add(q["col_types"], q["group_cols"], q["aggs"], d, sh["rows"], filters=[(fcol, "<", thr)],
                      est_groups=sh["groups"])
            b.run()
            for i, (sh, cols) in enumerate(zip(shapes, host)):
                q = _q(sh)
                fcol = 2 if sh["kind"] == "composite" else 1
                compare(_gpu(b.result(i), sh), oracle.run_query(q["col_types"], q["group_cols"], q["aggs"], cols,
                                                                filters=[(fcol, "<", thr)]))
    finally:
        b.close()


def test_set_filters_on_a_reset_handle():
    k, v = datagen.plain(200_000, seed=5)
    import torch
    dk, dv = torch.from_numpy(k).cuda(), torch.from_numpy(v).cuda()
    aggs = [("count_star", -1), ("sum", 1)]
    g = capi.GroupBy([capi.INTEGER, capi.BIGINT], [0], aggs, filters=[(1, "<", 1000)])
    try:
        for thr in (1000, 500_000):
            g.reset()
            g.set_filters([(1, "<", thr)])
            g.ingest([dk, dv], nrows=len(k), device=True)
            g.finalize()
            compare(gpu_to_dict(g.result(), 1, [capi.INTEGER, capi.BIGINT, capi.BIGINT]),
                    oracle.run_query([capi.INTEGER, capi.BIGINT], [0], aggs, [k, v], filters=[(1, "<", thr)]))
        with pytest.raises(capi.GbError):
            g.set_filters([(1, "<", 5)])   # after finalize, before reset
    finally:
        g.close()
