"""The served query stream (gb_server): results of queries executed in
mixed, continuously formed batches equal the same queries run alone;
admission by estimated bytes; the one-at-a-time mode; row-range slices."""
import threading

import numpy as np
import pytest

import oracle
from slothdb_gb300 import capi, datagen
from util import as_expected, compare, gpu_to_dict

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("oracle_lib", "gblib")]

COMP = datagen.BATCH_COMPOSITE
STR = datagen.BATCH_VARCHAR


def _dev(cols, types):
    import torch
    out = []
    for c, t in zip(cols, types):
        if t == capi.VARCHAR:
            out.append((torch.from_numpy(c[0]).cuda(), torch.from_numpy(c[1]).cuda()))
        else:
            out.append(torch.from_numpy(np.ascontiguousarray(c)).cuda())
    torch.cuda.synchronize()
    return out


def _slice_host(cols, types, r0, r1):
    out = []
    for c, t in zip(cols, types):
        if t == capi.VARCHAR:
            offs, data = c
            o = offs[r0:r1 + 1]
            out.append((o - o[0], data[o[0]:o[-1]] if o[-1] > o[0] else np.zeros(1, np.uint8)))
        else:
            out.append(c[r0:r1])
    return out


def _out_types(types, group_cols, aggs):
    return [types[g] for g in group_cols] + [oracle.agg_out_type(oracle.AGG_NAMES[k], types[c] if c >= 0 else 0)
                                             for k, c in aggs]


@pytest.fixture(scope="module")
def tables():
    comp = datagen.batch_table_host(dict(kind="composite", rows=400_000, groups=20_000, seed=61))
    vch = datagen.batch_table_host(dict(kind="varchar", rows=300_000, groups=5_000, seed=62))
    k, v = datagen.plain(500_000, seed=63)
    plain_types = [capi.INTEGER, capi.BIGINT]
    return [(COMP["col_types"], comp), (STR["col_types"], vch), (plain_types, [k, v])]


def _queries(rng, n, tabs):
    qs = []
    for i in range(n):
        t = int(rng.integers(0, len(tabs)))
        types, cols = tabs[t]
        nrows = len(cols[1]) if types[0] == capi.VARCHAR else len(cols[0])
        r0 = int(rng.integers(0, nrows // 2))
        r1 = int(rng.integers(r0 + 1, nrows + 1))
        sel = float(rng.uniform(0.01, 1.0))
        if t == 2:
            group_cols, aggs = [0], [("count_star", -1), ("sum", 1), ("min", 1), ("max", 1)]
            if i % 3 == 0:  # COUNT(DISTINCT), batched beside the others
                aggs = [("count_distinct", 1), ("count_star", -1), ("sum", 1)]
            filters = [(1, "<", int(sel * 10**6))]
        else:
            q = COMP if t == 0 else STR
            group_cols, aggs = q["group_cols"], q["aggs"]
            filters = [(2 if t == 0 else 1, "<", int(sel * 10**6))]
        # every fifth query estimates radix-sized group counts: it runs alone,
        # on the partitioned path, beside the other lanes' batches
        est = (1 << 20) if i % 5 == 4 and t != 1 else 0
        qs.append(dict(table=t, r0=r0, r1=r1, group_cols=group_cols, aggs=aggs, filters=filters, est=est))
    return qs


def _alone(types, dcols, q):
    """The same query through a plain handle on a device slice."""
    import torch
    cols = []
    for c, t in zip(dcols, types):
        if t == capi.VARCHAR:
            cols.append((c[0][q["r0"]:q["r1"] + 1], c[1]))
        else:
            cols.append(c[q["r0"]:q["r1"]])
    g = capi.GroupBy(types, q["group_cols"], q["aggs"], filters=q["filters"])
    try:
        g.ingest(cols, nrows=q["r1"] - q["r0"], device=True)
        g.finalize()
        return g.result()
    finally:
        g.close()


@pytest.mark.parametrize("mode,lanes", [(0, None), (0, 1), (0, 3), (1, None)])
def test_mixed_results_equal_alone(tables, mode, lanes):
    """Every result equals the query run alone (and the oracle's on a
    sample), with one, two (the default) or three execution lanes, and in
    one-at-a-time mode."""
    rng = np.random.default_rng(70 + mode)
    dtabs = [_dev(cols, types) for types, cols in tables]
    srv = capi.Server(budget_bytes=8 << 30, max_batch=64, mode=mode, lanes=lanes)
    try:
        for (types, cols), d in zip(tables, dtabs):
            n = len(cols[1]) if types[0] == capi.VARCHAR else len(cols[0])
            srv.add_table(types, d, n)
        qs = _queries(rng, 40, tables)
        tickets = [None] * len(qs)

        def submit(lo, hi):
            for i in range(lo, hi):
                q = qs[i]
                tickets[i] = srv.submit(q["table"], q["r0"], q["r1"], q["group_cols"], q["aggs"],
                                        filters=q["filters"], est_groups=q["est"])

        th = [threading.Thread(target=submit, args=(i * 10, i * 10 + 10)) for i in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        for i, q in enumerate(qs):
            assert srv.wait(tickets[i])
            types = tables[q["table"]][0]
            ot = _out_types(types, q["group_cols"], q["aggs"])
            got = gpu_to_dict(srv.result(tickets[i]), len(q["group_cols"]), ot)
            alone = gpu_to_dict(_alone(types, dtabs[q["table"]], q), len(q["group_cols"]), ot)
            compare(got, as_expected(alone), rel_tol=0.0)
            if i % 8 == 0:  # and against the oracle
                host = _slice_host(tables[q["table"]][1], types, q["r0"], q["r1"])
                compare(got, oracle.run_query(types, q["group_cols"], q["aggs"], host, filters=q["filters"]))
            qm, em, bs = srv.times(tickets[i])
            assert qm >= 0 and em >= 0 and bs >= 1
            srv.release(tickets[i])
        st = srv.stats()
        assert st["completed"] == len(qs) and st["failed"] == 0 and st["rejected"] == 0
        if mode == 0:
            assert st["batches"] < len(qs)  # queries were batched
    finally:
        srv.close()


def test_admission_budget_and_rejection(tables):
    types, cols = tables[0]
    d = _dev(cols, types)
    n = len(cols[0])
    small = capi.estimate_bytes(types, COMP["group_cols"], COMP["aggs"], 10_000, est_groups=1000)
    big = capi.estimate_bytes(types, COMP["group_cols"], COMP["aggs"], n, est_groups=1 << 22)
    assert big > small
    budget = 3 * small + small // 2  # three small queries per batch at most
    srv = capi.Server(budget_bytes=budget, max_batch=64, mode=0)
    try:
        srv.add_table(types, d, n)
        ts = [srv.submit(0, 0, 10_000, COMP["group_cols"], COMP["aggs"], est_groups=1000) for _ in range(9)]
        tb = srv.submit(0, 0, n, COMP["group_cols"], COMP["aggs"], est_groups=1 << 22)
        for t in ts:
            assert srv.wait(t)
        with pytest.raises(capi.GbError) as e:
            srv.wait(tb)
        assert e.value.status == capi.GB_ERR_BUDGET
        st = srv.stats()
        assert st["rejected"] == 1 and st["completed"] == 9  # executed queries; the rejected one is not
        assert st["peak_admitted_bytes"] <= budget
        assert st["batches"] >= 3
        r0 = srv.result(ts[0])
        for t in ts[1:]:
            r = srv.result(t)
            assert len(r[0][0]) == len(r0[0][0])
    finally:
        srv.close()


def test_high_cardinality_query_runs_alone_on_the_radix_path():
    import torch
    k, x = datagen.zipf(1_500_000, seed=64, n_values=1_000_000)
    types = [capi.BIGINT, capi.DOUBLE]
    srv = capi.Server(budget_bytes=16 << 30, max_batch=8, mode=0)
    try:
        srv.add_table(types, [torch.from_numpy(k).cuda(), torch.from_numpy(x).cuda()], len(k))
        aggs = [("count_star", -1), ("sum", 1), ("avg", 1)]
        t = srv.submit(0, 100_000, len(k), [0], aggs, est_groups=1 << 21)
        assert srv.wait(t)
        got = gpu_to_dict(srv.result(t), 1, [capi.BIGINT, capi.BIGINT, capi.DOUBLE, capi.DOUBLE])
        compare(got, oracle.run_query(types, [0], aggs, [k[100_000:], x[100_000:]]))
    finally:
        srv.close()


def test_submit_errors(tables):
    import torch
    types, cols = tables[2]
    d = _dev(cols, types)
    n = len(cols[0])
    valid = torch.from_numpy(capi.validity_words(np.ones(n, bool)).view(np.int64)).cuda()
    srv = capi.Server(budget_bytes=1 << 30)
    try:
        t0 = srv.add_table(types, d, n)
        t1 = srv.add_table(types, d, n, validity=[valid, None])
        aggs = [("count_star", -1)]
        with pytest.raises(capi.GbError):
            srv.submit(t0, 10, n + 1, [0], aggs)        # past the table
        with pytest.raises(capi.GbError):
            srv.submit(t1, 10, 100, [0], aggs)          # validity slice not at a multiple of 64
        t = srv.submit(t1, 64, 1000, [0], aggs, nullable=[0])
        assert srv.wait(t)
        with pytest.raises(capi.GbError):
            srv.add_table(types, d, n)                  # tables are registered before the first query
    finally:
        srv.close()


def test_lane_settings(tables):
    """Lanes are 1..8, set before the first submit; one-at-a-time mode runs
    one lane."""
    with pytest.raises(capi.GbError):
        capi.Server(budget_bytes=1 << 30, lanes=0)
    with pytest.raises(capi.GbError):
        capi.Server(budget_bytes=1 << 30, lanes=9)
    with pytest.raises(capi.GbError):
        capi.Server(budget_bytes=1 << 30, mode=1, lanes=2)
    types, cols = tables[2]
    srv = capi.Server(budget_bytes=1 << 30, lanes=4)
    try:
        srv.add_table(types, _dev(cols, types), len(cols[0]))
        t = srv.submit(0, 0, 1000, [0], [("count_star", -1)])
        assert srv.wait(t)
        srv.release(t)
        with pytest.raises(capi.GbError):
            capi.check(srv.lib.gb_server_set_lanes(srv.h, 2))  # after the first submit
    finally:
        srv.close()
