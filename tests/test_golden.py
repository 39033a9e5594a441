"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py):
the oracle reproduces them on CPU, and the GPU path reproduces them on the
GPU — integers bit-exact, DOUBLE within 1e-12 relative."""
import os
import sys

import numpy as np
import pytest

import oracle
from util import REL_TOL_F64, compare, gpu_to_dict

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import make_golden  # noqa: E402

CASES = make_golden.cases()


def _fixture(name, n_keys):
    z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=True)
    keys = [z["key%d" % i] for i in range(n_keys)]
    key_null = [z["key%d_null" % i] for i in range(n_keys)]
    aggs, a = [], 0
    while "agg%d" % a in z:
        aggs.append((z["agg%d" % a], z["agg%d_null" % a], z["agg%d_comp" % a]))
        a += 1
    return keys, key_null, aggs


def _expected(name):
    types, groups, aggs, filters, cols = CASES[name]
    keys, key_null, res = _fixture(name, len(groups))
    out_types = [types[g] for g in groups] + [oracle.agg_out_type(oracle.AGG_NAMES[k], types[c] if c >= 0 else 0)
                                              for k, c in aggs]
    return dict(keys=keys, key_null=key_null, aggs=res, out_types=out_types)


@pytest.mark.usefixtures("oracle_lib")
@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_golden(name):
    types, groups, aggs, filters, cols = CASES[name]
    got = oracle.run_query(types, groups, aggs, cols, filters=filters)
    exp = _expected(name)
    for i in range(len(groups)):
        assert len(got["keys"][i]) == len(exp["keys"][i])
    # the fixture in oracle shape, compared like a GPU result (exact / 1e-12)
    g = dict(keys=got["keys"], key_null=got["key_null"], out_types=exp["out_types"],
             aggs=[(v, n) for v, n, _ in got["aggs"]])
    compare(g, exp, rel_tol=REL_TOL_F64)


@pytest.mark.gpu
@pytest.mark.usefixtures("oracle_lib", "gblib")
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_reproduces_golden(name):
    from slothdb_gb300 import capi
    from slothdb_gb300 import parquet as pq
    types, groups, aggs, filters, cols = CASES[name]
    if name.startswith("parquet"):
        data, _, _, _ = pq.filter_groupby_file(n_rows=200_000, seed=2, n_dict=4096, row_group_rows=50_000,
                                               page_rows=8192)
        pf = capi.ParquetFile(data)
        g = capi.GroupBy(types, groups, aggs, filters=filters, est_groups=4096)
        try:
            capi.ingest_parquet(g, pf, [0, 1, 2])
            g.finalize()
            res = g.result()
        finally:
            g.close()
            pf.close()
    else:
        g = capi.GroupBy(types, groups, aggs, filters=filters)
        try:
            g.ingest(cols)
            g.finalize()
            res = g.result()
        finally:
            g.close()
    exp = _expected(name)
    compare(gpu_to_dict(res, len(groups), exp["out_types"]), exp)
