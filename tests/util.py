"""Result comparison helpers shared by the parity tests."""
from __future__ import annotations

import numpy as np

DOUBLE = 4
REL_TOL_F64 = 1e-12  # DOUBLE SUM/AVG tolerance vs the FP64 compensated sum


def _order(keys, key_null):
    cols = []
    for k, kn in zip(reversed(keys), reversed(key_null)):
        if k.dtype == object:
            # strings: rank by sorted unique values (NULL entries ranked first)
            k = np.array([b"" if n else x for x, n in zip(k, kn)], dtype=object)
            uniq = sorted(set(k.tolist()))
            pos = {s: i for i, s in enumerate(uniq)}
            k = np.array([pos[s] for s in k.tolist()], dtype=np.int64)
        cols.append(np.where(kn, np.iinfo(np.int64).min, k.astype(np.int64)))
        cols.append(~kn)
    return np.lexsort(cols) if cols else np.arange(0)


def gpu_to_dict(res, n_keys, out_types):
    keys = [res[i][0] for i in range(n_keys)]
    key_null = [~res[i][1] for i in range(n_keys)]
    aggs = [(res[n_keys + a][0], ~res[n_keys + a][1]) for a in range(len(res) - n_keys)]
    return dict(keys=keys, key_null=key_null, aggs=aggs, out_types=out_types)


def rel_err(got, ref):
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    denom = np.maximum(np.abs(ref), np.finfo(np.float64).tiny)
    return np.abs(got - ref) / denom


def compare(gpu, orc, rel_tol=REL_TOL_F64, check_order=False):
    """Assert GPU result == oracle result as group sets.  Integer columns
    bit-exact; DOUBLE SUM/AVG within rel_tol of the compensated FP64 value.
    Returns the max relative error seen on DOUBLE columns."""
    n_keys = len(orc["keys"])
    assert len(gpu["keys"][0]) == len(orc["keys"][0]), \
        "group count differs: gpu %d oracle %d" % (len(gpu["keys"][0]), len(orc["keys"][0]))
    go = np.arange(len(gpu["keys"][0])) if check_order else _order(gpu["keys"], gpu["key_null"])
    oo = np.arange(len(orc["keys"][0])) if check_order else _order(orc["keys"], orc["key_null"])
    for i in range(n_keys):
        gn, on = gpu["key_null"][i][go], orc["key_null"][i][oo]
        assert np.array_equal(gn, on), "key NULL flags differ (col %d)" % i
        gk, ok = gpu["keys"][i][go], orc["keys"][i][oo]
        if ok.dtype == object:
            gl = [b"" if n else x for x, n in zip(gk, gn)]
            ol = [b"" if n else x for x, n in zip(ok, on)]
            assert gl == ol, "string keys differ"
        else:
            assert np.array_equal(np.where(gn, 0, gk.astype(np.int64)), np.where(on, 0, ok.astype(np.int64))), \
                "keys differ (col %d)" % i
    worst = 0.0
    for a, ((gv, gnull), (ov, onull, ocomp)) in enumerate(zip(gpu["aggs"], orc["aggs"])):
        gv, gnull = gv[go], gnull[go]
        ov, onull, ocomp = ov[oo], onull[oo], ocomp[oo]
        assert np.array_equal(gnull, onull), "NULL flags differ (agg %d)" % a
        t = orc["out_types"][n_keys + a]
        m = ~onull
        if t == DOUBLE:
            # compensated reference where the oracle has one (SUM/AVG), else
            # the oracle's own value (MIN/MAX of DOUBLE are exact)
            ref = np.where(ocomp != 0.0, ocomp, ov)
            e = rel_err(gv[m], ref[m])
            mx = float(e.max()) if e.size else 0.0
            worst = max(worst, mx)
            assert mx <= rel_tol, "agg %d: DOUBLE rel err %.3e > %.1e" % (a, mx, rel_tol)
        else:
            bad = np.nonzero(gv[m].astype(np.int64) != ov[m].astype(np.int64))[0]
            assert bad.size == 0, "agg %d: %d integer mismatches, first gpu=%r oracle=%r" % (
                a, bad.size, gv[m][bad[0]], ov[m][bad[0]])
    return worst


def as_expected(gpu):
    """A GPU result in the oracle's shape, to compare two GPU results with
    compare(..., rel_tol=0.0) (exact equality of every column)."""
    return dict(keys=gpu["keys"], key_null=gpu["key_null"], out_types=gpu["out_types"],
                aggs=[(v, n, np.zeros(len(v))) for v, n in gpu["aggs"]])
