"""Seeded synthetic inputs with the shapes of the GROUP BY workloads.

All generators use numpy's PCG64 (``numpy.random.default_rng(seed)``) and
are deterministic across machines.  Workloads:

* ``plain``      — 1,000,000 rows, seed 0: k INT32 uniform over 1,024
                   values, v INT64 uniform in [0, 10^6).
* ``zipf``       — 100,000,000 rows, seed 1: k INT64 = Zipf(s=1.1) rank over
                   20,000,000 values mapped through a seeded permutation of
                   [0, 2^40); x DOUBLE ~ Normal(100, 25).
* ``composite`` / ``varchar`` — per-query tables of the batched workload.
"""
from __future__ import annotations

import numpy as np

MASK20 = np.uint64((1 << 20) - 1)


def _mix(x: np.ndarray) -> np.ndarray:
    x = x.astype(np.uint64, copy=True)
    with np.errstate(over="ignore"):
        x ^= x >> np.uint64(31)
        x *= np.uint64(0x7FB5D329728EA185)
        x ^= x >> np.uint64(27)
        x *= np.uint64(0x81DADEF4BC2DD44D)
        x ^= x >> np.uint64(33)
    return x


def permute40(r: np.ndarray, seed: int) -> np.ndarray:
    """Seeded bijection of [0, 2^40): a 4-round Feistel network on two
    20-bit halves (a random permutation of [0, 2^40) keyed by ``seed``)."""
    keys = _mix(np.arange(1, 5, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15 & ((1 << 63) - 1)) +
                np.uint64(seed))
    x = r.astype(np.uint64)
    L = (x >> np.uint64(20)) & MASK20
    R = x & MASK20
    for k in keys:
        F = _mix(R ^ k) & MASK20
        L, R = R, L ^ F
    return ((L << np.uint64(20)) | R).astype(np.int64)


def zipf_cdf(n_values: int, s: float) -> np.ndarray:
    w = np.arange(1, n_values + 1, dtype=np.float64) ** (-s)
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    return cdf


def zipf_ranks(u: np.ndarray, cdf: np.ndarray) -> np.ndarray:
    """Inverse-CDF Zipf ranks (0-based) for uniforms u.  Uses the GPU's
    searchsorted when torch with CUDA is present and the input is large
    (bit-identical to numpy: exact float64 comparisons)."""
    if len(u) >= (1 << 22):
        try:
            import torch
            if torch.cuda.is_available():
                cd = torch.from_numpy(cdf).cuda()
                out = np.empty(len(u), dtype=np.int64)
                step = 1 << 25
                for i in range(0, len(u), step):
                    ud = torch.from_numpy(u[i:i + step]).cuda()
                    out[i:i + step] = torch.searchsorted(cd, ud, right=True).cpu().numpy()
                del cd
                np.minimum(out, len(cdf) - 1, out=out)
                return out
        except Exception:
            pass
    r = np.searchsorted(cdf, u, side="right")
    np.minimum(r, len(cdf) - 1, out=r)
    return r.astype(np.int64)


def plain(n: int = 1_000_000, seed: int = 0, n_keys: int = 1024):
    """k INT32 uniform over n_keys values, v INT64 uniform in [0, 10^6)."""
    rng = np.random.default_rng(seed)
    k = rng.integers(0, n_keys, n, dtype=np.int32)
    v = rng.integers(0, 10**6, n, dtype=np.int64)
    return k, v


def zipf(n: int = 100_000_000, seed: int = 1, n_values: int = 20_000_000, s: float = 1.1):
    """k INT64 Zipf(s) over n_values ranks mapped into [0, 2^40) by a seeded
    permutation; x DOUBLE ~ Normal(100, 25).  Draw order: uniforms, then x."""
    rng = np.random.default_rng(seed)
    cdf = zipf_cdf(n_values, s)
    u = rng.random(n)
    ranks = zipf_ranks(u, cdf)
    del u
    k = permute40(ranks, seed)
    x = rng.normal(100.0, 25.0, n)
    return k, x


def composite(n: int, n_groups: int, seed: int):
    """Composite-key table: a INT32 uniform over max(1, n_groups // 64)
    values, b INT16 uniform in [0, 64), s INT64 uniform [0, 10^6),
    m INT32 uniform."""
    rng = np.random.default_rng(seed)
    na = max(1, n_groups // 64)
    a = rng.integers(0, na, n, dtype=np.int32)
    b = rng.integers(0, 64, n, dtype=np.int16)
    s = rng.integers(0, 10**6, n, dtype=np.int64)
    m = rng.integers(-(2**31), 2**31 - 1, n, dtype=np.int32)
    return a, b, s, m


ALNUM = np.frombuffer(b"abcdefghijklmnopqrstuvwxyz0123456789", dtype=np.uint8)


def varchar_pool(n_strings: int, rng) -> tuple[np.ndarray, np.ndarray]:
    """n_strings strings of length uniform 8..32 over [a-z0-9] → (offsets, bytes).
    Duplicates in the pool are possible (and harmless: they group together)."""
    lens = rng.integers(8, 33, n_strings)
    offs = np.zeros(n_strings + 1, dtype=np.int64)
    np.cumsum(lens, out=offs[1:])
    data = ALNUM[rng.integers(0, len(ALNUM), int(offs[-1]))]
    return offs, data


def varchar_table(n: int, n_groups: int, seed: int):
    """VARCHAR-key table: key drawn uniformly from a pool of n_groups
    strings; s INT64 uniform [0, 10^6), m INT32 uniform."""
    rng = np.random.default_rng(seed)
    poffs, pdata = varchar_pool(n_groups, rng)
    pick = rng.integers(0, n_groups, n)
    lens = poffs[pick + 1] - poffs[pick]
    offs = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(lens, out=offs[1:])
    # gather bytes of the picked strings
    starts = np.repeat(poffs[pick], lens)
    idx_in = np.arange(int(offs[-1]), dtype=np.int64) - np.repeat(offs[:-1], lens)
    data = pdata[starts + idx_in]
    s = rng.integers(0, 10**6, n, dtype=np.int64)
    m = rng.integers(-(2**31), 2**31 - 1, n, dtype=np.int32)
    return (offs, data), s, m


def batch_shapes(n_tables: int = 256, seed: int = 3, rows_exp=(4.0, 7.0), groups_exp=(2.0, 6.0),
                 varchar_frac: float = 0.25):
    """Shapes of a batch of independent GROUP BY tables: rows = floor(10^U(rows_exp)),
    groups = floor(10^U(groups_exp)) (log-uniform), a varchar_frac share of the
    tables (at seeded positions) keyed by VARCHAR, the rest by (INT32, INT16).
    Returns a list of dicts {kind, rows, groups, seed}."""
    rng = np.random.default_rng(seed)
    rows = np.floor(10 ** rng.uniform(rows_exp[0], rows_exp[1], n_tables)).astype(np.int64)
    groups = np.floor(10 ** rng.uniform(groups_exp[0], groups_exp[1], n_tables)).astype(np.int64)
    n_str = int(round(varchar_frac * n_tables))
    is_str = np.zeros(n_tables, dtype=bool)
    is_str[rng.permutation(n_tables)[:n_str]] = True
    return [dict(kind="varchar" if is_str[i] else "composite", rows=int(rows[i]), groups=int(max(1, groups[i])),
                 seed=seed * 100_003 + i) for i in range(n_tables)]


def batch_table_host(shape):
    """numpy columns of one batch table (composite: a, b, s, m; varchar:
    (offsets, bytes), s, m)."""
    if shape["kind"] == "composite":
        return list(composite(shape["rows"], shape["groups"], shape["seed"]))
    (offs, data), s, m = varchar_table(shape["rows"], shape["groups"], shape["seed"])
    return [(offs, data), s, m]


def batch_table_device(shape, device="cuda"):
    """The same table shape generated on the GPU (torch's generator: other
    values than batch_table_host, same distributions) — for full-size runs."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(shape["seed"])
    n, ng = shape["rows"], shape["groups"]
    s = torch.randint(0, 10**6, (n,), generator=g, device=device, dtype=torch.int64)
    m = torch.randint(-(2**31), 2**31 - 1, (n,), generator=g, device=device, dtype=torch.int64).to(torch.int32)
    if shape["kind"] == "composite":
        a = torch.randint(0, max(1, ng // 64), (n,), generator=g, device=device, dtype=torch.int32)
        b = torch.randint(0, 64, (n,), generator=g, device=device, dtype=torch.int16)
        return [a, b, s, m]
    rng = np.random.default_rng(shape["seed"])
    poffs, pdata = varchar_pool(ng, rng)
    poffs_d = torch.from_numpy(poffs).to(device)
    pdata_d = torch.from_numpy(pdata).to(device)
    pick = torch.randint(0, ng, (n,), generator=g, device=device, dtype=torch.int64)
    lens = poffs_d[pick + 1] - poffs_d[pick]
    offs = torch.zeros(n + 1, dtype=torch.int64, device=device)
    torch.cumsum(lens, 0, out=offs[1:])
    total = int(offs[-1].item())
    starts = torch.repeat_interleave(poffs_d[pick] - offs[:-1], lens, output_size=total)
    data = pdata_d[starts + torch.arange(total, device=device, dtype=torch.int64)]
    return [(offs, data), s, m]


BATCH_COMPOSITE = dict(col_types=[2, 1, 3, 2], group_cols=[0, 1], aggs=[("count_star", -1), ("sum", 2), ("max", 3)])
BATCH_VARCHAR = dict(col_types=[5, 3, 2], group_cols=[0], aggs=[("count_star", -1), ("sum", 1), ("max", 2)])


# ------------------------------------------------------------------ serving
# Resident tables of the served query stream: the column families of the
# plain (INT32 key, INT64 value), Zipf (INT64 key, DOUBLE value), filtered
# (dictionary-run INT32 key, INT16 filter column, INT64 value), composite
# and VARCHAR workloads, generated on the GPU (torch's generator) at
# `scale` × about 66 GB.
SERVE_TABLES = [
    dict(name="plain", family="plain", rows=500_000_000, groups=1024),
    dict(name="zipf0", family="zipf", rows=400_000_000, groups=20_000_000),
    dict(name="zipf1", family="zipf", rows=400_000_000, groups=20_000_000),
    dict(name="filter0", family="filter", rows=600_000_000, groups=65_536),
    dict(name="filter1", family="filter", rows=600_000_000, groups=65_536),
    dict(name="comp0", family="composite", rows=400_000_000, groups=1_000),
    dict(name="comp1", family="composite", rows=400_000_000, groups=30_000),
    dict(name="comp2", family="composite", rows=400_000_000, groups=1_000_000),
    dict(name="vch0", family="varchar", rows=100_000_000, groups=1_000),
    dict(name="vch1", family="varchar", rows=100_000_000, groups=100_000),
]

SERVE_TYPES = {
    "plain": [2, 3],            # k INTEGER, v BIGINT
    "zipf": [3, 4],             # k BIGINT, x DOUBLE
    "filter": [2, 1, 3],        # key INTEGER, f SMALLINT, v BIGINT
    "composite": [2, 1, 3, 2],  # a INTEGER, b SMALLINT, s BIGINT, m INTEGER
    "varchar": [5, 3, 2],       # key VARCHAR, s BIGINT, m INTEGER
}


def serve_table_device(t, scale=1.0, seed=4, device="cuda"):
    """Columns of one serving table on the GPU."""
    import torch
    n = max(1024, int(t["rows"] * scale))
    g = torch.Generator(device=device)
    g.manual_seed(seed * 1000 + SERVE_TABLES.index(t))
    fam = t["family"]
    if fam == "plain":
        k = torch.randint(0, t["groups"], (n,), generator=g, device=device, dtype=torch.int32)
        v = torch.randint(0, 10**6, (n,), generator=g, device=device, dtype=torch.int64)
        return [k, v], n
    if fam == "zipf":
        cdf = torch.from_numpy(zipf_cdf(t["groups"], 1.1)).to(device)
        k = torch.empty(n, dtype=torch.int64, device=device)
        x = torch.empty(n, dtype=torch.float64, device=device)
        step = 1 << 26
        for lo in range(0, n, step):
            hi = min(n, lo + step)
            u = torch.rand(hi - lo, generator=g, device=device, dtype=torch.float64)
            r = torch.searchsorted(cdf, u, right=True).clamp_(max=t["groups"] - 1)
            # ranks spread over [0, 2^40) by an odd multiplier (a bijection mod 2^40)
            k[lo:hi] = (r * 0x9E3779B97F4A7C15) & ((1 << 40) - 1)
            x[lo:hi] = torch.randn(hi - lo, generator=g, device=device, dtype=torch.float64) * 25 + 100
        return [k, x], n
    if fam == "filter":
        dict_vals = torch.randint(0, 2**31, (t["groups"],), generator=g, device=device, dtype=torch.int64)
        idx = torch.empty(n, dtype=torch.int64, device=device)
        pos = 0
        while pos < n:  # runs of Geometric(1/4) length, index uniform per run
            m = min(n - pos, 1 << 26)
            nr = m // 2 + 1
            lens = torch.empty(nr, device=device).geometric_(0.25, generator=g).to(torch.int64)
            vals = torch.randint(0, t["groups"], (nr,), generator=g, device=device, dtype=torch.int64)
            run = torch.repeat_interleave(vals, lens)[:m]
            idx[pos:pos + len(run)] = run
            pos += len(run)
        key = dict_vals[idx].to(torch.int32)
        del idx
        f = torch.randint(0, 1000, (n,), generator=g, device=device, dtype=torch.int16)
        v = torch.randint(-10**9, 10**9 + 1, (n,), generator=g, device=device, dtype=torch.int64)
        return [key, f, v], n
    shape = dict(kind="composite" if fam == "composite" else "varchar", rows=n, groups=t["groups"],
                 seed=seed * 1000 + SERVE_TABLES.index(t))
    return batch_table_device(shape, device=device), n


def serve_queries(duration_s, rate, rows_of, seed=4):
    """Poisson arrivals at `rate` q/s for `duration_s`; each query has the
    shape of one of the four GROUP BY workloads (uniformly chosen) over a
    random row range of a table of that family, with a WHERE clause of
    selectivity U[1%, 100%].  rows_of: table index -> resident rows."""
    from statistics import NormalDist
    rng = np.random.default_rng(seed)
    fam_tables = {}
    for i, t in enumerate(SERVE_TABLES):
        fam_tables.setdefault(t["family"], []).append(i)
    out = []
    t_at = 0.0
    while True:
        t_at += rng.exponential(1.0 / rate)
        if t_at >= duration_s:
            break
        shape = int(rng.integers(1, 5))
        sel = float(rng.uniform(0.01, 1.0))
        if shape == 1:
            ti, rows = fam_tables["plain"][0], 1_000_000
            q = dict(group_cols=[0], aggs=[("count_star", -1), ("sum", 1), ("min", 1), ("max", 1)],
                     filters=[(1, "<", int(sel * 10**6))], est_groups=1024)
        elif shape == 2:
            ti, rows = int(rng.choice(fam_tables["zipf"])), 100_000_000
            thr = 100.0 + 25.0 * NormalDist().inv_cdf(min(sel, 0.999999))
            q = dict(group_cols=[0], aggs=[("count_star", -1), ("sum", 1), ("avg", 1)],
                     filters=[(1, "<", thr)], est_groups=8_000_000)
        elif shape == 3:
            ti, rows = int(rng.choice(fam_tables["filter"])), 200_000_000
            q = dict(group_cols=[0], aggs=[("sum", 2), ("count_star", -1)],
                     filters=[(1, "<", int(sel * 1000))], est_groups=65_536)
        else:
            fam = "varchar" if rng.random() < 0.25 else "composite"
            ti = int(rng.choice(fam_tables[fam]))
            rows = int(10 ** rng.uniform(4, 7))
            spec = BATCH_VARCHAR if fam == "varchar" else BATCH_COMPOSITE
            q = dict(group_cols=spec["group_cols"], aggs=spec["aggs"],
                     filters=[(1 if fam == "varchar" else 2, "<", int(sel * 10**6))],
                     est_groups=SERVE_TABLES[ti]["groups"])
        n = rows_of[ti]
        rows = min(rows, n)
        r0 = int(rng.integers(0, n - rows + 1)) // 64 * 64
        q.update(table=ti, r0=r0, r1=r0 + rows, shape=shape, at=t_at)
        out.append(q)
    return out
