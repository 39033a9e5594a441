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
