"""The allocation-free entry point (gb_hash_aggregate_noalloc).

It serves callers that cannot allocate device memory during a query (an
engine that hands out device memory only from its own pre-reserved arena,
or a plugin host that forbids allocation inside operator calls): every
buffer it touches is either the caller's or fixed scratch inside the
library.  This file is collected last so that a run stopping at the first
failure has already run every other test.  The test calls the entry point
through the C ABI twice in a row, on different inputs (the second call must
not see the first call's groups in the shared scratch), and compares each
result with the ordinary allocating entry point (gb_agg_*), exactly, since
every output is an integer.
"""
import ctypes as C

import numpy as np
import pytest

from slothdb_gb300 import capi

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("gblib")]


def _allocating(keys, vals):
    g = capi.GroupBy([capi.BIGINT, capi.BIGINT], [0], [("sum", 1), ("count_star", -1)])
    try:
        g.ingest([keys, vals])
        g.finalize()
        r = g.result()
    finally:
        g.close()
    return r[0][0], r[1][0], r[2][0]


def _noalloc(lib, keys, vals, cap):
    import torch
    dk = torch.from_numpy(keys).cuda()
    dv = torch.from_numpy(vals).cuda()
    ok = torch.empty(cap, dtype=torch.int64, device="cuda")
    os_ = torch.empty(cap, dtype=torch.int64, device="cuda")
    oc = torch.empty(cap, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    n = C.c_uint64()
    capi.check(lib.gb_hash_aggregate_noalloc(dk.data_ptr(), dv.data_ptr(), len(keys), ok.data_ptr(),
                                             os_.data_ptr(), oc.data_ptr(), cap, C.byref(n), None))
    m = n.value
    return ok[:m].cpu().numpy(), os_[:m].cpu().numpy(), oc[:m].cpu().numpy()


def _same(a, b):
    oa, ob = np.argsort(a[0]), np.argsort(b[0])
    for x, y in zip(a, b):
        assert np.array_equal(x[oa], y[ob])


def test_noalloc_matches_allocating_path_two_calls(gblib):
    rng = np.random.default_rng(21)
    k1 = rng.integers(-(2**40), 2**40, 60_000, dtype=np.int64)[rng.integers(0, 60_000, 1_000_000)]
    v1 = rng.integers(-10**9, 10**9, 1_000_000, dtype=np.int64)
    k2 = rng.integers(0, 777, 300_000, dtype=np.int64)
    v2 = rng.integers(0, 10**6, 300_000, dtype=np.int64)
    cap = 131072
    r1 = _noalloc(gblib, k1, v1, cap)
    _same(r1, _allocating(k1, v1))
    r2 = _noalloc(gblib, k2, v2, cap)
    assert len(r2[0]) == 777
    _same(r2, _allocating(k2, v2))


def test_noalloc_rejects_sizes_beyond_limit(gblib):
    n = C.c_uint64()
    st = gblib.gb_hash_aggregate_noalloc(C.c_void_p(8), C.c_void_p(8), 10, C.c_void_p(8), C.c_void_p(8),
                                         C.c_void_p(8), 131073, C.byref(n), None)
    assert st == 1
    assert b"131072" in gblib.gb_last_error()


def _fmix64_inverse(h):
    """Keys whose murmur3 fmix64 hash is h (the hash is a bijection)."""
    m = np.uint64(0xFFFFFFFFFFFFFFFF)
    c1_inv = np.uint64(pow(0xff51afd7ed558ccd, -1, 1 << 64))
    c2_inv = np.uint64(pow(0xc4ceb9fe1a85ec53, -1, 1 << 64))
    k = h.astype(np.uint64)
    with np.errstate(over="ignore"):
        k ^= k >> np.uint64(33)
        k = (k * c2_inv) & m
        k ^= k >> np.uint64(33)
        k = (k * c1_inv) & m
        k ^= k >> np.uint64(33)
    return k.view(np.int64)


def test_noalloc_edges(gblib):
    """INT64_MIN (the table's empty marker) and INT64_MAX as keys; exactly
    GB_NOALLOC_MAX_GROUPS groups; one group more is refused; keys whose
    hashes all land on one slot (probe runs past the bound spill, and the
    spilled records fold back into the table)."""
    rng = np.random.default_rng(22)
    lo, hi = np.iinfo(np.int64).min, np.iinfo(np.int64).max
    k = np.concatenate([np.array([lo, hi, lo, 0, -1], dtype=np.int64), rng.integers(0, 50, 10_000)])
    v = rng.integers(-10**6, 10**6, len(k), dtype=np.int64)
    _same(_noalloc(gblib, k, v, 1000), _allocating(k, v))
    k = rng.permutation(np.arange(131_072, dtype=np.int64) * 7919 - 2**50)
    k = np.concatenate([k, k[:50_000]])
    v = rng.integers(0, 1000, len(k), dtype=np.int64)
    r = _noalloc(gblib, k, v, 131_072)
    assert len(r[0]) == 131_072
    _same(r, _allocating(k, v))
    k2 = np.concatenate([k, np.array([2**51 + 3], dtype=np.int64)])
    with pytest.raises(capi.GbError) as e:
        _noalloc(gblib, k2, np.ones(len(k2), dtype=np.int64), 131_072)
    assert e.value.status == capi.GB_ERR_UNSUPPORTED
    # 6000 keys on one slot of the 2^18-slot table (low 18 hash bits equal)
    h = (np.arange(6000, dtype=np.uint64) << np.uint64(18)) | np.uint64(777)
    k = _fmix64_inverse(h)
    k = np.repeat(k, 3)
    v = rng.integers(-10**6, 10**6, len(k), dtype=np.int64)
    r = _noalloc(gblib, k, v, 10_000)
    assert len(r[0]) == 6000
    _same(r, _allocating(k, v))
    # the next call starts from a clear table
    _same(_noalloc(gblib, k[:30], v[:30], 100), _allocating(k[:30], v[:30]))
