// gb_strdict.h — host interface of the device string dictionary.
#pragma once
#include "gb_kernels.cuh"

namespace gb {

struct StrDictRef {
    u64 *hash;        // cap slots (EMPTY_KEY = free)
    u64 *ref;         // cap slots: (arena offset << 24) | length, ~0 = being published
    u64 *id;          // cap slots: dense id of the slot's string
    u64 *ref_by_id;   // refs indexed by id (for emitting strings)
    u64 *next_id;     // id counter
    u64 cap;          // power of two
    uint8_t *arena;
    u64 arena_cap;
    u64 *arena_used;
    u32 *err;
    int32_t max_probe;
};

constexpr u64 REF_PENDING = ~0ull;
constexpr u64 DEAD_OFF = (1ull << 40) - 1;
constexpr int SPIN_LIMIT = 1 << 20;

// Bytes [8j, 8j+8) of the string at p (little-endian, zero past len), read
// with aligned 8-byte loads of only the words that hold bytes of the string
// (an aligned word never crosses a page, so nothing outside the pages of the
// string is touched).
__device__ __forceinline__ u64 str_chunk(const uint8_t *p, u32 len, u32 j) {
    const uintptr_t a = (uintptr_t)p + 8u * j;
    const u32 nb = min(8u, len - 8u * j);
    const u64 *w = (const u64 *)(a & ~(uintptr_t)7);
    const u32 lo = (u32)(a & 7);
    u64 v = __ldg(w) >> (8 * lo);
    if (lo && lo + nb > 8) v |= __ldg(w + 1) << (64 - 8 * lo);
    if (nb < 8) v &= (1ull << (8 * nb)) - 1ull;
    return v;
}

// FNV-1a over the 8-byte chunks (one final step for the partial, possibly
// empty, last chunk), then the 64-bit finaliser.
__device__ __forceinline__ u64 str_hash(const uint8_t *p, u32 len) {
    u64 h = 0xcbf29ce484222325ull ^ ((u64)len * 0x9e3779b97f4a7c15ull);
    const u32 full = len >> 3;
    for (u32 j = 0; j < full; j++) h = (h ^ str_chunk(p, len, j)) * 0x100000001b3ull;
    const u64 tail = (len & 7) ? str_chunk(p, len, full) : 0ull;
    h = (h ^ tail) * 0x100000001b3ull;
    return mix64(h);
}

__device__ __forceinline__ u64 dict_hash_value(u64 h) { return h == EMPTY_KEY ? h ^ 1ull : h; }

// Arena entries start at 8-byte offsets and hold the string's chunks (zero
// padded), so a comparison is one aligned load per chunk.
__device__ __forceinline__ bool arena_equal(const StrDictRef &D, u64 r, const uint8_t *s, u32 len) {
    const u32 rlen = (u32)(r & 0xffffffu);
    const u64 roff = r >> 24;
    if (rlen != len || roff + ((len + 7u) & ~7u) > D.arena_cap) return false;
    const u64 *aw = (const u64 *)(D.arena + roff);
    const u32 nc = (len + 7) >> 3;
    for (u32 j = 0; j < nc; j++)
        if (aw[j] != str_chunk(s, len, j)) return false;
    return true;
}

// Write the string into its arena entry, then its id, then publish the ref.
__device__ __forceinline__ void strdict_publish(const StrDictRef &D, u64 slot, const uint8_t *s, u32 len, u64 off,
                                                u64 id) {
    u64 *aw = (u64 *)(D.arena + off);
    const u32 nc = (len + 7) >> 3;
    for (u32 j = 0; j < nc; j++) aw[j] = str_chunk(s, len, j);
    const u64 rv = (off << 24) | (u64)len;
    D.id[slot] = id;
    D.ref_by_id[id] = rv;
    __threadfence();
    atomicExch((unsigned long long *)(D.ref + slot), (unsigned long long)rv);
}

__device__ __forceinline__ void strdict_kill(const StrDictRef &D, u64 slot, u32 len) {
    atomicExch((unsigned long long *)(D.ref + slot), (unsigned long long)((DEAD_OFF << 24) | (u64)len));
}

// Acquire load of a published ref (orders the later arena / id reads after it).
__device__ __forceinline__ u64 ld_acquire(const u64 *p) {
    u64 v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Bounded wait for a claimed slot's ref; REF_PENDING after the limit.
__device__ __forceinline__ u64 strdict_wait_ref(const StrDictRef &D, u64 slot) {
    u64 r = ld_acquire(D.ref + slot);
    int spin = 0;
    while (r == REF_PENDING) {
        if (++spin > SPIN_LIMIT) {
            atomicOr(D.err, (u32)ERR_TIMEOUT);
            return REF_PENDING;
        }
        __nanosleep(32);
        r = ld_acquire(D.ref + slot);
    }
    return r;
}

// One thread: find the string's id or insert it, probing from probe step p0.
// Returns the id, -1 if the probe bound was reached (table too full) or the
// arena is exhausted, or -2 on a timeout.  A thread holds a claimed slot only
// between its CAS and its publish, and never waits in between.
__device__ __forceinline__ long long strdict_find_or_insert(const StrDictRef &D, const uint8_t *s, u32 len, u64 h,
                                                            u32 *new_strs, int p0 = 0) {
    const u64 hv = dict_hash_value(h);
    u64 slot = (h + (u64)p0) & (D.cap - 1);
    for (int p = p0; p < D.max_probe; p++) {
        u64 *hk = D.hash + slot;
        u64 k = *(volatile u64 *)hk;
        if (k == EMPTY_KEY) {
            const u64 old = atomicCAS((unsigned long long *)hk, EMPTY_KEY, hv);
            if (old == EMPTY_KEY) {
                const u64 plen = (len + 7u) & ~7u;
                const u64 off = atomicAdd((unsigned long long *)D.arena_used, (unsigned long long)plen);
                if (off + plen > D.arena_cap || len >= (1u << 24)) {
                    strdict_kill(D, slot, len);  // an offset past the arena never matches
                    return -1;
                }
                const u64 id = atomicAdd((unsigned long long *)D.next_id, 1ull);
                strdict_publish(D, slot, s, len, off, id);
                atomicAdd(new_strs, 1u);
                return (long long)id;
            }
            k = old;
        }
        if (k == hv) {
            const u64 r = strdict_wait_ref(D, slot);
            if (r == REF_PENDING) return -2;
            if (arena_equal(D, r, s, len)) return (long long)*(volatile u64 *)(D.id + slot);
        }
        slot = (slot + 1) & (D.cap - 1);
    }
    return -1;
}

// A string of at most 32 bytes held as four zero-padded chunks in registers
// (read with at most five aligned 8-byte loads).
constexpr u32 SHORT_STR = 32;

__device__ __forceinline__ void short_chunks(const uint8_t *p, u32 len, u64 c[4]) {
    const uintptr_t a = (uintptr_t)p;
    const u64 *w = (const u64 *)(a & ~(uintptr_t)7);
    const u32 nw = len ? (u32)(((a + len - 1) >> 3) - (a >> 3) + 1) : 0u;
    u64 x[5];
#pragma unroll
    for (int i = 0; i < 5; i++) x[i] = (u32)i < nw ? __ldg(w + i) : 0ull;
    const u32 sh = 8u * (u32)(a & 7);
#pragma unroll
    for (int j = 0; j < 4; j++) {
        u64 v = sh ? ((x[j] >> sh) | (x[j + 1] << (64 - sh))) : x[j];
        const int nb = (int)len - 8 * j;
        v = nb >= 8 ? v : (nb <= 0 ? 0ull : (v & ((1ull << (8 * nb)) - 1ull)));
        c[j] = v;
    }
}

// str_hash of a short string from its chunks (same value).
__device__ __forceinline__ u64 short_hash(const u64 c[4], u32 len) {
    u64 h = 0xcbf29ce484222325ull ^ ((u64)len * 0x9e3779b97f4a7c15ull);
    const u32 full = len >> 3;
#pragma unroll
    for (u32 j = 0; j < 4; j++)
        if (j < full) h = (h ^ c[j]) * 0x100000001b3ull;
    u64 tail = 0;
#pragma unroll
    for (u32 j = 0; j < 4; j++)
        if (j == full) tail = c[j];
    h = (h ^ tail) * 0x100000001b3ull;  // a whole last chunk leaves tail = 0 (c[j] beyond len is 0)
    return mix64(h);
}

__device__ __forceinline__ bool short_arena_equal(const StrDictRef &D, u64 r, const u64 c[4], u32 len) {
    const u32 rlen = (u32)(r & 0xffffffu);
    const u64 roff = r >> 24;
    if (rlen != len || roff + ((len + 7u) & ~7u) > D.arena_cap) return false;
    const u64 *aw = (const u64 *)(D.arena + roff);
    const u32 nc = (len + 7) >> 3;
    bool eq = true;
#pragma unroll
    for (u32 j = 0; j < 4; j++)
        if (j < nc) eq &= aw[j] == c[j];
    return eq;
}

// Warp-cooperative encode, one row per lane (all 32 lanes call it; `act`
// marks lanes with a row).  Lanes with equal hashes elect a leader that
// probes; the warp's new strings take their arena bytes and ids with one
// atomic each per warp and are published before any lane of the warp waits
// on a slot another warp has claimed but not yet published — so no two warps
// can wait on each other.  Followers check they hold the leader's bytes (a
// hash collision falls back to the one-thread path).  Strings of at most 32
// bytes stay in registers; longer ones are re-read chunk by chunk.
// Returns as strdict_find_or_insert.
__device__ __forceinline__ long long strdict_warp_encode(const StrDictRef &D, const uint8_t *s, u32 len, bool act,
                                                         u32 *new_strs) {
    const int lane = threadIdx.x & 31;
    const bool shrt = len <= SHORT_STR;
    u64 c[4] = {0ull, 0ull, 0ull, 0ull};
    u64 h = 0;
    if (act) {
        if (shrt) {
            short_chunks(s, len, c);
            h = short_hash(c, len);
        } else {
            h = str_hash(s, len);
        }
    }
    const unsigned am = __ballot_sync(0xffffffffu, act);
    const unsigned peers = __match_any_sync(0xffffffffu, h) & am;
    const int lead = act ? __ffs(peers) - 1 : lane;
    const bool leader = act && lead == lane;
    // phase 1 (leaders): probe without waiting
    long long id = -1;
    long long claimed = -1, waitslot = -1;
    int waitp = 0;
    if (leader) {
        const u64 hv = dict_hash_value(h);
        u64 slot = h & (D.cap - 1);
        for (int p = 0; p < D.max_probe; p++) {
            u64 *hk = D.hash + slot;
            u64 k = *(volatile u64 *)hk;
            // the slot's ref is loaded beside its key (the acquire orders the
            // arena and id loads after it), so a hit costs two round trips:
            // key + ref, then arena bytes + id
            u64 r = ld_acquire(D.ref + slot);
            if (k == EMPTY_KEY) {
                const u64 old = atomicCAS((unsigned long long *)hk, EMPTY_KEY, hv);
                if (old == EMPTY_KEY) {
                    claimed = (long long)slot;
                    break;
                }
                k = old;
                r = ld_acquire(D.ref + slot);  // claimed by another thread meanwhile
            }
            if (k == hv) {
                if (r == REF_PENDING) {
                    waitslot = (long long)slot;
                    waitp = p;
                    break;
                }
                const long long sid = (long long)D.id[slot];  // written before the ref was published
                if (shrt ? short_arena_equal(D, r, c, len) : arena_equal(D, r, s, len)) {
                    id = sid;
                    break;
                }
            }
            slot = (slot + 1) & (D.cap - 1);
        }
    }
    // phase 2 (warp): arena bytes, then ids, for every claimed slot; publish
    const bool need = claimed >= 0;
    const unsigned needm = __ballot_sync(0xffffffffu, need);
    if (needm) {
        const u32 plen = need ? ((len + 7u) & ~7u) : 0u;
        u64 incl = plen;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u64 y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const u64 total = __shfl_sync(0xffffffffu, incl, 31);
        u64 base = 0;
        if (lane == 0) base = atomicAdd((unsigned long long *)D.arena_used, (unsigned long long)total);
        base = __shfl_sync(0xffffffffu, base, 0);
        const u64 off = base + incl - plen;
        const bool ok = need && off + plen <= D.arena_cap && len < (1u << 24);
        const unsigned okm = __ballot_sync(0xffffffffu, ok);
        u64 idb = 0;
        if (lane == 0 && okm) idb = atomicAdd((unsigned long long *)D.next_id, (unsigned long long)__popc(okm));
        idb = __shfl_sync(0xffffffffu, idb, 0);
        if (ok) {
            id = (long long)(idb + __popc(okm & ((1u << lane) - 1u)));
            strdict_publish(D, (u64)claimed, s, len, off, (u64)id);
        } else if (need) {
            strdict_kill(D, (u64)claimed, len);
            id = -1;
        }
        if (lane == 0 && okm) atomicAdd(new_strs, (u32)__popc(okm));
    }
    // phase 3 (leaders): wait for slots claimed by other warps
    if (waitslot >= 0) {
        const u64 r = strdict_wait_ref(D, (u64)waitslot);
        if (r == REF_PENDING) id = -2;
        else if (shrt ? short_arena_equal(D, r, c, len) : arena_equal(D, r, s, len)) id = (long long)D.id[waitslot];
        else id = strdict_find_or_insert(D, s, len, h, new_strs, waitp + 1);
    }
    // followers take the leader's id when they hold the same bytes
    const long long lid = __shfl_sync(0xffffffffu, id, lead);
    const u32 llen = __shfl_sync(0xffffffffu, len, lead);
    u64 lc[4];
#pragma unroll
    for (int j = 0; j < 4; j++) lc[j] = __shfl_sync(0xffffffffu, c[j], lead);
    const uint8_t *ls = (const uint8_t *)__shfl_sync(0xffffffffu, (unsigned long long)(uintptr_t)s, lead);
    if (act && !leader) {
        bool same = llen == len;
        if (same && shrt) {
#pragma unroll
            for (int j = 0; j < 4; j++) same &= lc[j] == c[j];
        } else {
            for (u32 j = 0; same && j < ((len + 7) >> 3); j++) same = str_chunk(s, len, j) == str_chunk(ls, len, j);
        }
        id = same ? lid : strdict_find_or_insert(D, s, len, h, new_strs);
    }
    return id;
}


gb_status strdict_launch_encode(const StrDictRef &D, const uint8_t *bytes, const int64_t *offsets, int64_t off_base,
                                const uint64_t *valid, u64 n, const u32 *rows, long long *ids, u32 *retry, u32 *retry_n,
                                u32 *new_strs, cudaStream_t st);
gb_status strdict_launch_rehash(const u64 *old_hash, const u64 *old_ref, const u64 *old_id, u64 old_cap,
                                const StrDictRef &D, cudaStream_t st);
gb_status strdict_fill(u64 *p, u64 n, u64 v, cudaStream_t st);
gb_status strdict_launch_lengths(const StrDictRef &D, const long long *ids, u64 n, int64_t *lens, cudaStream_t st,
                                 uint64_t *valid = nullptr);
gb_status strdict_launch_gather(const StrDictRef &D, const long long *ids, u64 n, const int64_t *offs, uint8_t *out,
                                cudaStream_t st);
gb_status device_exclusive_scan(const int64_t *lens, int64_t *offs, u64 n, int64_t *tmp, cudaStream_t st,
                                int64_t *total);

}  // namespace gb
