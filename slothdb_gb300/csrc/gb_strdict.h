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

__device__ __forceinline__ u64 str_hash(const uint8_t *p, u32 len) {
    // FNV-1a over 8-byte words, then the 64-bit finaliser
    u64 h = 0xcbf29ce484222325ull ^ ((u64)len * 0x9e3779b97f4a7c15ull);
    u32 i = 0;
    for (; i + 8 <= len; i += 8) {
        u64 w = 0;
#pragma unroll
        for (int b = 0; b < 8; b++) w |= (u64)p[i + b] << (8 * b);
        h = (h ^ w) * 0x100000001b3ull;
    }
    u64 w = 0;
    for (u32 b = 0; i + b < len; b++) w |= (u64)p[i + b] << (8 * b);
    h = (h ^ w) * 0x100000001b3ull;
    return mix64(h);
}

__device__ __forceinline__ bool bytes_equal(const uint8_t *a, const uint8_t *b, u32 len) {
    for (u32 i = 0; i < len; i++)
        if (a[i] != b[i]) return false;
    return true;
}

// Returns the slot index (= string id), or -1 if the probe bound was reached
// (table too full) or the arena is exhausted, or -2 on a timeout.
__device__ __forceinline__ long long strdict_find_or_insert(const StrDictRef &D, const uint8_t *s, u32 len, u64 h, u32 *new_strs) {
    u64 slot = h & (D.cap - 1);
    for (int p = 0; p < D.max_probe; p++) {
        u64 *hk = D.hash + slot;
        u64 k = *(volatile u64 *)hk;
        if (k == EMPTY_KEY) {
            const u64 old = atomicCAS(hk, EMPTY_KEY, h == EMPTY_KEY ? h ^ 1ull : h);
            if (old == EMPTY_KEY) {
                // claimed: copy the bytes into the arena, assign the id, then
                // publish ref (readers wait for it)
                const u64 off = atomicAdd(D.arena_used, (u64)len);
                if (off + len > D.arena_cap || len >= (1u << 24)) {
                    // dead slot: an offset past the arena never matches
                    atomicExch(D.ref + slot, (DEAD_OFF << 24) | (u64)len);
                    return -1;
                }
                for (u32 i = 0; i < len; i++) D.arena[off + i] = s[i];
                const u64 id = atomicAdd(D.next_id, 1ull);
                const u64 rv = (off << 24) | (u64)len;
                D.id[slot] = id;
                D.ref_by_id[id] = rv;
                __threadfence();
                atomicExch(D.ref + slot, rv);
                atomicAdd(new_strs, 1u);
                return (long long)id;
            }
            k = old;
        }
        if (k == (h == EMPTY_KEY ? h ^ 1ull : h)) {
            u64 r = *(volatile u64 *)(D.ref + slot);
            int spin = 0;
            while (r == REF_PENDING) {
                if (++spin > SPIN_LIMIT) {
                    atomicOr(D.err, (u32)ERR_TIMEOUT);
                    return -2;
                }
                __nanosleep(32);
                r = *(volatile u64 *)(D.ref + slot);
            }
            __threadfence();
            const u32 rlen = (u32)(r & 0xffffffu);
            const u64 roff = r >> 24;
            if (rlen == len && roff + rlen <= D.arena_cap && bytes_equal(D.arena + roff, s, len))
                return (long long)*(volatile u64 *)(D.id + slot);
        }
        slot = (slot + 1) & (D.cap - 1);
    }
    return -1;
}


gb_status strdict_launch_encode(const StrDictRef &D, const uint8_t *bytes, const int64_t *offsets, int64_t off_base,
                                const uint64_t *valid, u64 n, const u32 *rows, long long *ids, u32 *retry, u32 *retry_n,
                                u32 *new_strs, cudaStream_t st);
gb_status strdict_launch_rehash(const u64 *old_hash, const u64 *old_ref, const u64 *old_id, u64 old_cap,
                                const StrDictRef &D, cudaStream_t st);
gb_status strdict_fill(u64 *p, u64 n, u64 v, cudaStream_t st);
gb_status strdict_launch_lengths(const StrDictRef &D, const long long *ids, u64 n, int64_t *lens, cudaStream_t st);
gb_status strdict_launch_gather(const StrDictRef &D, const long long *ids, u64 n, const int64_t *offs, uint8_t *out,
                                cudaStream_t st);
gb_status device_exclusive_scan(const int64_t *lens, int64_t *offs, u64 n, int64_t *tmp, cudaStream_t st,
                                int64_t *total);

}  // namespace gb
