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
