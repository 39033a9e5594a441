// gb_internal.cuh — device/host internals shared by the GROUP BY kernels.
//
// Hash-table layout (HBM): a power-of-two array of slots, each `stride`
// 64-bit words: word 0 = packed group key (EMPTY_KEY = free), words
// 1..words = aggregate state words.  State word 0 is always the row count
// of the group (COUNT(*) reads it; it also marks the two out-of-band slots
// cap+0 = "key equals EMPTY_KEY" and cap+1 = "NULL key" as used).
//
// The per-group state is the GPU restatement of the reference's AggState
// (src/execution/physical_planner.cpp:6080-6128): count, sum, min, max.
// Integer sums/min/max are int64 words (exact), DOUBLE sums are IEEE double
// words, DOUBLE min/max use an order-preserving int64 encoding so that
// atomicMin/atomicMax on int64 order them like doubles.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "../../include/slothdb_gb300.h"

#define GB_MAX_COLS 16
#define GB_MAX_OPS 12
#define GB_MAX_FILTERS 8
#define GB_MAX_WORDS 16
#define GB_MAX_AGGS 16

namespace gb {

typedef unsigned long long u64;
typedef long long i64;
typedef unsigned int u32;

constexpr u64 EMPTY_KEY = 0x8000000000000000ull;
constexpr unsigned FULL = 0xffffffffu;

// Device error flags (bitwise OR into a device word, read by the host).
enum ErrFlag : u32 {
    ERR_SPILL_OVERFLOW = 1u,
    ERR_NULL_IN_WIDE_KEY = 2u,
    ERR_TIMEOUT = 4u,
    ERR_CORRUPT = 8u,
    ERR_OUT_OVERFLOW = 16u,
};

enum OpKind : uint8_t {
    OP_NONE = 0,
    OP_ADD_I = 1,   // int64 sum
    OP_ADD_F = 2,   // double sum
    OP_MIN_I = 3,
    OP_MAX_I = 4,
    OP_MIN_F = 5,   // ordered-int64-encoded double
    OP_MAX_F = 6,
    OP_CNT_NN = 7,  // count of non-NULL values of a column
    OP_DIST = 8,    // distinct non-NULL values: contributes 1 per new (group, value) pair
};

enum KeyMode : int32_t {
    KEY_SINGLE = 0,  // one SMALLINT/INTEGER/BIGINT key, sign-extended
    KEY_PACKED = 1,  // two keys of <= 32+16 bits packed, NULL flags in spare bits
    KEY_WIDE = 2,    // two 32-bit keys packed into 64 bits (no NULLs allowed)
    KEY_STRING = 3,  // VARCHAR key (dictionary-encoded to ids first)
};

struct DevCol {
    const void *data;
    const uint64_t *valid;
    const int64_t *offsets;
    int32_t type;
    int32_t pad;
};

struct Op {
    uint8_t kind;
    uint8_t col;
    uint8_t word;  // state word index (1..words-1)
    uint8_t dset;  // OP_DIST: index of the op's pair set
};

struct Filter {
    int32_t col;
    int32_t op;
    int64_t ic;
    double dc;
    const void *ptr;  // device copy of an IN set (sorted int64) or a string literal
    u64 n;            // its members / bytes
};

struct Plan {
    DevCol cols[GB_MAX_COLS];
    Filter filters[GB_MAX_FILTERS];
    Op ops[GB_MAX_OPS];
    int32_t n_cols, n_filters, n_ops;
    int32_t n_keys;
    int32_t key_col[2];
    int32_t key_type[2];
    int32_t key_mode;
    int32_t key_bits_b;   // KEY_PACKED: width of the second key
    int32_t key_bits_a;   // KEY_PACKED: width of the first key
    int32_t words;        // state words (word 0 = row count)
    int32_t stride;       // words per table slot incl. key, power of two
    int32_t n_dist;       // OP_DIST ops (COUNT(DISTINCT) columns)
    int32_t dnarrow;      // 1: pair sets of 8-byte slots (a non-NULL 16/32-bit key, 16/32-bit values)
    int32_t str_key;      // a pair key's VARCHAR position (its 32-bit string ids are packed), -1: none
    uint64_t word_init[GB_MAX_WORDS];
    // COUNT(DISTINCT): per OP_DIST op a set of (group key, value) pairs,
    // 16-byte slots (8-byte when dnarrow) of which dmask + 1 per set; the
    // NULL-key group of a nullable BIGINT key keeps its pairs in twin sets
    // (null_sets, or null)
    u64 *dsets;
    u64 *null_sets;
    unsigned long long *dmeta;  // [0] pairs inserted, [1] overflow flag, [2 + d] marker pair of set d seen
    u64 dmask;
};

// --------------------------------------------------------------- device utils
// Hint: start pulling [p, p + bytes) into L2 with one bulk prefetch (no data
// returned, nothing to wait for).  Skipped unless p is 16-byte aligned; the
// size is rounded down to 16 bytes, so the range never leaves [p, p + bytes).
__device__ __forceinline__ void l2_prefetch(const void *p, u64 bytes) {
    if ((((u64)p) & 15) || bytes < 16) return;
    if (bytes > (1ull << 30)) bytes = 1ull << 30;
    u64 g;
    asm("cvta.to.global.u64 %0, %1;" : "=l"(g) : "l"(p));
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(g), "r"((unsigned)(bytes & ~15ull)) : "memory");
}

__device__ __forceinline__ u64 mix64(u64 k) {
    // murmur3 fmix64 finaliser
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

__host__ __device__ __forceinline__ i64 enc_f64(double d) {
#ifdef __CUDA_ARCH__
    i64 b = __double_as_longlong(d);
#else
    i64 b;
    memcpy(&b, &d, 8);
#endif
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffll);
}

__host__ __device__ __forceinline__ double dec_f64(i64 e) {
    i64 b = e >= 0 ? e : (e ^ 0x7fffffffffffffffll);
#ifdef __CUDA_ARCH__
    return __longlong_as_double(b);
#else
    double d;
    memcpy(&d, &b, 8);
    return d;
#endif
}

__device__ __forceinline__ bool row_valid(const uint64_t *v, u64 r) {
    return v == nullptr || ((__ldg(v + (r >> 6)) >> (r & 63)) & 1ull);
}

// Load column value as int64 (integer types) — type is warp-uniform.
__device__ __forceinline__ i64 load_int(const DevCol &c, u64 r) {
    switch (c.type) {
    case GB_T_SMALLINT: return (i64)__ldg((const int16_t *)c.data + r);
    case GB_T_INTEGER: return (i64)__ldg((const int32_t *)c.data + r);
    case GB_T_BIGINT: return (i64)__ldg((const long long *)c.data + r);
    default: return 0;
    }
}

__device__ __forceinline__ double load_f64(const DevCol &c, u64 r) {
    return __ldg((const double *)c.data + r);
}

__device__ __forceinline__ bool cmp_i(int op, i64 a, i64 b) {
    switch (op) {
    case GB_CMP_EQ: return a == b;
    case GB_CMP_NE: return a != b;
    case GB_CMP_LT: return a < b;
    case GB_CMP_LE: return a <= b;
    case GB_CMP_GT: return a > b;
    default: return a >= b;
    }
}

__device__ __forceinline__ bool cmp_f(int op, double a, double b) {
    switch (op) {
    case GB_CMP_EQ: return a == b;
    case GB_CMP_NE: return a != b;
    case GB_CMP_LT: return a < b;
    case GB_CMP_LE: return a <= b;
    case GB_CMP_GT: return a > b;
    default: return a >= b;
    }
}

// Membership of x in a sorted int64 set of n members (IN).
__device__ __forceinline__ bool in_set(const void *set, u64 n, i64 x) {
    const long long *a = (const long long *)set;
    u64 lo = 0, hi = n;  // first member >= x
    while (lo < hi) {
        const u64 mid = (lo + hi) >> 1;
        if (__ldg(a + mid) < x) lo = mid + 1;
        else hi = mid;
    }
    return lo < n && __ldg(a + lo) == x;
}

// A VARCHAR predicate on the bytes s[0, len): = / <> the literal, or LIKE /
// NOT LIKE '%needle%' (byte substring; an empty needle is in every string).
__device__ __forceinline__ bool str_pred(int op, const uint8_t *s, u64 len, const void *lit_, u64 n) {
    const uint8_t *lit = (const uint8_t *)lit_;
    if (op == GB_CMP_STR_EQ || op == GB_CMP_STR_NE) {
        bool eq = len == n;
        for (u64 i = 0; eq && i < n; i++) eq = s[i] == __ldg(lit + i);
        return (op == GB_CMP_STR_EQ) == eq;
    }
    bool found = n == 0;
    for (u64 i = 0; !found && i + n <= len; i++) {
        bool m = true;
        for (u64 k = 0; m && k < n; k++) m = s[i + k] == __ldg(lit + k);
        found = m;
    }
    return (op == GB_CMP_LIKE) == found;
}

// Combine two partial values of one op (registers, no atomics).
__device__ __forceinline__ u64 op_combine(int kind, u64 a, u64 b) {
    switch (kind) {
    case OP_ADD_F:
        return (u64)__double_as_longlong(__longlong_as_double((i64)a) + __longlong_as_double((i64)b));
    case OP_MIN_I:
    case OP_MIN_F:
        return (i64)a < (i64)b ? a : b;
    case OP_MAX_I:
    case OP_MAX_F:
        return (i64)a > (i64)b ? a : b;
    default:  // ADD_I, CNT_NN
        return a + b;
    }
}

// Atomically fold a partial value into a state word (shared or global).
__device__ __forceinline__ void op_apply(int kind, u64 *w, u64 v, u64 ident) {
    if (v == ident) return;
    switch (kind) {
    case OP_ADD_F: atomicAdd((double *)w, __longlong_as_double((i64)v)); break;
    case OP_MIN_I:
    case OP_MIN_F: atomicMin((long long *)w, (long long)v); break;
    case OP_MAX_I:
    case OP_MAX_F: atomicMax((long long *)w, (long long)v); break;
    default: atomicAdd(w, v); break;
    }
}

}  // namespace gb

// ----------------------------------------------------------------- host side
#ifndef __CUDACC_RTC__
#include <string>
namespace gb {
void set_error(const char *fmt, ...);
gb_status cuda_fail(cudaError_t e, const char *what);
int sm_count();
}  // namespace gb

#define GB_CUDA(call)                                          \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return gb::cuda_fail(e_, #call); \
    } while (0)
#endif
