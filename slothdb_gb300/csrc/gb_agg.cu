// gb_agg.cu — single-query GROUP BY on GB300: plan compilation, the
// persistent hash-aggregation kernel, table growth, result compaction
// (emit), the fused TopN select, and the C ABI of include/slothdb_gb300.h.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "gb_agg_host.h"
#include "gb_kernels.cuh"
#include "gb_radix.h"
#include "gb_strdict.h"

namespace gb {

// ----------------------------------------------------------------- errors
static thread_local std::string g_err;

void set_error(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
}

gb_status cuda_fail(cudaError_t e, const char *what) {
    set_error("CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), what);
    if (e == cudaErrorMemoryAllocation) return GB_ERR_OOM;
    return GB_ERR_CUDA;
}

int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

// ================================================================ kernels
__global__ void k_table_init(u64 *slots, u64 nslots, int stride, const __grid_constant__ Plan P) {
    u64 total = nslots * (u64)stride;
    for (u64 i = blockIdx.x * (u64)blockDim.x + threadIdx.x; i < total; i += (u64)gridDim.x * blockDim.x) {
        int w = (int)(i % (u64)stride);
        u64 v;
        if (w == 0) v = EMPTY_KEY;
        else if (w - 1 < P.words) v = P.word_init[w - 1];
        else v = 0;
        slots[i] = v;
    }
}

struct IngestArgs {
    u64 n_rows;
    u32 tile_rows;
    u32 n_tiles;      // tiles remaining from first_tile
    u32 first_tile;
    int32_t smem_slots;
    int32_t smem_probe;
    int32_t pad;
};

// Persistent ingest: CTAs claim tiles of rows until none are left or the
// spill buffer nears its threshold (then the host grows the table, merges
// the spill records and relaunches from the first unclaimed tile).
template <bool PRECOMBINE>
__global__ void __launch_bounds__(512) k_ingest(const __grid_constant__ Plan P, const TableRef T, const IngestArgs A) {
    extern __shared__ u64 smem[];
    __shared__ u32 s_tile;
    __shared__ u32 s_new;
    __shared__ u32 s_pairs;
    SmemTable sm;
    sm.S = A.smem_slots;
    sm.probe = A.smem_probe;
    sm.keys = smem;
    sm.st = smem + sm.S;
    if (threadIdx.x == 0) s_new = s_pairs = 0;
    smem_init(P, sm);
    __syncthreads();
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (;;) {
        if (threadIdx.x == 0) {
            u32 t = ~0u;
            if (*(volatile u32 *)&T.ctl->stop == 0) {
                u32 c = atomicAdd(&T.ctl->tile_counter, 1u);
                if (c < A.n_tiles) t = c;
            }
            s_tile = t;
        }
        __syncthreads();
        const u32 t = s_tile;
        __syncthreads();
        if (t == ~0u) break;
        const u64 t0 = (u64)(A.first_tile + t) * A.tile_rows;
        const u64 t1 = min(A.n_rows, t0 + A.tile_rows);
        for (u64 base = t0 + (u64)warp * 32; base < t1; base += (u64)nwarps * 32)
            warp_rows<PRECOMBINE>(P, T, sm, base, t1, &s_new, &s_pairs);
        if (threadIdx.x == 0 && *(volatile u32 *)&T.ctl->spill_count > T.spill_threshold)
            atomicExch(&T.ctl->stop, 1u);
    }
    __syncthreads();
    smem_flush(P, T, sm, &s_new);
    __syncthreads();
    if (threadIdx.x == 0 && s_new) atomicAdd(&T.ctl->n_groups, s_new);
    if (threadIdx.x == 0 && s_pairs) atomicAdd(P.dmeta, (unsigned long long)s_pairs);
}

// Re-insert every pair of the old sets into the new (larger, emptied) ones.
__global__ void k_dset_rehash(const u64 *old_sets, u64 old_mask, int n_sets, u64 *new_sets, u64 new_mask,
                              unsigned long long *meta, int narrow) {
    const u64 old_slots = old_mask + 1, new_slots = new_mask + 1;
    const u64 total = old_slots * (u64)n_sets;
    for (u64 i = blockIdx.x * (u64)blockDim.x + threadIdx.x; i < total; i += (u64)gridDim.x * blockDim.x) {
        const int d = (int)(i / old_slots);
        if (narrow) {
            const u64 e = old_sets[i];
            if (e != ~0ull) dset_insert_narrow(new_sets + new_slots * d, new_mask, e, meta, d);
            continue;
        }
        const u64 g = old_sets[2 * i], v = old_sets[2 * i + 1];
        if (g == EMPTY_KEY && v == EMPTY_KEY) continue;
        dset_insert(new_sets + 2 * new_slots * d, new_mask, g, v, meta, d);
    }
}

// Re-insert every used slot of `old` into the (larger, initialised) table.
__global__ void k_rehash(const __grid_constant__ Plan P, const u64 *old, u64 old_cap, int stride, const TableRef T) {
    __shared__ u32 s_new;
    if (threadIdx.x == 0) s_new = 0;
    __syncthreads();
    for (u64 s = blockIdx.x * (u64)blockDim.x + threadIdx.x; s < old_cap + 2; s += (u64)gridDim.x * blockDim.x) {
        const u64 *src = old + s * (u64)stride;
        if (s >= old_cap) {
            if (src[1] == 0) continue;
            u64 *dst = T.slots + (T.cap + (s - old_cap)) * (u64)T.stride;
            for (int w = 0; w < P.words; w++) dst[1 + w] = src[1 + w];
            continue;
        }
        u64 k = src[0];
        if (k == EMPTY_KEY) continue;
        long long d = g_slot(T, k, mix64(k), &s_new);
        if (d < 0) {
            u64 v[GB_MAX_OPS];
            for (int i = 0; i < P.n_ops; i++) v[i] = src[1 + P.ops[i].word];
            spill_record(P, T, k, src[1], v);
            continue;
        }
        u64 *dst = T.slots + (u64)d * (u64)T.stride;
        for (int w = 0; w < P.words; w++) dst[1 + w] = src[1 + w];
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_new) atomicAdd(&T.ctl->n_groups, s_new);
}

// Merge spill records [0, n) into the table; records that still do not fit
// are re-spilled at the tail (index >= n), so the host can loop.
__global__ void k_merge_records(const __grid_constant__ Plan P, const u64 *recs, u32 n, const TableRef T) {
    __shared__ u32 s_new;
    if (threadIdx.x == 0) s_new = 0;
    __syncthreads();
    for (u64 i = blockIdx.x * (u64)blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
        const u64 *rec = recs + i * (u64)(1 + P.words);
        u64 v[GB_MAX_OPS];
        for (int j = 0; j < P.n_ops; j++) v[j] = rec[1 + P.ops[j].word];
        global_fold(P, T, rec[0], rec[1], v, &s_new);
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_new) atomicAdd(&T.ctl->n_groups, s_new);
}

// Compact used slots into dense result columns (the direct emit of
// physical_planner.cpp:8027-8173 with agg_emit_helpers.cpp:26-165 rules).
// Each CTA takes chunks of `per` * blockDim slots (per <= COMPACT_PER; small
// tables use fewer slots per thread so that more CTAs share them); one
// output reservation per chunk.
#define COMPACT_PER 8
__global__ void k_compact(const __grid_constant__ Plan P, const u64 *slots, u64 cap, int stride,
                          const __grid_constant__ EmitArgs E, Ctl *ctl, int per) {
    const u64 total = cap + 2;
    const u64 chunk = (u64)per * blockDim.x;
    for (u64 c0 = blockIdx.x * chunk; c0 < total; c0 += (u64)gridDim.x * chunk) {
        u32 mine = 0;
#pragma unroll
        for (int j = 0; j < COMPACT_PER; j++) {
            const u64 s = c0 + (u64)j * blockDim.x + threadIdx.x;
            if (j >= per || s >= total) break;
            const u64 *sl = slots + s * (u64)stride;
            mine += (s < cap) ? (sl[0] != EMPTY_KEY) : (sl[1] != 0);
        }
        u64 o = block_out_base(ctl, mine);
#pragma unroll
        for (int j = 0; j < COMPACT_PER; j++) {
            const u64 s = c0 + (u64)j * blockDim.x + threadIdx.x;
            if (j >= per || s >= total) break;
            const u64 *sl = slots + s * (u64)stride;
            const bool occ = (s < cap) ? (sl[0] != EMPTY_KEY) : (sl[1] != 0);
            if (!occ) continue;
            if (o >= E.out_cap) {
                atomicOr(&ctl->err, (u32)ERR_OUT_OVERFLOW);
                continue;
            }
            const u64 pk = (s < cap) ? sl[0] : (s == cap ? EMPTY_KEY : 0ull);
            emit_group(P, E, o, pk, s == cap + 1, sl + 1);
            o++;
        }
    }
}

// ------------------------------------------------------------ TopN
// Order code: a pair (primary, secondary) of u64 where smaller is better.
struct TopnArgs {
    const void *order_col;
    int32_t order_type;   // gb_type of the order column
    int32_t ascending;
    const uint64_t *order_valid;
    const void *key0;
    const void *key1;
    int32_t key_type0, key_type1;
    int32_t n_keys;
    int32_t K;            // <= 1024
};

__device__ __forceinline__ u64 ord_u64(i64 v) { return (u64)v ^ 0x8000000000000000ull; }

__device__ __forceinline__ i64 load_any_int(const void *p, int type, u64 i) {
    switch (type) {
    case GB_T_SMALLINT: return ((const int16_t *)p)[i];
    case GB_T_INTEGER: return ((const int32_t *)p)[i];
    default: return ((const long long *)p)[i];
    }
}

__device__ __forceinline__ void topn_code(const TopnArgs &A, u64 i, u64 &p, u64 &s) {
    u64 prim;
    bool valid = A.order_valid == nullptr || ((A.order_valid[i >> 6] >> (i & 63)) & 1ull);
    if (!valid) prim = 0;  // NULL orders first ascending, last descending
    else if (A.order_type == GB_T_DOUBLE) prim = ord_u64(enc_f64(((const double *)A.order_col)[i]));
    else prim = ord_u64(load_any_int(A.order_col, A.order_type, i));
    p = A.ascending ? prim : ~prim;
    if (A.n_keys == 1) {
        s = ord_u64(load_any_int(A.key0, A.key_type0, i));
    } else {
        u64 a = ord_u64(load_any_int(A.key0, A.key_type0, i)) >> 32;
        u64 b = ord_u64(load_any_int(A.key1, A.key_type1, i)) >> 32;
        if (A.key_type0 == GB_T_BIGINT || A.key_type1 == GB_T_BIGINT) {
            a = ord_u64(load_any_int(A.key0, A.key_type0, i));
            b = 0;
        }
        s = (a << 32) | (b & 0xffffffffull);
    }
}

__device__ __forceinline__ bool code_less(u64 ap, u64 as, u64 bp, u64 bs) {
    return ap < bp || (ap == bp && as < bs);
}

// Bitonic sort of n (power of two) entries in shared memory, ascending.
__device__ void smem_bitonic(u64 *P_, u64 *S_, u32 *I_, int n) {
    for (int k = 2; k <= n; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                int ixj = i ^ j;
                if (ixj > i) {
                    bool up = ((i & k) == 0);
                    // ties on the code order by id, so a real row whose code
                    // is all ones still sorts before the empty entries (~0u)
                    bool gt = code_less(P_[ixj], S_[ixj], P_[i], S_[i]) ||
                              (P_[ixj] == P_[i] && S_[ixj] == S_[i] && I_[ixj] < I_[i]);
                    if (gt == up) {
                        u64 tp = P_[i]; P_[i] = P_[ixj]; P_[ixj] = tp;
                        u64 ts = S_[i]; S_[i] = S_[ixj]; S_[ixj] = ts;
                        u32 ti = I_[i]; I_[i] = I_[ixj]; I_[ixj] = ti;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// Each CTA selects the K best of its slice of items; items are either
// result rows (ids == nullptr) or a candidate list of row ids (~0u = none).
// Survivors of the running threshold go to a candidate buffer; when it
// fills, best ∪ candidates is bitonic-sorted and the best K kept.
__global__ void __launch_bounds__(512) k_topn(const __grid_constant__ TopnArgs A, const u32 *ids, u64 n,
                                              u32 *out_ids, u32 *out_n, int sortn) {
    extern __shared__ u64 tsm[];
    u64 *Pp = tsm;
    u64 *Ss = tsm + sortn;
    u32 *Ii = (u32 *)(tsm + 2 * sortn);
    __shared__ int s_nbest, s_ncand;
    __shared__ u64 s_thr_p, s_thr_s;
    const int K = A.K;
    const int CAPC = sortn - K;  // candidates collected before a sort
    if (threadIdx.x == 0) { s_nbest = 0; s_ncand = 0; s_thr_p = ~0ull; s_thr_s = ~0ull; }
    // entries [0, K) = best (sorted), [K, sortn) = candidates
    for (int i = threadIdx.x; i < sortn; i += blockDim.x) { Pp[i] = ~0ull; Ss[i] = ~0ull; Ii[i] = ~0u; }
    __syncthreads();
    const u64 per = (n + gridDim.x - 1) / gridDim.x;
    const u64 lo = blockIdx.x * per, hi = min(n, lo + per);
    constexpr int TR = 8;  // rows per thread per pass: their loads are issued together
    // Until K rows are held, rows no better than `bound` are skipped: bound
    // is the K-th best of the warps' best rows of the first pass (K distinct
    // rows are at least that good, so every row of the final top K is too).
    __shared__ u64 s_bp, s_bs;
    __shared__ u64 s_wp[32], s_ws[32];
    if (threadIdx.x == 0) {
        s_bp = ~0ull;
        s_bs = ~0ull;
    }
    __syncthreads();
    bool first = true;
    for (u64 base = lo; base < hi; base += (u64)blockDim.x * TR) {
        u64 cpv[TR], csv[TR];
        u32 rowv[TR];
        bool wantv[TR];
        bool any = false;
#pragma unroll
        for (int j = 0; j < TR; j++) {
            const u64 it = base + (u64)j * blockDim.x + threadIdx.x;
            cpv[j] = ~0ull;
            csv[j] = ~0ull;
            rowv[j] = ~0u;
            wantv[j] = false;
            if (it < hi) {
                rowv[j] = ids ? ids[it] : (u32)it;
                if (rowv[j] != ~0u) {
                    topn_code(A, rowv[j], cpv[j], csv[j]);
                    wantv[j] = s_nbest < K ? !code_less(s_bp, s_bs, cpv[j], csv[j])
                                           : code_less(cpv[j], csv[j], s_thr_p, s_thr_s);
                }
            }
            any |= wantv[j];
        }
        const int nwarps = blockDim.x >> 5;
        if (first && K <= nwarps) {
            first = false;
            u64 bp = ~0ull, bs = ~0ull;
#pragma unroll
            for (int j = 0; j < TR; j++)
                if (code_less(cpv[j], csv[j], bp, bs)) {
                    bp = cpv[j];
                    bs = csv[j];
                }
            for (int o = 16; o > 0; o >>= 1) {
                const u64 op = __shfl_xor_sync(0xffffffffu, bp, o), os = __shfl_xor_sync(0xffffffffu, bs, o);
                if (code_less(op, os, bp, bs)) {
                    bp = op;
                    bs = os;
                }
            }
            if ((threadIdx.x & 31) == 0) {
                s_wp[threadIdx.x >> 5] = bp;
                s_ws[threadIdx.x >> 5] = bs;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                // insertion sort of the warps' best rows; the K-th is the bound
                for (int a = 1; a < nwarps; a++)
                    for (int b = a; b > 0 && code_less(s_wp[b], s_ws[b], s_wp[b - 1], s_ws[b - 1]); b--) {
                        const u64 tp = s_wp[b], ts = s_ws[b];
                        s_wp[b] = s_wp[b - 1];
                        s_ws[b] = s_ws[b - 1];
                        s_wp[b - 1] = tp;
                        s_ws[b - 1] = ts;
                    }
                s_bp = s_wp[K - 1];
                s_bs = s_ws[K - 1];
            }
            __syncthreads();
            const u64 qp = s_bp, qs = s_bs;
            any = false;
#pragma unroll
            for (int j = 0; j < TR; j++) {
                wantv[j] = wantv[j] && (s_nbest >= K || !code_less(qp, qs, cpv[j], csv[j]));
                any |= wantv[j];
            }
        }
        first = false;
        // once the threshold has settled, no row of a pass usually beats it:
        // one barrier for TR * blockDim rows
        if (!__syncthreads_or(any)) continue;
        for (int j = 0; j < TR; j++) {
            const u64 cp = cpv[j], cs = csv[j];
            const u32 row = rowv[j];
            bool want = wantv[j] && (s_nbest < K ? !code_less(s_bp, s_bs, cp, cs)
                                                 : code_less(cp, cs, s_thr_p, s_thr_s));
            while (__syncthreads_or(want)) {
                if (want) {
                    int pos = atomicAdd(&s_ncand, 1);
                    if (pos < CAPC) {
                        Pp[K + pos] = cp; Ss[K + pos] = cs; Ii[K + pos] = row;
                        want = false;
                    }
                }
                __syncthreads();
                if (s_ncand >= CAPC) {
                    smem_bitonic(Pp, Ss, Ii, sortn);
                    if (threadIdx.x == 0) {
                        s_nbest = min(s_nbest + CAPC, K);
                        s_ncand = 0;
                        s_thr_p = Pp[K - 1];
                        s_thr_s = Ss[K - 1];
                    }
                    for (int i = K + threadIdx.x; i < sortn; i += blockDim.x) { Pp[i] = ~0ull; Ss[i] = ~0ull; Ii[i] = ~0u; }
                    __syncthreads();
                    if (want) want = code_less(cp, cs, s_thr_p, s_thr_s);
                }
            }
        }
    }
    __syncthreads();
    if (s_ncand > 0) {
        smem_bitonic(Pp, Ss, Ii, sortn);
        if (threadIdx.x == 0) s_nbest = min(s_nbest + s_ncand, K);
        __syncthreads();
    }
    const int nb = s_nbest;
    for (int i = threadIdx.x; i < K; i += blockDim.x) out_ids[(u64)blockIdx.x * K + i] = (i < nb) ? Ii[i] : ~0u;
    if (threadIdx.x == 0) out_n[blockIdx.x] = nb;
}

// TopN for K <= 32: each warp keeps its best K rows in registers, sorted
// (lane i holds the i-th best; lanes >= K hold nothing); a row better than
// the warp's K-th enters by one shuffle insertion.  Warp 0 then merges the
// block's warp lists the same way.  Items: result rows (ids == nullptr) or a
// candidate list of row ids (~0u = none).  Output: the block's best K ids in
// out_ids[blockIdx.x * K + i] (~0u past out_n[blockIdx.x]).
struct TopItem {
    u64 p, s;
    u32 id;
};

// Insert (p, s, id) into the warp's sorted list (every lane calls it with the
// same item); returns the new K-th best.
__device__ __forceinline__ void warp_list_insert(TopItem &mine, int K, u64 p, u64 s, u32 id) {
    const int lane = threadIdx.x & 31;
    const bool better = lane < K && code_less(mine.p, mine.s, p, s);  // my slot stays ahead of the item
    const int pos = __popc(__ballot_sync(FULL, better));
    const u64 up = __shfl_up_sync(FULL, mine.p, 1), us = __shfl_up_sync(FULL, mine.s, 1);
    const u32 ui = __shfl_up_sync(FULL, mine.id, 1);
    if (lane < K) {
        if (lane == pos) {
            mine.p = p;
            mine.s = s;
            mine.id = id;
        } else if (lane > pos) {
            mine.p = up;
            mine.s = us;
            mine.id = ui;
        }
    }
}

__global__ void __launch_bounds__(512) k_topn_small(const __grid_constant__ TopnArgs A, const u32 *ids, u64 n,
                                                    u32 *out_ids, u32 *out_n) {
    __shared__ TopItem s_list[16][32];
    const int K = A.K;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    TopItem mine{~0ull, ~0ull, ~0u};
    const u64 per = (n + gridDim.x - 1) / gridDim.x;
    const u64 lo = blockIdx.x * per, hi = min(n, lo + per);
    constexpr int TR = 4;  // rows per lane per step: their loads are issued together
    u64 tp = ~0ull, ts = ~0ull;  // the warp's K-th best
    bool full = false;           // K rows held: only better rows enter
    for (u64 base = lo + (u64)warp * 32 * TR; base < hi; base += (u64)nwarps * 32 * TR) {
        u64 cp[TR], cs[TR];
        u32 row[TR];
#pragma unroll
        for (int j = 0; j < TR; j++) {
            const u64 it = base + (u64)j * 32 + lane;
            cp[j] = cs[j] = ~0ull;
            row[j] = ~0u;
            if (it < hi) {
                row[j] = ids ? ids[it] : (u32)it;
                if (row[j] != ~0u) topn_code(A, row[j], cp[j], cs[j]);
            }
        }
#pragma unroll
        for (int j = 0; j < TR; j++) {
            bool want = row[j] != ~0u && (!full || code_less(cp[j], cs[j], tp, ts));
            unsigned m;
            while ((m = __ballot_sync(FULL, want))) {
                const int src = __ffs(m) - 1;
                const u64 p = __shfl_sync(FULL, cp[j], src), s = __shfl_sync(FULL, cs[j], src);
                const u32 id = __shfl_sync(FULL, row[j], src);
                warp_list_insert(mine, K, p, s, id);
                tp = __shfl_sync(FULL, mine.p, K - 1);
                ts = __shfl_sync(FULL, mine.s, K - 1);
                full = __shfl_sync(FULL, mine.id, K - 1) != ~0u;
                if (lane == src) want = false;
                want = want && (!full || code_less(cp[j], cs[j], tp, ts));
            }
        }
    }
    s_list[warp][lane] = mine;
    __syncthreads();
    if (warp == 0) {
        TopItem best{~0ull, ~0ull, ~0u};
        u64 bp = ~0ull, bs = ~0ull;
        bool bfull = false;
        for (int w = 0; w < nwarps; w++) {
            const TopItem c = s_list[w][lane];
            bool want = lane < K && c.id != ~0u && (!bfull || code_less(c.p, c.s, bp, bs));
            unsigned m;
            while ((m = __ballot_sync(FULL, want))) {
                const int src = __ffs(m) - 1;
                const u64 p = __shfl_sync(FULL, c.p, src), s = __shfl_sync(FULL, c.s, src);
                const u32 id = __shfl_sync(FULL, c.id, src);
                warp_list_insert(best, K, p, s, id);
                bp = __shfl_sync(FULL, best.p, K - 1);
                bs = __shfl_sync(FULL, best.s, K - 1);
                bfull = __shfl_sync(FULL, best.id, K - 1) != ~0u;
                if (lane == src) want = false;
                want = want && (!bfull || code_less(c.p, c.s, bp, bs));
            }
        }
        if (lane < K) out_ids[(u64)blockIdx.x * K + lane] = best.id;
        const unsigned have = __ballot_sync(FULL, lane < K && best.id != ~0u);
        if (lane == 0) out_n[blockIdx.x] = (u32)__popc(have);
    }
}

// Gather rows `ids[0..k)` of the dense result into TopN output buffers.
__global__ void k_gather_rows(const u32 *ids, u32 k, int ncols, const __grid_constant__ EmitArgs src,
                              const __grid_constant__ EmitArgs dst, const int32_t *types) {
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < k; i += gridDim.x * blockDim.x) {
        u32 r = ids[i];
        if (r == ~0u) continue;
        for (int c = 0; c < ncols; c++) {
            int t = types[c];
            int sz = (t == GB_T_SMALLINT) ? 2 : (t == GB_T_INTEGER ? 4 : 8);
            const char *sp = (const char *)src.out[c] + (u64)r * sz;
            char *dp = (char *)dst.out[c] + (u64)i * sz;
            for (int b = 0; b < sz; b++) dp[b] = sp[b];
            bool v = (src.valid[c][r >> 6] >> (r & 63)) & 1ull;
            if (!v) clear_valid(dst.valid[c], i);
        }
    }
}

}  // namespace gb

// ======================================================================= host
using namespace gb;

static int type_size(int t) {
    switch (t) {
    case GB_T_SMALLINT: return 2;
    case GB_T_INTEGER: return 4;
    case GB_T_BIGINT: return 8;
    case GB_T_DOUBLE: return 8;
    default: return 0;
    }
}

static int type_bits(int t) { return type_size(t) * 8; }

static u64 next_pow2(u64 x) {
    u64 p = 1;
    while (p < x) p <<= 1;
    return p;
}

struct DevBuf {
    void *p = nullptr;
    size_t n = 0;
    gb_status ensure(size_t bytes) {
        if (bytes <= n) return GB_OK;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        size_t want = std::max(bytes, (size_t)256);
        cudaError_t e = cudaMalloc(&p, want);
        if (e != cudaSuccess) {
            p = nullptr;
            (void)cudaGetLastError();  // do not leave the failure as the runtime's last error
            char what[96];
            snprintf(what, sizeof what, "cudaMalloc(%zu bytes)", want);
            return cuda_fail(e, what);
        }
        n = want;
        return GB_OK;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct HostBuf {
    void *p = nullptr;
    size_t n = 0;
    gb_status ensure(size_t bytes) {
        if (bytes <= n) return GB_OK;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        size_t want = std::max(bytes, (size_t)256);
        cudaError_t e = cudaMallocHost(&p, want);
        if (e != cudaSuccess) { p = nullptr; return cuda_fail(e, "cudaMallocHost"); }
        n = want;
        return GB_OK;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
    }
};

struct gb_agg {
    // spec copy
    std::vector<int32_t> col_types;
    std::vector<int32_t> group_cols;
    std::vector<gb_agg_desc> aggs;
    std::vector<gb_filter> filters;
    std::vector<uint8_t> filt_host;  // the filters' literals (host copy they point at)
    DevBuf filt_dev;                 // ... and their device copy
    uint64_t nullable_mask = 0;
    uint64_t est_groups = 0;

    Plan plan{};
    std::vector<EmitAgg> emit;
    std::vector<int32_t> out_types;  // per output column

    // HBM table
    DevBuf table, table_old, spill, ctl_buf;
    u64 cap = 0;
    u32 spill_cap = 0, spill_threshold = 0;
    u64 n_groups = 0;
    // dense result
    std::vector<DevBuf> out_cols, out_valid;
    u64 out_cap = 0;
    u64 n_rows_out = 0;
    // topn
    bool topn = false;
    u32 topn_col = 0;
    bool topn_asc = false;
    u64 topn_limit = 0;
    u64 row_limit = 0;
    DevBuf topn_ids_a, topn_ids_b, topn_cnt;
    std::vector<DevBuf> top_cols, top_valid;
    DevBuf types_dev;
    bool topn_applied = false;
    // host result
    std::vector<HostBuf> host_cols, host_valid;
    std::vector<const void *> res_ptrs;
    std::vector<const uint64_t *> res_valid;
    std::vector<const int64_t *> res_offsets;
    // host staging
    std::vector<DevBuf> stage[2];
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_copied[2] = {nullptr, nullptr}, ev_done[2] = {nullptr, nullptr};
    // radix mode (high-cardinality keys)
    int mode = 0;          // 0 = hash, 1 = radix
    int mode_option = 0;   // 0 = auto, 1 = force hash, 2 = force radix
    RadixPlan rplan{};
    bool r_ready = false;
    bool pending_reset = false;  // gb_agg_reset's device work waits for the next ingest / finalize
    DevBuf r_skeys, r_scnt, r_hist, r_hot_keys, r_hot_part, r_cursor, r_part, r_part2, r_ovf;
    DevBuf r_off, r_cap, r_off2, r_cap2;    // per-partition region start / capacity (device)
    DevBuf r_hot_idx, r_hot_list, r_hstate, r_cand;
    DevBuf r_p2w;                           // P2 state words folded in L2 (plans whose ops are all DOUBLE SUM)
    std::vector<u64> h_off;                 // host copies
    std::vector<u32> h_capv;
    u64 r_cap_p = 0;
    u32 r_ovf_cap = 0;
    int r_grid = 0;
    u64 rows_ingested = 0;
    // COUNT(DISTINCT): (group, value) pair sets, one per distinct column
    DevBuf dsets, dsets_old, null_sets, null_sets_old, dmeta;
    u64 dslots = 0;               // slots per set (power of two; 0 = none yet)
    u64 dpairs = 0;               // pairs inserted (host copy)
    bool dist_null_sets = false;  // NULL-key group of a nullable BIGINT key in twin sets
    unsigned long long dmeta_host[2 + GB_MAX_DISTINCT] = {};
    // VARCHAR group key: device string dictionary (string -> dense id)
    int str_col = -1;
    DevBuf sd_hash, sd_ref, sd_id, sd_refid, sd_ctr, sd_arena, sd_old_hash, sd_old_ref, sd_old_id, sd_old_refid;
    DevBuf sd_ids, sd_retry_a, sd_retry_b;
    u64 sd_cap = 0, sd_arena_cap = 0;
    DevBuf out_str_offs, out_str_bytes, str_lens, scan_tmp;
    HostBuf host_str_offs, host_str_bytes;
    // tuning
    int block = 512;
    int ctas_per_sm = 2;
    int smem_slots = 4096;
    int smem_probe = 8;
    int gmax_probe = 256;
    bool precombine = true;
    bool precombine_set = false;  // the "precombine" option was given (else the fast path chooses)
    bool fast_ingest = true;      // integer plans take the register-resident fast kernel
    bool topn_small = true;       // K <= 32: warp-register TopN lists
    u32 tile_rows = 8192;
    // profiling (CUDA events around each kernel, resolved at sync points)
    bool profiling = false;
    struct ProfEv { int stat; cudaEvent_t a, b; };
    std::vector<ProfEv> prof_pending;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<gb_kernel_stat> stats;
    // accounting / state
    u64 launches = 0;
    u64 rg_pruned = 0;  // Parquet row groups skipped by zone maps
    bool finalized = false;
    bool has_result = false;
    Ctl ctl_host{};
};

static TableRef table_ref(gb_agg *h) {
    TableRef T;
    T.slots = (u64 *)h->table.p;
    T.cap = h->cap;
    T.stride = h->plan.stride;
    T.gmax_probe = h->gmax_probe;
    T.ctl = (Ctl *)h->ctl_buf.p;
    T.spill = (u64 *)h->spill.p;
    T.spill_cap = h->spill_cap;
    T.spill_threshold = h->spill_threshold;
    return T;
}

static cudaEvent_t prof_event(gb_agg *h) {
    if (!h->ev_pool.empty()) {
        cudaEvent_t e = h->ev_pool.back();
        h->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

static int prof_stat(gb_agg *h, const char *name) {
    for (size_t i = 0; i < h->stats.size(); i++)
        if (strncmp(h->stats[i].name, name, sizeof(h->stats[i].name)) == 0) return (int)i;
    gb_kernel_stat s{};
    strncpy(s.name, name, sizeof(s.name) - 1);
    h->stats.push_back(s);
    return (int)h->stats.size() - 1;
}

// Bracket one kernel launch with events on its stream (profiling only).
struct ProfScope {
    gb_agg *h;
    cudaStream_t st;
    int stat;
    cudaEvent_t a = nullptr;
    ProfScope(gb_agg *h_, const char *name, cudaStream_t st_) : h(h_), st(st_), stat(-1) {
        if (!h->profiling) return;
        stat = prof_stat(h, name);
        a = prof_event(h);
        cudaEventRecord(a, st);
    }
    ~ProfScope() {
        if (!h->profiling) return;
        cudaEvent_t b = prof_event(h);
        cudaEventRecord(b, st);
        h->prof_pending.push_back({stat, a, b});
    }
};

// Resolve pending event pairs (the stream has been synchronised).
static void prof_collect(gb_agg *h) {
    for (auto &p : h->prof_pending) {
        float ms = 0.f;
        if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            h->stats[p.stat].launches++;
            h->stats[p.stat].ms += ms;
        }
        h->ev_pool.push_back(p.a);
        h->ev_pool.push_back(p.b);
    }
    h->prof_pending.clear();
}

static int grid_for(u64 work, int block, int max_ctas) {
    u64 g = (work + block - 1) / block;
    if (g < 1) g = 1;
    if (g > (u64)max_ctas) g = max_ctas;
    return (int)g;
}

static gb_status init_table(gb_agg *h, DevBuf &buf, u64 cap, cudaStream_t st) {
    size_t bytes = (size_t)(cap + 2) * h->plan.stride * 8;
    gb_status s = buf.ensure(bytes);
    if (s) return s;
    u64 words = (cap + 2) * (u64)h->plan.stride;
    {
        ProfScope ps(h, "k_table_init", st);
        k_table_init<<<grid_for(words, 256, sm_count() * 8), 256, 0, st>>>((u64 *)buf.p, cap + 2, h->plan.stride,
                                                                           h->plan);
    }
    h->launches++;
    GB_CUDA(cudaGetLastError());
    return GB_OK;
}

static gb_status dist_clear(gb_agg *h, cudaStream_t st);

// The device part of gb_agg_reset, on the stream of the call that follows it.
static gb_status apply_reset(gb_agg *h, cudaStream_t st) {
    if (!h->pending_reset) return GB_OK;
    gb_status s = init_table(h, h->table, h->cap, st);
    if (s) return s;
    if ((s = dist_clear(h, st))) return s;
    GB_CUDA(cudaMemsetAsync(h->ctl_buf.p, 0, sizeof(Ctl), st));
    h->pending_reset = false;
    return GB_OK;
}

static gb_status read_ctl(gb_agg *h, cudaStream_t st) {
    GB_CUDA(cudaMemcpyAsync(&h->ctl_host, h->ctl_buf.p, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    return GB_OK;
}

static gb_status check_err(gb_agg *h) {
    u32 e = h->ctl_host.err;
    if (e & ERR_NULL_IN_WIDE_KEY) {
        set_error("NULL in a two-column key whose packed width leaves no NULL bits (two 32-bit keys)");
        return GB_ERR_UNSUPPORTED;
    }
    if (e & ERR_SPILL_OVERFLOW) {
        set_error("spill buffer overflow (internal invariant violated)");
        return GB_ERR_OOM;
    }
    if (e & ERR_OUT_OVERFLOW) {
        set_error("result buffer overflow (internal invariant violated)");
        return GB_ERR_CUDA;
    }
    return GB_OK;
}

// Grow the HBM table to new_cap (rehash) and merge `pending` spill records
// (already at the front of the spill buffer).  Loops until nothing spills.
static gb_status grow_and_merge(gb_agg *h, u64 new_cap, u32 pending, cudaStream_t st) {
    Ctl *dctl = (Ctl *)h->ctl_buf.p;
    const int recw = 1 + h->plan.words;
    for (int round = 0; round < 40; round++) {
        if (new_cap > h->cap) {
            std::swap(h->table, h->table_old);
            u64 old_cap = h->cap;
            gb_status s = init_table(h, h->table, new_cap, st);
            if (s) return s;
            h->cap = new_cap;
            // move pending records out of the way: they live at [0, pending)
            // and rehash spills append after them.
            GB_CUDA(cudaMemsetAsync(&dctl->n_groups, 0, sizeof(u32), st));
            GB_CUDA(cudaMemcpyAsync(&dctl->spill_count, &pending, sizeof(u32), cudaMemcpyHostToDevice, st));
            TableRef T = table_ref(h);
            k_rehash<<<grid_for(old_cap + 2, 256, sm_count() * 8), 256, 0, st>>>(h->plan, (const u64 *)h->table_old.p,
                                                                                 old_cap, h->plan.stride, T);
            h->launches++;
            GB_CUDA(cudaGetLastError());
        }
        if (pending == 0) {
            gb_status s = read_ctl(h, st);
            if (s) return s;
            if ((s = check_err(h))) return s;
            h->n_groups = h->ctl_host.n_groups;
            u32 sp = h->ctl_host.spill_count;
            if (sp == 0) return GB_OK;
            pending = sp;  // rehash itself spilled: grow again
            new_cap = h->cap * 2;
            continue;
        }
        // merge [0, pending) — re-spills land at [pending, ...)
        TableRef T = table_ref(h);
        GB_CUDA(cudaMemcpyAsync(&dctl->spill_count, &pending, sizeof(u32), cudaMemcpyHostToDevice, st));
        k_merge_records<<<grid_for(pending, 256, sm_count() * 8), 256, 0, st>>>(h->plan, (const u64 *)h->spill.p,
                                                                              pending, T);
        h->launches++;
        GB_CUDA(cudaGetLastError());
        gb_status s = read_ctl(h, st);
        if (s) return s;
        if ((s = check_err(h))) return s;
        u32 total = h->ctl_host.spill_count;
        u32 again = total - pending;
        h->n_groups = h->ctl_host.n_groups;
        if (again == 0) {
            GB_CUDA(cudaMemsetAsync(&dctl->spill_count, 0, sizeof(u32), st));
            return GB_OK;
        }
        // compact the re-spilled tail to the front
        GB_CUDA(cudaMemcpyAsync(h->spill.p, (u64 *)h->spill.p + (size_t)pending * recw, (size_t)again * recw * 8,
                                cudaMemcpyDeviceToDevice, st));
        pending = again;
        new_cap = h->cap * 2;
    }
    set_error("hash table growth did not converge");
    return GB_ERR_OOM;
}

static gb_status ensure_capacity(gb_agg *h, cudaStream_t st) {
    // keep the load factor <= 0.5 for the next batch
    if (h->n_groups * 2 > h->cap) {
        u64 nc = h->cap;
        while (h->n_groups * 2 > nc) nc *= 2;
        return grow_and_merge(h, nc, 0, st);
    }
    return GB_OK;
}

// COUNT(DISTINCT): size the pair sets for `n_rows` more rows (load <= 1/2
// even if every row brings a new pair), rehashing what they hold, and point
// the plan at them.
static gb_status dist_reserve(gb_agg *h, u64 n_rows, cudaStream_t st) {
    Plan &P = h->plan;
    const int nd = P.n_dist;
    if ((P.dsets && P.dmask + 1 == h->dslots) && h->dslots >= 2 * (h->dpairs + n_rows)) return GB_OK;
    gb_status s;
    if ((s = h->dmeta.ensure(sizeof(h->dmeta_host)))) return s;
    if (h->dslots == 0) GB_CUDA(cudaMemsetAsync(h->dmeta.p, 0, sizeof(h->dmeta_host), st));
    u64 slots = std::max<u64>(1024, h->dslots);
    while (slots < 2 * (h->dpairs + n_rows)) slots *= 2;
    const u64 wps = P.dnarrow ? 1 : 2;  // words per slot
    const u64 empty = P.dnarrow ? ~0ull : EMPTY_KEY;
    const size_t bytes = (size_t)slots * 8 * wps * nd;
    if (slots != h->dslots) {
        std::swap(h->dsets, h->dsets_old);
        std::swap(h->null_sets, h->null_sets_old);
        if ((s = h->dsets.ensure(bytes))) return s;
        if ((s = radix_fill_u64((u64 *)h->dsets.p, (u64)slots * wps * nd, empty, st))) return s;
        if (h->dist_null_sets) {
            if ((s = h->null_sets.ensure(bytes))) return s;
            if ((s = radix_fill_u64((u64 *)h->null_sets.p, (u64)slots * wps * nd, empty, st))) return s;
        }
        if (h->dslots) {
            const u64 old_mask = h->dslots - 1, total = h->dslots * (u64)nd;
            const int grid = grid_for(total, 256, sm_count() * 8);
            k_dset_rehash<<<grid, 256, 0, st>>>((const u64 *)h->dsets_old.p, old_mask, nd, (u64 *)h->dsets.p,
                                                slots - 1, (unsigned long long *)h->dmeta.p, P.dnarrow);
            h->launches++;
            if (h->dist_null_sets) {
                k_dset_rehash<<<grid, 256, 0, st>>>((const u64 *)h->null_sets_old.p, old_mask, nd,
                                                    (u64 *)h->null_sets.p, slots - 1, (unsigned long long *)h->dmeta.p,
                                                    P.dnarrow);
                h->launches++;
            }
            GB_CUDA(cudaGetLastError());
        }
        h->dsets_old.release();
        h->null_sets_old.release();
        h->dslots = slots;
    }
    P.dsets = (u64 *)h->dsets.p;
    P.null_sets = h->dist_null_sets ? (u64 *)h->null_sets.p : nullptr;
    P.dmeta = (unsigned long long *)h->dmeta.p;
    P.dmask = slots - 1;
    return GB_OK;
}

// Empty the pair sets (reset).
static gb_status dist_clear(gb_agg *h, cudaStream_t st) {
    h->dpairs = 0;
    memset(h->dmeta_host, 0, sizeof(h->dmeta_host));
    if (!h->dslots) return GB_OK;
    const u64 words = h->dslots * (h->plan.dnarrow ? 1 : 2) * (u64)h->plan.n_dist;
    const u64 empty = h->plan.dnarrow ? ~0ull : EMPTY_KEY;
    gb_status s;
    if ((s = radix_fill_u64((u64 *)h->dsets.p, words, empty, st))) return s;
    if (h->dist_null_sets && (s = radix_fill_u64((u64 *)h->null_sets.p, words, empty, st))) return s;
    GB_CUDA(cudaMemsetAsync(h->dmeta.p, 0, sizeof(h->dmeta_host), st));
    return GB_OK;
}

// defined with the fast tile path (gb_batch.cuh): launches the
// single-query fast ingest when the plan allows it (*launched = true)
static gb_status launch_ingest_fast(gb_agg *h, const TableRef &T, IngestArgs A, int grid, cudaStream_t st,
                                    bool *launched);

static gb_status run_ingest(gb_agg *h, u64 n_rows, cudaStream_t st) {
    if (n_rows == 0) return GB_OK;
    if (h->plan.n_dist) {
        gb_status s = dist_reserve(h, n_rows, st);
        if (s) return s;
    }
    Ctl *dctl = (Ctl *)h->ctl_buf.p;
    const int words = h->plan.words;
    u32 tile_rows = h->tile_rows;
    const int max_ctas = sm_count() * h->ctas_per_sm;
    // small inputs: shrink tiles so every CTA gets work
    u64 want_tiles = (u64)max_ctas * 4;
    if (n_rows / tile_rows < want_tiles) {
        u64 tr = (n_rows + want_tiles - 1) / want_tiles;
        tr = ((tr + 511) / 512) * 512;
        tile_rows = (u32)std::max<u64>(1024, std::min<u64>(tr, h->tile_rows));
    }
    const u64 n_tiles_total = (n_rows + tile_rows - 1) / tile_rows;
    int grid = (int)std::min<u64>((u64)max_ctas, n_tiles_total);
    // the shared table pays when the estimated groups fit it; past that every
    // row would probe a full table before its HBM fold
    int S = h->smem_slots;
    if (h->est_groups > (u64)S) S = 0;
    size_t smem = (size_t)S * 8 * (1 + words);
    // spill capacity: threshold + what in-flight tiles and the final flush can add
    u64 margin = (u64)grid * ((u64)tile_rows + (u64)S) + 1024;
    u64 need_cap = (1u << 20) + margin;
    if (h->spill_cap < need_cap) {
        gb_status s = h->spill.ensure((size_t)need_cap * (1 + words) * 8);
        if (s) return s;
        h->spill_cap = (u32)need_cap;
    }
    h->spill_threshold = (u32)(h->spill_cap - margin);
    static bool attr_set[2] = {false, false};
    if (!attr_set[0]) {
        cudaFuncSetAttribute(k_ingest<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(k_ingest<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr_set[0] = attr_set[1] = true;
    }
    u64 first = 0;
    while (first < n_tiles_total) {
        GB_CUDA(cudaMemsetAsync(&dctl->spill_count, 0, 4 * 4, st));  // spill_count, tile_counter, stop, err
        IngestArgs A;
        A.n_rows = n_rows;
        A.tile_rows = tile_rows;
        A.first_tile = (u32)first;
        A.n_tiles = (u32)(n_tiles_total - first);
        A.smem_slots = S;
        A.smem_probe = h->smem_probe;
        A.pad = 0;
        TableRef T = table_ref(h);
        int g = (int)std::min<u64>((u64)grid, n_tiles_total - first);
        bool fast = false;
        if (gb_status fs = launch_ingest_fast(h, T, A, g, st, &fast)) return fs;
        if (!fast) {
            ProfScope ps(h, "k_ingest", st);
            if (h->precombine) k_ingest<true><<<g, h->block, smem, st>>>(h->plan, T, A);
            else k_ingest<false><<<g, h->block, smem, st>>>(h->plan, T, A);
        }
        h->launches++;
        GB_CUDA(cudaGetLastError());
        if (h->plan.n_dist)
            GB_CUDA(cudaMemcpyAsync(h->dmeta_host, h->dmeta.p, sizeof(h->dmeta_host), cudaMemcpyDeviceToHost, st));
        gb_status s = read_ctl(h, st);
        if (s) return s;
        if ((s = check_err(h))) return s;
        if (h->plan.n_dist) {
            if (h->dmeta_host[1]) {
                set_error("COUNT(DISTINCT) pair set overflow (internal invariant violated)");
                return GB_ERR_CUDA;
            }
            h->dpairs = h->dmeta_host[0];
        }
        h->n_groups = h->ctl_host.n_groups;
        u64 claimed = std::min<u64>(h->ctl_host.tile_counter, n_tiles_total - first);
        first += claimed;
        u32 sp = h->ctl_host.spill_count;
        if (sp > 0) {
            u64 nc = h->cap * 2;
            while ((h->n_groups + sp) * 2 > nc) nc *= 2;
            s = grow_and_merge(h, nc, sp, st);
            if (s) return s;
        }
        if ((s = ensure_capacity(h, st))) return s;
    }
    return GB_OK;
}


// ------------------------------------------------------------- radix mode
static RadixRef radix_ref(gb_agg *h) {
    RadixRef X;
    X.part = (u64 *)h->r_part.p;
    X.part_off = (const u64 *)h->r_off.p;
    X.part_cap = (const u32 *)h->r_cap.p;
    X.cursor = (u32 *)h->r_cursor.p;
    X.ovf = (u64 *)h->r_ovf.p;
    X.ovf_cap = h->r_ovf_cap;
    // tiles still in flight after the threshold trips add at most grid * tile rows
    const u64 inflight = radix_inflight_rows(h->rplan, h->r_grid) + 4096;
    X.ovf_threshold = h->r_ovf_cap > inflight ? (u32)(h->r_ovf_cap - inflight) : 0u;
    X.hot_keys = (const u64 *)h->r_hot_keys.p;
    X.hot_idx = (const uint16_t *)h->r_hot_idx.p;
    X.hot_list = (const u64 *)h->r_hot_list.p;
    X.hot_part = (u64 *)h->r_hot_part.p;
    X.p2_words = nullptr;
    return X;
}

// The per-CTA hot slices (identity-initialised) and the overflow list of a
// run whose partition layout is in place.
static gb_status radix_begin_slices(gb_agg *h, cudaStream_t st) {
    const RadixPlan &R = h->rplan;
    const int W = h->plan.words;
    const int TV = 1 + R.V;
    gb_status s;
    h->r_grid = sm_count();
    if ((s = h->r_hot_part.ensure((size_t)h->r_grid * R.nh * W * 8))) return s;
    if ((s = radix_fill_identity((u64 *)h->r_hot_part.p, (u64)h->r_grid * R.nh * W, W, h->plan, st))) return s;
    h->launches++;
    u32 ovf_cap = (1u << 21) + (u32)radix_inflight_rows(R, h->r_grid) + 4096;
    if (h->r_ovf_cap < ovf_cap) {
        if ((s = h->r_ovf.ensure((size_t)ovf_cap * (TV + 1) * 8))) return s;
        h->r_ovf_cap = ovf_cap;
    }
    h->r_ready = true;
    return GB_OK;
}

static gb_status radix_begin(gb_agg *h, u64 n, cudaStream_t st) {
    const RadixPlan &R = h->rplan;
    const u64 np = 1ull << R.pbits;
    const int W = h->plan.words;
    const int TV = 1 + R.V;
    gb_status s;
    // sample the first batch
    u64 m = std::min<u64>(n, 1u << 18);
    u64 scap = 1024;
    while (scap < 2 * m) scap <<= 1;
    if ((s = h->r_skeys.ensure(scap * 8)) || (s = h->r_scnt.ensure(scap * 4)) ||
        (s = h->r_hist.ensure(HIST_BINS * 4)) || (s = h->r_hstate.ensure(16)) ||
        (s = h->r_hot_keys.ensure((size_t)R.HS * 8)) || (s = h->r_hot_idx.ensure((size_t)R.HS * 2)) ||
        (s = h->r_hot_list.ensure((size_t)R.nh * 8)) || (s = h->r_cand.ensure((size_t)R.nh * 12)))
        return s;
    if ((s = radix_fill_u64((u64 *)h->r_skeys.p, scap, EMPTY_KEY, st))) return s;
    GB_CUDA(cudaMemsetAsync(h->r_scnt.p, 0, scap * 4, st));
    GB_CUDA(cudaMemsetAsync(h->r_hist.p, 0, HIST_BINS * 4, st));
    GB_CUDA(cudaMemsetAsync(h->r_hstate.p, 0, 16, st));
    GB_CUDA(cudaMemsetAsync(h->r_hot_idx.p, 0, (size_t)R.HS * 2, st));
    if ((s = radix_fill_u64((u64 *)h->r_hot_keys.p, R.HS, EMPTY_KEY, st))) return s;
    h->launches += 2;
    {
        ProfScope ps(h, "k_sample", st);
        if ((s = radix_launch_sample(h->plan, R, n, (u64 *)h->r_skeys.p, (u32 *)h->r_scnt.p, scap,
                                     (u32 *)h->r_hist.p, (u32 *)h->r_hstate.p, (u64 *)h->r_cand.p,
                                     (u32 *)((u64 *)h->r_cand.p + R.nh), (u64 *)h->r_hot_keys.p,
                                     (uint16_t *)h->r_hot_idx.p, (u64 *)h->r_hot_list.p, st, &h->launches)))
            return s;
    }
    if (h->h_capv.size() == np && h->h_off.size() == np + 1) {
        // a re-execution keeps the partition layout of the earlier runs (the
        // regions they grew to stay large; a region that overflows grows
        // again), so the sample's hot fraction need not come back to the host
        GB_CUDA(cudaMemsetAsync(h->r_cursor.p, 0, (size_t)np * CURSOR_PAD * 4, st));
        return radix_begin_slices(h, st);
    }
    u32 hst[4] = {0, 0, 0, 0};
    GB_CUDA(cudaMemcpyAsync(hst, h->r_hstate.p, 16, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    u32 hot_rows = hst[2];
    u64 sampled = std::max<u64>(1, std::min<u64>(n, m));
    double hot_frac = std::min(1.0, (double)hot_rows / (double)sampled);
    double tail = (double)n * (1.0 - hot_frac);
    u64 cap_p = (u64)(tail / (double)np * 1.5) + 2048;
    cap_p = (cap_p + 31) / 32 * 32;
    h->r_cap_p = cap_p;
    h->h_capv.assign(np, (u32)cap_p);
    h->h_off.assign(np + 1, 0);
    for (u64 p = 0; p < np; p++) h->h_off[p + 1] = h->h_off[p] + h->h_capv[p];
    if ((s = h->r_part.ensure((size_t)h->h_off[np] * TV * 8))) return s;
    if ((s = h->r_off.ensure((np + 1) * 8)) || (s = h->r_cap.ensure(np * 4))) return s;
    GB_CUDA(cudaMemcpyAsync(h->r_off.p, h->h_off.data(), (np + 1) * 8, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync(h->r_cap.p, h->h_capv.data(), np * 4, cudaMemcpyHostToDevice, st));
    if ((s = h->r_cursor.ensure((size_t)np * CURSOR_PAD * 4))) return s;
    GB_CUDA(cudaMemsetAsync(h->r_cursor.p, 0, (size_t)np * CURSOR_PAD * 4, st));
    return radix_begin_slices(h, st);
}

// Grow the regions of the partitions that overflowed (each to what it
// needs, so one skewed partition does not inflate the others), move the
// filled prefixes, then append the overflow tuples.
static gb_status radix_grow(gb_agg *h, u32 novf, cudaStream_t st) {
    const RadixPlan &R = h->rplan;
    const u64 np = 1ull << R.pbits;
    const int TV = 1 + R.V;
    std::vector<u32> cur((size_t)np * CURSOR_PAD);
    GB_CUDA(cudaMemcpyAsync(cur.data(), h->r_cursor.p, cur.size() * 4, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    std::vector<u64> noff(np + 1, 0);
    std::vector<u32> ncap(np);
    for (u64 p = 0; p < np; p++) {
        const u64 want = cur[p * CURSOR_PAD];
        u64 c = h->h_capv[p];
        if (want > c) c = std::max<u64>(c * 2, want + want / 4 + 256);
        c = (c + 31) / 32 * 32;
        if (c > 0xffffffffull) {
            set_error("partition %llu exceeds 2^32 tuples", (unsigned long long)p);
            return GB_ERR_UNSUPPORTED;
        }
        ncap[p] = (u32)c;
        noff[p + 1] = noff[p] + c;
    }
    gb_status s;
    if ((s = h->r_part2.ensure((size_t)noff[np] * TV * 8)) || (s = h->r_off2.ensure((np + 1) * 8)) ||
        (s = h->r_cap2.ensure(np * 4)))
        return s;
    GB_CUDA(cudaMemcpyAsync(h->r_off2.p, noff.data(), (np + 1) * 8, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync(h->r_cap2.p, ncap.data(), np * 4, cudaMemcpyHostToDevice, st));
    RadixRef from = radix_ref(h);
    RadixRef to = from;
    to.part = (u64 *)h->r_part2.p;
    to.part_off = (const u64 *)h->r_off2.p;
    to.part_cap = (const u32 *)h->r_cap2.p;
    if ((s = radix_launch_move(from, to, R.V, (int)np, st))) return s;
    h->launches++;
    // cursors := tuples actually stored in each region
    for (u64 p = 0; p < np; p++) cur[p * CURSOR_PAD] = std::min<u32>(cur[p * CURSOR_PAD], h->h_capv[p]);
    GB_CUDA(cudaMemcpyAsync(h->r_cursor.p, cur.data(), cur.size() * 4, cudaMemcpyHostToDevice, st));
    std::swap(h->r_part, h->r_part2);
    std::swap(h->r_off, h->r_off2);
    std::swap(h->r_cap, h->r_cap2);
    h->h_off.swap(noff);
    h->h_capv.swap(ncap);
    RadixRef X = radix_ref(h);
    if ((s = radix_launch_drain(X, R.V, novf, st))) return s;
    h->launches++;
    GB_CUDA(cudaStreamSynchronize(st));
    Ctl *dctl = (Ctl *)h->ctl_buf.p;
    GB_CUDA(cudaMemsetAsync(&dctl->aux0, 0, 4, st));
    return GB_OK;
}

static gb_status radix_ingest(gb_agg *h, u64 n, cudaStream_t st) {
    if (n == 0) return GB_OK;
    gb_status s;
    if (!h->r_ready && (s = radix_begin(h, n, st))) return s;
    Ctl *dctl = (Ctl *)h->ctl_buf.p;
    const u32 tr = radix_tile_rows(h->rplan);
    const u64 n_tiles = (n + tr - 1) / tr;
    u64 first = 0;
    while (first < n_tiles) {
        GB_CUDA(cudaMemsetAsync(&dctl->spill_count, 0, 4 * 4, st));
        GB_CUDA(cudaMemsetAsync(&dctl->aux0, 0, 4, st));
        RadixTile A;
        A.n_rows = n;
        A.first_tile = (u32)first;
        A.n_tiles = (u32)(n_tiles - first);
        TableRef T = table_ref(h);
        RadixRef X = radix_ref(h);
        {
            ProfScope ps(h, "k_partition", st);
            if ((s = radix_launch_p1(h->plan, h->rplan, X, T, A, h->r_grid, st))) return s;
        }
        h->launches++;
        if ((s = read_ctl(h, st))) return s;
        if ((s = check_err(h))) return s;
        first += std::min<u64>(h->ctl_host.tile_counter, n_tiles - first);
        if (h->ctl_host.aux0 > 0 && (s = radix_grow(h, h->ctl_host.aux0, st))) return s;
    }
    return GB_OK;
}

static gb_status alloc_outputs(gb_agg *h, u64 rows);
static void fill_emit(gb_agg *h, EmitArgs &E, std::vector<DevBuf> &cols, std::vector<DevBuf> &valid, u64 cap);

static gb_status radix_emit(gb_agg *h, cudaStream_t st) {
    const RadixPlan &R = h->rplan;
    const u64 np = 1ull << R.pbits;
    gb_status s;
    Ctl *dctl = (Ctl *)h->ctl_buf.p;
    // capacity bound: tuples the partition regions hold (their capacities,
    // known on the host: no device round trip) + hot keys + HBM-table slots
    u64 tuples = 0;
    if (h->r_ready)
        for (u64 p = 0; p < np; p++) tuples += h->h_capv[p];
    u64 cap = tuples + (u64)R.nh + h->cap + 2;
    if ((s = alloc_outputs(h, cap))) return s;
    // a partition whose groups overflow its shared table folds the rest into
    // the HBM table, which spills (at most once per tuple) when full
    {
        const u64 need = tuples + 4096;
        if (h->spill_cap < need) {
            if ((s = h->spill.ensure((size_t)need * (1 + h->plan.words) * 8))) return s;
            h->spill_cap = (u32)need;
        }
        h->spill_threshold = h->spill_cap;
    }
    for (size_t c = 0; c < h->out_valid.size(); c++)
        GB_CUDA(cudaMemsetAsync(h->out_valid[c].p, 0xff, (cap + 63) / 64 * 8, st));
    GB_CUDA(cudaMemsetAsync(&dctl->spill_count, 0, 4 * 4, st));
    GB_CUDA(cudaMemsetAsync(&dctl->out_count, 0, 4, st));
    EmitArgs E;
    fill_emit(h, E, h->out_cols, h->out_valid, h->out_cap);
    if (h->r_ready) {
        TableRef T = table_ref(h);
        RadixRef X = radix_ref(h);
        if (radix_p2_global_words(h->plan, R)) {
            if ((s = h->r_p2w.ensure((size_t)np * R.sub * (h->plan.words - 1) * 8))) return s;
            X.p2_words = (u64 *)h->r_p2w.p;
        }
        {
            ProfScope ps(h, "k_part_agg", st);
            if ((s = radix_launch_p2(h->plan, R, X, T, E, st))) return s;
        }
        {
            ProfScope ps(h, "k_hot_emit", st);
            if ((s = radix_launch_p3(h->plan, R, X, h->r_grid, (const u32 *)h->r_hstate.p, dctl, E, st))) return s;
        }
        h->launches += 2;
        if ((s = read_ctl(h, st))) return s;
        if ((s = check_err(h))) return s;
        h->n_groups = h->ctl_host.n_groups;
        if (h->ctl_host.spill_count > 0) {
            u32 sp = h->ctl_host.spill_count;
            u64 nc = h->cap * 2;
            while ((h->n_groups + sp) * 2 > nc) nc *= 2;
            // T's groups are keys of partition tuples, so `cap` still bounds the result
            if ((s = grow_and_merge(h, nc, sp, st))) return s;
        }
    }
    return GB_OK;
}


// ------------------------------------------------------------- VARCHAR keys
static StrDictRef strdict_ref(gb_agg *h) {
    StrDictRef D;
    D.hash = (u64 *)h->sd_hash.p;
    D.ref = (u64 *)h->sd_ref.p;
    D.id = (u64 *)h->sd_id.p;
    D.ref_by_id = (u64 *)h->sd_refid.p;
    u64 *ctr = (u64 *)h->sd_ctr.p;  // [0] next id, [1] arena used, [2] err (u32)
    D.next_id = ctr;
    D.arena_used = ctr + 1;
    D.err = (u32 *)(ctr + 2);
    D.cap = h->sd_cap;
    D.arena = (uint8_t *)h->sd_arena.p;
    D.arena_cap = h->sd_arena_cap;
    D.max_probe = 64;
    return D;
}

static gb_status strdict_init(gb_agg *h, u64 cap, cudaStream_t st) {
    gb_status s;
    if ((s = h->sd_hash.ensure(cap * 8)) || (s = h->sd_ref.ensure(cap * 8)) || (s = h->sd_id.ensure(cap * 8)) ||
        (s = h->sd_refid.ensure(cap * 8)) || (s = h->sd_ctr.ensure(64)))
        return s;
    if ((s = strdict_fill((u64 *)h->sd_hash.p, cap, EMPTY_KEY, st)) || (s = strdict_fill((u64 *)h->sd_ref.p, cap, ~0ull, st)))
        return s;
    GB_CUDA(cudaMemsetAsync(h->sd_ctr.p, 0, 64, st));
    h->sd_cap = cap;
    h->launches += 2;
    return GB_OK;
}

// Grow the dictionary table (ids are kept; slots move).
static gb_status strdict_grow(gb_agg *h, u64 ncap, cudaStream_t st) {
    std::swap(h->sd_hash, h->sd_old_hash);
    std::swap(h->sd_ref, h->sd_old_ref);
    std::swap(h->sd_id, h->sd_old_id);
    const u64 old_cap = h->sd_cap;
    gb_status s;
    if ((s = h->sd_hash.ensure(ncap * 8)) || (s = h->sd_ref.ensure(ncap * 8)) || (s = h->sd_id.ensure(ncap * 8)))
        return s;
    if ((s = strdict_fill((u64 *)h->sd_hash.p, ncap, EMPTY_KEY, st)) || (s = strdict_fill((u64 *)h->sd_ref.p, ncap, ~0ull, st)))
        return s;
    // ref_by_id grows with the table (ids < claimed slots <= cap)
    if (h->sd_refid.n < ncap * 8) {
        if ((s = h->sd_old_refid.ensure(ncap * 8))) return s;
        GB_CUDA(cudaMemcpyAsync(h->sd_old_refid.p, h->sd_refid.p, old_cap * 8, cudaMemcpyDeviceToDevice, st));
        std::swap(h->sd_refid, h->sd_old_refid);
    }
    h->sd_cap = ncap;
    StrDictRef D = strdict_ref(h);
    if ((s = strdict_launch_rehash((const u64 *)h->sd_old_hash.p, (const u64 *)h->sd_old_ref.p,
                                   (const u64 *)h->sd_old_id.p, old_cap, D, st)))
        return s;
    h->launches += 3;
    return GB_OK;
}

// Encode a VARCHAR column (device bytes/offsets; offsets rebased by off_base)
// into h->sd_ids.  batch_bytes bounds the bytes a new string can add.
static gb_status strdict_encode(gb_agg *h, const uint8_t *bytes, const int64_t *offs, int64_t off_base,
                                const uint64_t *valid, u64 n, u64 batch_bytes, cudaStream_t st) {
    gb_status s;
    if (!h->sd_cap) {
        u64 cap = 1024;
        while (cap < 2 * std::max<u64>(h->est_groups, 512)) cap <<= 1;
        if ((s = strdict_init(h, cap, st))) return s;
    }
    // the arena can take every string of this batch
    u64 used = 0;
    GB_CUDA(cudaMemcpyAsync(&used, (u64 *)h->sd_ctr.p + 1, 8, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    // arena entries are padded to 8 bytes: at most 7 more per non-empty string
    batch_bytes += 7 * std::min<u64>(n, batch_bytes);
    if (used + batch_bytes + 64 > h->sd_arena_cap) {
        const u64 ncap = std::max<u64>((used + batch_bytes) * 3 / 2 + 4096, h->sd_arena_cap * 2);
        DevBuf nb;
        if ((s = nb.ensure(ncap))) return s;
        if (used) GB_CUDA(cudaMemcpyAsync(nb.p, h->sd_arena.p, used, cudaMemcpyDeviceToDevice, st));
        GB_CUDA(cudaStreamSynchronize(st));
        h->sd_arena.release();
        h->sd_arena = nb;
        h->sd_arena_cap = ncap;
    }
    if ((s = h->sd_ids.ensure(n * 8 + 8)) || (s = h->sd_retry_a.ensure(n * 4 + 8)) ||
        (s = h->sd_retry_b.ensure(n * 4 + 8)))
        return s;
    const u32 *rows = nullptr;
    u64 count = n;
    u32 *retry = (u32 *)h->sd_retry_a.p;
    u32 *other = (u32 *)h->sd_retry_b.p;
    Ctl *dctl = (Ctl *)h->ctl_buf.p;
    for (int round = 0; round < 40 && count; round++) {
        GB_CUDA(cudaMemsetAsync(&dctl->aux1, 0, 4, st));
        StrDictRef D = strdict_ref(h);
        {
            ProfScope ps(h, "k_strdict_encode", st);
            if ((s = strdict_launch_encode(D, bytes, offs, off_base, valid, count, rows, (long long *)h->sd_ids.p, retry,
                                           &dctl->aux1, &dctl->aux0, st)))
                return s;
        }
        h->launches++;
        u32 nretry = 0, err = 0;
        GB_CUDA(cudaMemcpyAsync(&nretry, &dctl->aux1, 4, cudaMemcpyDeviceToHost, st));
        GB_CUDA(cudaMemcpyAsync(&err, (u64 *)h->sd_ctr.p + 2, 4, cudaMemcpyDeviceToHost, st));
        GB_CUDA(cudaStreamSynchronize(st));
        if (err & ERR_TIMEOUT) {
            set_error("string dictionary: a bounded wait for a published string gave up");
            return GB_ERR_TIMEOUT;
        }
        if (!nretry) return GB_OK;
        if ((s = strdict_grow(h, h->sd_cap * 2, st))) return s;
        rows = retry;
        count = nretry;
        std::swap(retry, other);
    }
    set_error("string dictionary growth did not converge");
    return GB_ERR_OOM;
}

// The output column of the VARCHAR key.
static int str_out_col(const gb_agg *h) { return h->plan.key_mode == KEY_STRING ? 0 : std::max(0, h->plan.str_key); }

// Turn the emitted ids of a VARCHAR key column into offsets + bytes (a
// negative id, the NULL string of a pair key, becomes NULL).
static gb_status strdict_emit(gb_agg *h, const long long *ids, u64 n, cudaStream_t st) {
    gb_status s;
    if ((s = h->str_lens.ensure(n * 8 + 8)) || (s = h->out_str_offs.ensure(n * 8 + 16)) ||
        (s = h->scan_tmp.ensure(((n + 1023) / 1024 + 1) * 8)))
        return s;
    StrDictRef D = strdict_ref(h);
    if ((s = strdict_launch_lengths(D, ids, n, (int64_t *)h->str_lens.p, st,
                                    (uint64_t *)h->out_valid[str_out_col(h)].p)))
        return s;
    int64_t total = 0;
    if ((s = device_exclusive_scan((const int64_t *)h->str_lens.p, (int64_t *)h->out_str_offs.p, n,
                                   (int64_t *)h->scan_tmp.p, st, &total)))
        return s;
    if ((s = h->out_str_bytes.ensure((size_t)total + 16))) return s;
    if ((s = strdict_launch_gather(D, ids, n, (const int64_t *)h->out_str_offs.p, (uint8_t *)h->out_str_bytes.p, st)))
        return s;
    h->launches += 4;
    return GB_OK;
}

// ---------------------------------------------------------------- compile
// The plan's predicates from h->filters (validated).
static gb_status compile_filters(gb_agg *h) {
    Plan &P = h->plan;
    const int nc = (int)h->col_types.size();
    // literals (IN sets sorted and deduplicated, string bytes) are copied into
    // the handle: a host copy the filters point at, and one device buffer
    std::vector<uint8_t> lit;
    std::vector<size_t> at(h->filters.size(), 0);
    std::vector<u64> cnt(h->filters.size(), 0);
    for (size_t i = 0; i < h->filters.size(); i++) {
        const gb_filter &f = h->filters[i];
        if (i >= GB_MAX_FILTERS) {
            set_error("too many filters (max %d)", GB_MAX_FILTERS);
            return GB_ERR_UNSUPPORTED;
        }
        const int t = (f.col >= 0 && f.col < nc) ? h->col_types[f.col] : -1;
        const bool is_int = t == GB_T_SMALLINT || t == GB_T_INTEGER || t == GB_T_BIGINT;
        const bool num_op = f.op >= GB_CMP_EQ && f.op <= GB_CMP_GE;
        const bool str_op = f.op >= GB_CMP_STR_EQ && f.op <= GB_CMP_NOT_LIKE;
        if (t < 0 || (num_op && t == GB_T_VARCHAR) || (f.op == GB_CMP_IN && !is_int) || (str_op && t != GB_T_VARCHAR) ||
            (!num_op && !str_op && f.op != GB_CMP_IN)) {
            set_error("filter %zu invalid (column %d, operator %d)", i, f.col, f.op);
            return GB_ERR_INVALID;
        }
        if (num_op) continue;
        const u64 lim = f.op == GB_CMP_IN ? GB_MAX_IN_SET : GB_MAX_STR_LITERAL;
        if (f.n > lim || (f.n && !f.data)) {
            set_error("filter %zu: literal of %llu elements (max %llu) or without data", i, (unsigned long long)f.n,
                      (unsigned long long)lim);
            return f.n > lim ? GB_ERR_UNSUPPORTED : GB_ERR_INVALID;
        }
        while (lit.size() % 8) lit.push_back(0);
        at[i] = lit.size();
        if (f.op == GB_CMP_IN) {
            std::vector<int64_t> v((const int64_t *)f.data, (const int64_t *)f.data + f.n);
            std::sort(v.begin(), v.end());
            v.erase(std::unique(v.begin(), v.end()), v.end());
            cnt[i] = v.size();
            lit.insert(lit.end(), (const uint8_t *)v.data(), (const uint8_t *)(v.data() + v.size()));
        } else {
            cnt[i] = f.n;
            lit.insert(lit.end(), (const uint8_t *)f.data, (const uint8_t *)f.data + f.n);
        }
    }
    lit.resize(lit.size() + 8, 0);
    if (lit.size() > 8) {
        if (gb_status s = h->filt_dev.ensure(lit.size())) return s;
        GB_CUDA(cudaMemcpy(h->filt_dev.p, lit.data(), lit.size(), cudaMemcpyHostToDevice));
    }
    h->filt_host.swap(lit);
    for (size_t i = 0; i < h->filters.size(); i++) {
        gb_filter &f = h->filters[i];
        const bool has_lit = f.op >= GB_CMP_IN;
        if (has_lit) {  // the handle's own copy from now on
            f.data = h->filt_host.data() + at[i];
            f.n = cnt[i];
        } else {
            f.data = nullptr;
            f.n = 0;
        }
        P.filters[i].col = f.col;
        P.filters[i].op = f.op;
        P.filters[i].ic = f.i_const;
        P.filters[i].dc = f.d_const;
        P.filters[i].ptr = has_lit ? (const uint8_t *)h->filt_dev.p + at[i] : nullptr;
        P.filters[i].n = has_lit ? cnt[i] : 0;
    }
    P.n_filters = (int)h->filters.size();
    return GB_OK;
}

static gb_status compile_plan(gb_agg *h) {
    Plan &P = h->plan;
    memset(&P, 0, sizeof P);
    const int nc = (int)h->col_types.size();
    if (nc <= 0 || nc > GB_MAX_COLS) {
        set_error("n_cols must be in [1, %d]", GB_MAX_COLS);
        return GB_ERR_INVALID;
    }
    for (int c = 0; c < nc; c++) {
        int t = h->col_types[c];
        if (t < GB_T_SMALLINT || t > GB_T_VARCHAR) {
            set_error("column %d: unknown type %d", c, t);
            return GB_ERR_INVALID;
        }
        P.cols[c].type = t;
    }
    P.n_cols = nc;
    const int ng = (int)h->group_cols.size();
    if (ng < 1 || ng > 2) {
        set_error("GROUP BY needs 1 or 2 key columns on the GPU path (got %d)", ng);
        return ng < 1 ? GB_ERR_INVALID : GB_ERR_UNSUPPORTED;
    }
    for (int i = 0; i < ng; i++) {
        int c = h->group_cols[i];
        if (c < 0 || c >= nc) {
            set_error("group column %d out of range", c);
            return GB_ERR_INVALID;
        }
        int t = h->col_types[c];
        if (t == GB_T_DOUBLE) {
            set_error("DOUBLE group keys are not supported on the GPU path");
            return GB_ERR_UNSUPPORTED;
        }
        P.key_col[i] = c;
        P.key_type[i] = t;
    }
    P.n_keys = ng;
    P.str_key = -1;
    if (ng == 1) {
        P.key_mode = (h->col_types[P.key_col[0]] == GB_T_VARCHAR) ? KEY_STRING : KEY_SINGLE;
        if (P.key_mode == KEY_STRING) {
            // the aggregation keys on a hidden BIGINT column of string ids
            if (nc + 1 > GB_MAX_COLS) {
                set_error("too many columns for a VARCHAR key (max %d)", GB_MAX_COLS - 1);
                return GB_ERR_UNSUPPORTED;
            }
            h->str_col = P.key_col[0];
            P.cols[nc].type = GB_T_BIGINT;
            P.key_col[0] = nc;
            P.key_type[0] = GB_T_BIGINT;
        }
    } else {
        P.str_key = -1;
        const bool s0 = P.key_type[0] == GB_T_VARCHAR, s1 = P.key_type[1] == GB_T_VARCHAR;
        if (s0 && s1) {
            set_error("two VARCHAR columns in one key are not supported on the GPU path");
            return GB_ERR_UNSUPPORTED;
        }
        if (s0 || s1) {
            // (int, varchar): the string column becomes 32-bit dense ids on a
            // hidden BIGINT column, packed beside the integer key
            // (RadixCount2ColIntStr, radix_count_agg.cpp:767-1358, keys the
            // pair by its string's hash; here by its dictionary id)
            const int pos = s0 ? 0 : 1;
            const int other = P.key_type[1 - pos];
            if (other != GB_T_SMALLINT && other != GB_T_INTEGER) {
                set_error("a VARCHAR pair key needs a SMALLINT or INTEGER partner on the GPU path");
                return GB_ERR_UNSUPPORTED;
            }
            if (nc + 1 > GB_MAX_COLS) {
                set_error("too many columns for a VARCHAR key (max %d)", GB_MAX_COLS - 1);
                return GB_ERR_UNSUPPORTED;
            }
            h->str_col = P.key_col[pos];
            P.cols[nc].type = GB_T_BIGINT;
            P.key_col[pos] = nc;
            P.key_type[pos] = GB_T_INTEGER;
            P.str_key = pos;
        }
        int ba = type_bits(P.key_type[0]), bb = type_bits(P.key_type[1]);
        if (ba + bb + 2 <= 64) {
            P.key_mode = KEY_PACKED;
            P.key_bits_a = ba;
            P.key_bits_b = bb;
        } else if (ba + bb == 64) {
            P.key_mode = KEY_WIDE;
        } else {
            set_error("two-column key wider than 64 bits (BIGINT in a pair) is not supported on the GPU path");
            return GB_ERR_UNSUPPORTED;
        }
    }
    if (gb_status fs = compile_filters(h)) return fs;

    // state words: 0 = row count; ops deduplicated per (kind, column)
    int words = 1;
    P.word_init[0] = 0;
    auto find_or_add_op = [&](int kind, int col) -> int {
        for (int i = 0; i < P.n_ops; i++)
            if (P.ops[i].kind == kind && P.ops[i].col == col) return P.ops[i].word;
        if (P.n_ops >= GB_MAX_OPS || words >= GB_MAX_WORDS) return -1;
        Op &o = P.ops[P.n_ops++];
        o.kind = (uint8_t)kind;
        o.col = (uint8_t)col;
        o.word = (uint8_t)words;
        u64 init = 0;
        if (kind == OP_MIN_I || kind == OP_MIN_F) init = 0x7fffffffffffffffull;
        if (kind == OP_MAX_I || kind == OP_MAX_F) init = 0x8000000000000000ull;
        P.word_init[words] = init;
        return words++;
    };
    h->emit.clear();
    h->out_types.clear();
    for (int i = 0; i < ng; i++)
        h->out_types.push_back((P.key_mode == KEY_STRING || (ng == 2 && P.str_key == i)) ? GB_T_VARCHAR : P.key_type[i]);
    if (h->aggs.empty() || h->aggs.size() > GB_MAX_AGGS) {
        set_error("need 1..%d aggregates", GB_MAX_AGGS);
        return GB_ERR_INVALID;
    }
    for (size_t a = 0; a < h->aggs.size(); a++) {
        const gb_agg_desc &d = h->aggs[a];
        EmitAgg e{};
        e.kind = d.kind;
        e.val_word = -1;
        e.cnt_word = 0;
        e.in_type = -1;
        if (d.kind == GB_AGG_COUNT_STAR) {
            e.out_type = GB_T_BIGINT;
        } else {
            if (d.col < 0 || d.col >= nc || d.kind < 0 || d.kind > GB_AGG_COUNT_DISTINCT) {
                set_error("aggregate %zu: invalid kind or column", a);
                return GB_ERR_INVALID;
            }
            int t = h->col_types[d.col];
            e.in_type = t;
            if (t == GB_T_VARCHAR) {
                set_error("aggregate %zu over VARCHAR is not supported on the GPU path", a);
                return GB_ERR_UNSUPPORTED;
            }
            if (d.kind == GB_AGG_COUNT_DISTINCT) {
                // NULLs never enter the value set: no non-NULL count word
                if (t == GB_T_DOUBLE) {
                    set_error("COUNT(DISTINCT) over DOUBLE is not supported on the GPU path");
                    return GB_ERR_UNSUPPORTED;
                }
                e.out_type = GB_T_BIGINT;
                e.val_word = find_or_add_op(OP_DIST, d.col);
                if (e.val_word < 0) goto too_many;
                h->emit.push_back(e);
                h->out_types.push_back(e.out_type);
                continue;
            }
            bool nullable = (h->nullable_mask >> d.col) & 1ull;
            int cntw = 0;
            if (nullable) cntw = find_or_add_op(OP_CNT_NN, d.col);
            if (cntw < 0) goto too_many;
            e.cnt_word = cntw;
            bool isf = (t == GB_T_DOUBLE);
            switch (d.kind) {
            case GB_AGG_COUNT: e.out_type = GB_T_BIGINT; break;
            case GB_AGG_SUM:
                e.out_type = isf ? GB_T_DOUBLE : GB_T_BIGINT;
                e.val_word = find_or_add_op(isf ? OP_ADD_F : OP_ADD_I, d.col);
                break;
            case GB_AGG_AVG:
                e.out_type = GB_T_DOUBLE;
                e.val_word = find_or_add_op(isf ? OP_ADD_F : OP_ADD_I, d.col);
                break;
            case GB_AGG_MIN:
                e.out_type = t;
                e.val_word = find_or_add_op(isf ? OP_MIN_F : OP_MIN_I, d.col);
                break;
            case GB_AGG_MAX:
                e.out_type = t;
                e.val_word = find_or_add_op(isf ? OP_MAX_F : OP_MAX_I, d.col);
                break;
            }
            if (d.kind != GB_AGG_COUNT && e.val_word < 0) goto too_many;
        }
        h->emit.push_back(e);
        h->out_types.push_back(e.out_type);
    }
    P.words = words;
    P.n_dist = 0;
    for (int i = 0; i < P.n_ops; i++) {
        P.ops[i].dset = 0;
        if (P.ops[i].kind == OP_DIST) P.ops[i].dset = (uint8_t)P.n_dist++;
    }
    if (P.n_dist > GB_MAX_DISTINCT) {
        set_error("at most %d COUNT(DISTINCT) columns per query", GB_MAX_DISTINCT);
        return GB_ERR_UNSUPPORTED;
    }
    // the NULL-key group of a nullable BIGINT key has no spare key value
    h->dist_null_sets = P.n_dist && P.key_mode == KEY_SINGLE && P.key_type[0] == GB_T_BIGINT &&
                        ((h->nullable_mask >> P.key_col[0]) & 1ull);
    // a non-NULL 16/32-bit key and 16/32-bit distinct columns: 8-byte pair slots
    P.dnarrow = 0;
    if (P.n_dist && P.key_mode == KEY_SINGLE && h->str_col < 0 &&
        (P.key_type[0] == GB_T_SMALLINT || P.key_type[0] == GB_T_INTEGER) &&
        !((h->nullable_mask >> P.key_col[0]) & 1ull)) {
        P.dnarrow = 1;
        for (int i = 0; i < P.n_ops; i++)
            if (P.ops[i].kind == OP_DIST && h->col_types[P.ops[i].col] != GB_T_SMALLINT &&
                h->col_types[P.ops[i].col] != GB_T_INTEGER)
                P.dnarrow = 0;
    }
    if (h->str_col >= 0) P.n_cols = nc + 1;
    {
        int need = words + 1;
        int stride = need <= 4 ? (int)next_pow2(need) : ((need + 3) / 4) * 4;
        P.stride = stride;
    }
    return GB_OK;
too_many:
    set_error("too many distinct aggregate states (max %d)", GB_MAX_OPS);
    return GB_ERR_UNSUPPORTED;
}

static gb_status alloc_outputs(gb_agg *h, u64 rows) {
    size_t nout = h->out_types.size();
    h->out_cols.resize(nout);
    h->out_valid.resize(nout);
    for (size_t c = 0; c < nout; c++) {
        const int tsz = h->out_types[c] == GB_T_VARCHAR ? 8 : type_size(h->out_types[c]);
        gb_status s = h->out_cols[c].ensure((size_t)rows * tsz + 64);
        if (s) return s;
        s = h->out_valid[c].ensure(((size_t)rows + 63) / 64 * 8 + 64);
        if (s) return s;
    }
    h->out_cap = rows;
    return GB_OK;
}

static void fill_emit(gb_agg *h, EmitArgs &E, std::vector<DevBuf> &cols, std::vector<DevBuf> &valid, u64 cap) {
    memset(&E, 0, sizeof E);
    E.n_aggs = (int)h->emit.size();
    E.n_keys = h->plan.n_keys;
    for (int a = 0; a < E.n_aggs; a++) E.aggs[a] = h->emit[a];
    for (size_t c = 0; c < cols.size(); c++) {
        E.out[c] = cols[c].p;
        E.valid[c] = (uint64_t *)valid[c].p;
    }
    E.out_cap = cap;
}

// ------------------------------------------------------------ TopN host
static gb_status run_topn(gb_agg *h, cudaStream_t st) {
    const u64 n = h->n_rows_out;
    const int K = (int)h->topn_limit;
    const size_t nout = h->out_types.size();
    TopnArgs A{};
    A.order_col = h->out_cols[h->topn_col].p;
    A.order_type = h->out_types[h->topn_col];
    A.order_valid = (const uint64_t *)h->out_valid[h->topn_col].p;
    A.ascending = h->topn_asc ? 1 : 0;
    A.n_keys = h->plan.n_keys;
    A.key0 = h->out_cols[0].p;
    A.key_type0 = h->out_types[0];
    if (A.n_keys > 1) {
        A.key1 = h->out_cols[1].p;
        A.key_type1 = h->out_types[1];
    }
    A.K = K;
    // the best K plus up to sortn - K candidates between sorts: a wide
    // candidate buffer lets the threshold rise after few sorts
    int sortn = (int)next_pow2((u64)2 * K);
    if (sortn < 1024) sortn = 1024;
    size_t smem = (size_t)sortn * (8 + 8 + 4);
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_topn, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
        attr = true;
    }
    int grid = (int)std::min<u64>((u64)sm_count() * 2, std::max<u64>(1, n / 4096));
    gb_status s;
    if ((s = h->topn_ids_a.ensure((size_t)grid * K * 4))) return s;
    if ((s = h->topn_ids_b.ensure((size_t)K * 4 + 64))) return s;
    if ((s = h->topn_cnt.ensure((size_t)grid * 4 + 64))) return s;
    GB_CUDA(cudaMemsetAsync(h->topn_ids_a.p, 0xff, (size_t)grid * K * 4, st));
    const bool small = K <= 32 && h->topn_small;  // warp-register lists
    {
        ProfScope ps(h, "k_topn", st);
        if (small) k_topn_small<<<grid, 512, 0, st>>>(A, nullptr, n, (u32 *)h->topn_ids_a.p, (u32 *)h->topn_cnt.p);
        else k_topn<<<grid, 512, smem, st>>>(A, nullptr, n, (u32 *)h->topn_ids_a.p, (u32 *)h->topn_cnt.p, sortn);
    }
    h->launches++;
    GB_CUDA(cudaGetLastError());
    // second pass over the grid*K candidate ids (padding ids are skipped)
    if (small)
        k_topn_small<<<1, 512, 0, st>>>(A, (const u32 *)h->topn_ids_a.p, (u64)grid * K, (u32 *)h->topn_ids_b.p,
                                        (u32 *)h->topn_cnt.p);
    else
        k_topn<<<1, 512, smem, st>>>(A, (const u32 *)h->topn_ids_a.p, (u64)grid * K, (u32 *)h->topn_ids_b.p,
                                     (u32 *)h->topn_cnt.p, sortn);
    h->launches++;
    GB_CUDA(cudaGetLastError());
    u32 kf = 0;
    GB_CUDA(cudaMemcpyAsync(&kf, h->topn_cnt.p, 4, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    // gather rows into top_cols
    h->top_cols.resize(nout);
    h->top_valid.resize(nout);
    for (size_t c = 0; c < nout; c++) {
        if ((s = h->top_cols[c].ensure((size_t)K * 8 + 64))) return s;
        if ((s = h->top_valid[c].ensure(((size_t)K + 63) / 64 * 8 + 64))) return s;
        GB_CUDA(cudaMemsetAsync(h->top_valid[c].p, 0xff, ((size_t)K + 63) / 64 * 8 + 8, st));
    }
    if ((s = h->types_dev.ensure(nout * 4))) return s;
    GB_CUDA(cudaMemcpyAsync(h->types_dev.p, h->out_types.data(), nout * 4, cudaMemcpyHostToDevice, st));
    EmitArgs src, dst;
    fill_emit(h, src, h->out_cols, h->out_valid, h->out_cap);
    fill_emit(h, dst, h->top_cols, h->top_valid, K);
    if (kf > 0) {
        k_gather_rows<<<1, 256, 0, st>>>((const u32 *)h->topn_ids_b.p, kf, (int)nout, src, dst,
                                         (const int32_t *)h->types_dev.p);
        h->launches++;
        GB_CUDA(cudaGetLastError());
    }
    h->n_rows_out = kf;
    h->topn_applied = true;
    return GB_OK;
}

// =================================================================== C ABI
extern "C" {

const char *gb_last_error(void) { return g_err.c_str(); }
int gb_abi_version(void) { return GB_ABI_VERSION; }

gb_status gb_agg_estimate_bytes(const gb_agg_spec *spec, uint64_t nrows, uint64_t *bytes) {
    if (!spec || !bytes || spec->n_cols == 0 || !spec->col_types || spec->n_groups == 0 || !spec->group_cols ||
        spec->n_aggs == 0 || !spec->aggs || (spec->n_filters && !spec->filters)) {
        set_error("incomplete spec");
        return GB_ERR_INVALID;
    }
    gb_agg h;  // plan only: nothing is allocated on the device
    h.col_types.assign(spec->col_types, spec->col_types + spec->n_cols);
    h.group_cols.assign(spec->group_cols, spec->group_cols + spec->n_groups);
    h.aggs.assign(spec->aggs, spec->aggs + spec->n_aggs);
    if (spec->n_filters) h.filters.assign(spec->filters, spec->filters + spec->n_filters);
    h.nullable_mask = spec->nullable_mask;
    gb_status s = compile_plan(&h);
    if (s) return s;
    const u64 est = std::max<u64>(1, std::min<u64>(spec->est_groups ? spec->est_groups : (1u << 15),
                                                   std::max<u64>(nrows, 1)));
    const u64 cap = std::max<u64>(1024, next_pow2(est * 2));
    u64 b = (cap + 2) * (u64)h.plan.stride * 8;                        // hash table
    for (int t : h.out_types) b += (cap + 2) * (u64)(t == GB_T_VARCHAR ? 8 : type_size(t)) + (cap + 2) / 8;
    b += (u64)((1u << 16) + 4096) * (1 + h.plan.words) * 8;            // spill records
    if (h.str_col >= 0) b += 4 * 2 * cap * 8 + 40 * est + 16 * est;    // dictionary, arena, emitted strings
    if (h.plan.n_dist)                                                   // (group, value) pair sets
        b += std::max<u64>(1024, next_pow2(2 * std::max<u64>(nrows, 1))) * 16 * h.plan.n_dist *
             (h.dist_null_sets ? 2 : 1);
    *bytes = b;
    return GB_OK;
}

gb_status gb_agg_set_filters(gb_agg *h, const gb_filter *filters, uint32_t n_filters) {
    if (!h || (n_filters && !filters)) return GB_ERR_INVALID;
    if (h->rows_ingested || h->finalized) {
        set_error("filters are replaced after create or reset, before the first ingest");
        return GB_ERR_STATE;
    }
    std::vector<gb_filter> old = h->filters;
    h->filters.assign(filters, filters + n_filters);
    if (gb_status s = compile_filters(h)) {
        h->filters = old;
        compile_filters(h);
        return s;
    }
    // a radix handle's partition pass depends on the predicates: re-prepare
    // when they change which pass it takes
    if (h->mode == 1 && radix_spec_of(h->plan, h->rplan, h->nullable_mask) != h->rplan.spec) {
        RadixPlan R;
        if (gb_status s = radix_prepare(h->plan, R, std::max<u64>(h->est_groups, 1u << 16), h->nullable_mask)) {
            h->filters = old;
            compile_filters(h);
            set_error("these filters do not fit the handle's radix plan");
            return s;
        }
        h->rplan = R;
    }
    return GB_OK;
}

gb_status gb_agg_create(const gb_agg_spec *spec, gb_agg **out) {
    if (!spec || !out) {
        set_error("null spec/out");
        return GB_ERR_INVALID;
    }
    *out = nullptr;
    if (spec->n_cols == 0 || !spec->col_types || spec->n_groups == 0 || !spec->group_cols || spec->n_aggs == 0 ||
        !spec->aggs || (spec->n_filters && !spec->filters)) {
        set_error("incomplete spec");
        return GB_ERR_INVALID;
    }
    gb_agg *h = new gb_agg();
    h->col_types.assign(spec->col_types, spec->col_types + spec->n_cols);
    h->group_cols.assign(spec->group_cols, spec->group_cols + spec->n_groups);
    h->aggs.assign(spec->aggs, spec->aggs + spec->n_aggs);
    if (spec->n_filters) h->filters.assign(spec->filters, spec->filters + spec->n_filters);
    h->nullable_mask = spec->nullable_mask;
    h->est_groups = spec->est_groups;
    gb_status s = compile_plan(h);
    if (s) {
        delete h;
        return s;
    }
    gb_apply_tuning(h);
    u64 est = h->est_groups ? h->est_groups : (1u << 15);
    h->cap = h->mode == 1 ? 4096 : std::max<u64>(1024, next_pow2(est * 2));
    if ((s = h->ctl_buf.ensure(sizeof(Ctl)))) {
        delete h;
        return s;
    }
    cudaError_t e = cudaMemset(h->ctl_buf.p, 0, sizeof(Ctl));
    if (e != cudaSuccess) {
        delete h;
        return cuda_fail(e, "cudaMemset");
    }
    if ((s = init_table(h, h->table, h->cap, 0))) {
        delete h;
        return s;
    }
    // the table is initialised on the legacy stream: finish before the caller
    // ingests on a stream that does not synchronise with it
    e = cudaStreamSynchronize(0);
    if (e != cudaSuccess) {
        delete h;
        return cuda_fail(e, "cudaStreamSynchronize");
    }
    *out = h;
    return GB_OK;
}

gb_status gb_agg_set_topn(gb_agg *h, uint32_t col_idx, int32_t ascending, uint64_t limit) {
    if (!h) return GB_ERR_INVALID;
    if (col_idx >= h->out_types.size()) {
        set_error("TopN column %u out of range", col_idx);
        return GB_ERR_INVALID;
    }
    h->topn = true;
    h->topn_col = col_idx;
    h->topn_asc = ascending != 0;
    h->topn_limit = limit;
    return GB_OK;
}

gb_status gb_agg_set_row_limit(gb_agg *h, uint64_t limit) {
    if (!h) return GB_ERR_INVALID;
    h->row_limit = limit;
    return GB_OK;
}

gb_status gb_agg_ingest(gb_agg *h, const gb_col *cols, uint64_t nrows, int32_t mem, void *stream) {
    if (!h || (!cols && nrows)) {
        set_error("null handle/columns");
        return GB_ERR_INVALID;
    }
    if (h->finalized) {
        set_error("ingest after finalize (call gb_agg_reset first)");
        return GB_ERR_STATE;
    }
    if (nrows == 0) return GB_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (gb_status s0 = apply_reset(h, st)) return s0;
    const int nc = (int)h->col_types.size();  // spec columns (the plan may add a hidden id column)
    for (int c = 0; c < nc; c++) {
        if (!cols[c].data && !(h->col_types[c] == GB_T_VARCHAR && cols[c].offsets)) {
            set_error("column %d has no data pointer", c);
            return GB_ERR_INVALID;
        }
        if (h->col_types[c] == GB_T_VARCHAR && !cols[c].offsets) {
            set_error("VARCHAR column %d needs offsets", c);
            return GB_ERR_INVALID;
        }
        if (cols[c].validity && !((h->nullable_mask >> c) & 1ull)) {
            set_error("column %d carries a validity mask but the spec declares it NOT NULL", c);
            return GB_ERR_INVALID;
        }
    }
    gb_status s;
    if (mem == GB_MEM_DEVICE) {
        for (int c = 0; c < nc; c++) {
            h->plan.cols[c].data = cols[c].data;
            h->plan.cols[c].valid = cols[c].validity;
            h->plan.cols[c].offsets = cols[c].offsets;
        }
        if (h->str_col >= 0) {
            const gb_col &sc = cols[h->str_col];
            int64_t ends[2];
            GB_CUDA(cudaMemcpyAsync(&ends[0], sc.offsets, 8, cudaMemcpyDeviceToHost, st));
            GB_CUDA(cudaMemcpyAsync(&ends[1], sc.offsets + nrows, 8, cudaMemcpyDeviceToHost, st));
            GB_CUDA(cudaStreamSynchronize(st));
            if ((s = strdict_encode(h, (const uint8_t *)sc.data, sc.offsets, 0, sc.validity, nrows,
                                    (u64)(ends[1] - ends[0]), st)))
                return s;
            h->plan.cols[nc].data = h->sd_ids.p;
            h->plan.cols[nc].valid = nullptr;
        }
        s = h->mode == 1 ? radix_ingest(h, nrows, st) : run_ingest(h, nrows, st);
        h->rows_ingested += nrows;
        prof_collect(h);
        return s;
    }
    if (mem != GB_MEM_HOST) {
        set_error("mem must be GB_MEM_HOST or GB_MEM_DEVICE");
        return GB_ERR_INVALID;
    }
    // Host vectors: double-buffered chunks, copy of chunk i+1 overlaps the
    // aggregation of chunk i.
    if (!h->copy_stream) {
        GB_CUDA(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
        for (int b = 0; b < 2; b++) {
            GB_CUDA(cudaEventCreateWithFlags(&h->ev_copied[b], cudaEventDisableTiming));
            GB_CUDA(cudaEventCreateWithFlags(&h->ev_done[b], cudaEventDisableTiming));
        }
    }
    const u64 chunk = std::min<u64>(nrows, (u64)16 << 20);
    for (int b = 0; b < 2; b++) {
        h->stage[b].resize(3 * nc);
        for (int c = 0; c < nc; c++) {
            if (h->col_types[c] == GB_T_VARCHAR) {
                if ((s = h->stage[b][2 * nc + c].ensure((size_t)(chunk + 1) * 8))) return s;
            } else if ((s = h->stage[b][c].ensure((size_t)chunk * type_size(h->col_types[c]) + 64))) {
                return s;
            }
            if (cols[c].validity && (s = h->stage[b][nc + c].ensure((size_t)(chunk / 64 + 2) * 8))) return s;
        }
    }
    const u64 nchunks = (nrows + chunk - 1) / chunk;
    auto issue_copy = [&](u64 i) -> gb_status {
        int b = (int)(i & 1);
        u64 r0 = i * chunk, r1 = std::min<u64>(nrows, r0 + chunk);
        if (i >= 2) GB_CUDA(cudaStreamWaitEvent(h->copy_stream, h->ev_done[b], 0));
        for (int c = 0; c < nc; c++) {
            if (h->col_types[c] == GB_T_VARCHAR) {
                const int64_t *ho = cols[c].offsets;
                const u64 nb = (u64)(ho[r1] - ho[r0]);
                if (h->stage[b][c].n < nb + 16) {
                    GB_CUDA(cudaStreamSynchronize(h->copy_stream));
                    GB_CUDA(cudaDeviceSynchronize());
                    gb_status s2 = h->stage[b][c].ensure(nb + 16);
                    if (s2) return s2;
                }
                GB_CUDA(cudaMemcpyAsync(h->stage[b][c].p, (const char *)cols[c].data + ho[r0], nb,
                                        cudaMemcpyHostToDevice, h->copy_stream));
                GB_CUDA(cudaMemcpyAsync(h->stage[b][2 * nc + c].p, ho + r0, (r1 - r0 + 1) * 8, cudaMemcpyHostToDevice,
                                        h->copy_stream));
            } else {
                int ts = type_size(h->col_types[c]);
                GB_CUDA(cudaMemcpyAsync(h->stage[b][c].p, (const char *)cols[c].data + r0 * ts, (r1 - r0) * ts,
                                        cudaMemcpyHostToDevice, h->copy_stream));
            }
            if (cols[c].validity) {
                // chunk boundaries are multiples of 64 rows (chunk = 16Mi)
                GB_CUDA(cudaMemcpyAsync(h->stage[b][nc + c].p, cols[c].validity + r0 / 64, ((r1 - r0) + 63) / 64 * 8,
                                        cudaMemcpyHostToDevice, h->copy_stream));
            }
        }
        GB_CUDA(cudaEventRecord(h->ev_copied[b], h->copy_stream));
        return GB_OK;
    };
    s = issue_copy(0);
    if (s) return s;
    for (u64 i = 0; i < nchunks; i++) {
        int b = (int)(i & 1);
        if (i + 1 < nchunks && (s = issue_copy(i + 1))) return s;
        GB_CUDA(cudaStreamWaitEvent(st, h->ev_copied[b], 0));
        u64 r0 = i * chunk, r1 = std::min<u64>(nrows, r0 + chunk);
        for (int c = 0; c < nc; c++) {
            h->plan.cols[c].data = h->stage[b][c].p;
            h->plan.cols[c].valid = cols[c].validity ? (const uint64_t *)h->stage[b][nc + c].p : nullptr;
            h->plan.cols[c].offsets = nullptr;
            if (h->col_types[c] == GB_T_VARCHAR) {
                // the staged offsets are the caller's (absolute): the bytes
                // pointer is shifted so that data + offsets[r] is row r's string
                h->plan.cols[c].offsets = (const int64_t *)h->stage[b][2 * nc + c].p;
                h->plan.cols[c].data = (const uint8_t *)h->stage[b][c].p - cols[c].offsets[r0];
            }
        }
        if (h->str_col >= 0) {
            const int c = h->str_col;
            const int64_t *ho = cols[c].offsets;
            if ((s = strdict_encode(h, (const uint8_t *)h->stage[b][c].p, (const int64_t *)h->stage[b][2 * nc + c].p,
                                    ho[r0], h->plan.cols[c].valid, r1 - r0, (u64)(ho[r1] - ho[r0]), st)))
                return s;
            h->plan.cols[nc].data = h->sd_ids.p;
            h->plan.cols[nc].valid = nullptr;
        }
        if ((s = (h->mode == 1 ? radix_ingest(h, r1 - r0, st) : run_ingest(h, r1 - r0, st)))) return s;
        h->rows_ingested += r1 - r0;
        GB_CUDA(cudaEventRecord(h->ev_done[b], st));
    }
    // the caller may reuse its host buffers once the call returns
    GB_CUDA(cudaStreamSynchronize(h->copy_stream));
    prof_collect(h);
    return GB_OK;
}

gb_status gb_agg_finalize(gb_agg *h, void *stream) {
    if (!h) return GB_ERR_INVALID;
    if (h->finalized) return GB_OK;
    cudaStream_t st = (cudaStream_t)stream;
    gb_status s;
    if ((s = apply_reset(h, st))) return s;
    Ctl *dctl = (Ctl *)h->ctl_buf.p;
    if (h->mode == 1) {
        if ((s = radix_emit(h, st))) return s;
    } else {
        if ((s = alloc_outputs(h, h->cap + 2))) return s;
        for (size_t c = 0; c < h->out_valid.size(); c++)
            GB_CUDA(cudaMemsetAsync(h->out_valid[c].p, 0xff, (h->out_cap + 63) / 64 * 8, st));
        GB_CUDA(cudaMemsetAsync(&dctl->out_count, 0, 4, st));
    }
    GB_CUDA(cudaMemsetAsync(&dctl->err, 0, 4, st));
    EmitArgs E;
    fill_emit(h, E, h->out_cols, h->out_valid, h->out_cap);
    {
        ProfScope ps(h, "k_compact", st);
        // slots per thread: up to COMPACT_PER, fewer where the table would
        // otherwise occupy under two CTAs per SM
        const u64 slots_n = h->cap + 2;
        int per = COMPACT_PER;
        while (per > 1 && slots_n / ((u64)per * 256) < (u64)sm_count() * 2) per >>= 1;
        k_compact<<<grid_for((slots_n + per - 1) / per, 256, sm_count() * 4), 256, 0, st>>>(
            h->plan, (const u64 *)h->table.p, h->cap, h->plan.stride, E, dctl, per);
    }
    h->launches++;
    GB_CUDA(cudaGetLastError());
    if ((s = read_ctl(h, st))) return s;
    if ((s = check_err(h))) return s;
    h->n_rows_out = h->ctl_host.out_count;
    h->topn_applied = false;
    if (h->str_col >= 0) {
        // VARCHAR keys: the TopN hint is not applied (the ORDER BY above sorts
        // the full result); ids become offsets + bytes
        if ((s = strdict_emit(h, (const long long *)h->out_cols[str_out_col(h)].p, h->n_rows_out, st))) return s;
    } else if (h->topn && h->topn_limit > 0 && h->topn_limit <= 1024 && h->n_rows_out > 0) {
        if ((s = run_topn(h, st))) return s;
    }
    h->finalized = true;
    h->has_result = false;
    prof_collect(h);
    return GB_OK;
}

static void fill_result_view(gb_agg *h, gb_result *out, bool host) {
    size_t nout = h->out_types.size();
    h->res_ptrs.resize(nout);
    h->res_valid.resize(nout);
    h->res_offsets.assign(nout, nullptr);
    for (size_t c = 0; c < nout; c++) {
        if (h->out_types[c] == GB_T_VARCHAR) {
            h->res_ptrs[c] = host ? h->host_str_bytes.p : h->out_str_bytes.p;
            h->res_offsets[c] = (const int64_t *)(host ? h->host_str_offs.p : h->out_str_offs.p);
            h->res_valid[c] = (const uint64_t *)(host ? h->host_valid[c].p : h->out_valid[c].p);
            continue;
        }
        if (host) {
            h->res_ptrs[c] = h->host_cols[c].p;
            h->res_valid[c] = (const uint64_t *)h->host_valid[c].p;
        } else {
            auto &cols = h->topn_applied ? h->top_cols : h->out_cols;
            auto &val = h->topn_applied ? h->top_valid : h->out_valid;
            h->res_ptrs[c] = cols[c].p;
            h->res_valid[c] = (const uint64_t *)val[c].p;
        }
    }
    out->n_rows = h->n_rows_out;
    out->n_cols = (uint32_t)nout;
    out->types = h->out_types.data();
    out->data = h->res_ptrs.data();
    out->offsets = h->res_offsets.data();
    out->validity = h->res_valid.data();
}

gb_status gb_agg_result(gb_agg *h, gb_result *out) {
    if (!h || !out) return GB_ERR_INVALID;
    if (!h->finalized) {
        set_error("result before finalize");
        return GB_ERR_STATE;
    }
    if (!h->has_result) {
        size_t nout = h->out_types.size();
        h->host_cols.resize(nout);
        h->host_valid.resize(nout);
        u64 n = h->n_rows_out;
        if (h->row_limit && n > h->row_limit) n = h->row_limit;
        auto &cols = h->topn_applied ? h->top_cols : h->out_cols;
        auto &val = h->topn_applied ? h->top_valid : h->out_valid;
        for (size_t c = 0; c < nout; c++) {
            size_t vbytes = ((size_t)n + 63) / 64 * 8;
            gb_status s;
            if ((s = h->host_valid[c].ensure(vbytes + 8))) return s;
            if (vbytes) GB_CUDA(cudaMemcpyAsync(h->host_valid[c].p, val[c].p, vbytes, cudaMemcpyDeviceToHost, 0));
            if (h->out_types[c] == GB_T_VARCHAR) {
                if ((s = h->host_str_offs.ensure((n + 1) * 8))) return s;
                GB_CUDA(cudaMemcpy(h->host_str_offs.p, h->out_str_offs.p, (n + 1) * 8, cudaMemcpyDeviceToHost));
                const int64_t nb = ((const int64_t *)h->host_str_offs.p)[n];
                if ((s = h->host_str_bytes.ensure((size_t)nb + 8))) return s;
                if (nb) GB_CUDA(cudaMemcpy(h->host_str_bytes.p, h->out_str_bytes.p, nb, cudaMemcpyDeviceToHost));
                if ((s = h->host_cols[c].ensure(8))) return s;
                continue;
            }
            size_t bytes = (size_t)n * type_size(h->out_types[c]);
            if ((s = h->host_cols[c].ensure(bytes + 8))) return s;
            if (bytes) GB_CUDA(cudaMemcpyAsync(h->host_cols[c].p, cols[c].p, bytes, cudaMemcpyDeviceToHost, 0));
        }
        GB_CUDA(cudaStreamSynchronize(0));
        h->n_rows_out = n;
        h->has_result = true;
    }
    fill_result_view(h, out, true);
    return GB_OK;
}

gb_status gb_agg_result_device(gb_agg *h, gb_result *out) {
    if (!h || !out) return GB_ERR_INVALID;
    if (!h->finalized) {
        set_error("result before finalize");
        return GB_ERR_STATE;
    }
    fill_result_view(h, out, false);
    return GB_OK;
}

gb_status gb_agg_reset(gb_agg *h) {
    if (!h) return GB_ERR_INVALID;
    // the device work of the rewind (table, COUNT(DISTINCT) sets, control
    // words) runs on the stream of the handle's next ingest or finalize, so
    // a reset neither blocks the host nor races work on another stream
    h->pending_reset = true;
    h->n_groups = 0;
    h->sd_cap = 0;  // the string dictionary is rebuilt by the next ingest
    h->r_ready = false;
    h->rows_ingested = 0;
    h->finalized = false;
    h->has_result = false;
    h->topn_applied = false;
    h->n_rows_out = 0;
    h->launches = 0;
    h->rg_pruned = 0;
    return GB_OK;
}

void gb_agg_destroy(gb_agg *h) {
    if (!h) return;
    cudaDeviceSynchronize();
    gb_pq_release_scratch(h);
    h->table.release();
    h->table_old.release();
    h->spill.release();
    h->ctl_buf.release();
    for (auto &b : h->out_cols) b.release();
    for (auto &b : h->out_valid) b.release();
    for (auto &b : h->top_cols) b.release();
    for (auto &b : h->top_valid) b.release();
    for (DevBuf *b : {&h->sd_hash, &h->sd_ref, &h->sd_id, &h->sd_refid, &h->sd_ctr, &h->sd_arena, &h->sd_old_hash,
                      &h->sd_old_ref, &h->sd_old_id, &h->sd_old_refid, &h->sd_ids, &h->sd_retry_a, &h->sd_retry_b,
                      &h->out_str_offs, &h->out_str_bytes, &h->str_lens, &h->scan_tmp})
        b->release();
    h->host_str_offs.release();
    h->host_str_bytes.release();
    for (DevBuf *b : {&h->r_skeys, &h->r_scnt, &h->r_hist, &h->r_hot_keys, &h->r_hot_part, &h->r_cursor, &h->r_part,
                      &h->r_part2, &h->r_ovf, &h->r_off, &h->r_cap, &h->r_off2, &h->r_cap2, &h->r_hot_idx,
                      &h->r_hot_list, &h->r_hstate, &h->r_cand, &h->r_p2w, &h->filt_dev, &h->dsets, &h->dsets_old,
                      &h->null_sets,
                      &h->null_sets_old, &h->dmeta})
        b->release();
    h->topn_ids_a.release();
    h->topn_ids_b.release();
    h->topn_cnt.release();
    h->types_dev.release();
    for (auto &b : h->host_cols) b.release();
    for (auto &b : h->host_valid) b.release();
    for (int i = 0; i < 2; i++) {
        for (auto &b : h->stage[i]) b.release();
        if (h->ev_copied[i]) cudaEventDestroy(h->ev_copied[i]);
        if (h->ev_done[i]) cudaEventDestroy(h->ev_done[i]);
    }
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    for (auto &p : h->prof_pending) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    for (auto e : h->ev_pool) cudaEventDestroy(e);
    delete h;
}

uint64_t gb_agg_kernel_launches(const gb_agg *h) { return h ? h->launches : 0; }

uint64_t gb_agg_row_groups_pruned(const gb_agg *h) { return h ? h->rg_pruned : 0; }

gb_status gb_agg_set_option(gb_agg *h, const char *name, int64_t value) {
    if (!h || !name) return GB_ERR_INVALID;
    if (h->rows_ingested || h->finalized) {
        set_error("options must be set before the first ingest (or after reset)");
        return GB_ERR_STATE;
    }
    std::string n(name);
    if (n == "mode") {
        if (value < 0 || value > 2) {
            set_error("mode must be 0 (auto), 1 (hash) or 2 (radix)");
            return GB_ERR_INVALID;
        }
        h->mode_option = (int)value;
        int old_mode = h->mode;
        gb_apply_tuning(h);
        if (h->mode_option == 2 && h->mode != 1) {
            set_error("plan not eligible for radix mode (nullable value column or too many value columns)");
            return GB_ERR_UNSUPPORTED;
        }
        if (h->mode != old_mode) {
            u64 est = h->est_groups ? h->est_groups : (1u << 15);
            h->cap = h->mode == 1 ? 4096 : std::max<u64>(1024, next_pow2(est * 2));
            gb_status s = init_table(h, h->table, h->cap, 0);
            if (s) return s;
            GB_CUDA(cudaDeviceSynchronize());
        }
    } else if (n == "smem_slots") {
        if (value < 0 || value > 8192 || (value & (value - 1))) {
            set_error("smem_slots must be 0 or a power of two <= 8192");
            return GB_ERR_INVALID;
        }
        h->smem_slots = (int)value;
    } else if (n == "precombine") {
        h->precombine = value != 0;
        h->precombine_set = true;
    } else if (n == "topn_small") {
        if (value < 0 || value > 1) return GB_ERR_INVALID;
        h->topn_small = value != 0;
    } else if (n == "fast_ingest") {
        if (value < 0 || value > 1) return GB_ERR_INVALID;
        h->fast_ingest = value != 0;
    } else if (n == "ctas_per_sm") {
        if (value < 1 || value > 4) return GB_ERR_INVALID;
        h->ctas_per_sm = (int)value;
    } else if (n == "tile_rows") {
        if (value < 512 || value > (1 << 20) || value % 512) return GB_ERR_INVALID;
        h->tile_rows = (u32)value;
    } else if (n == "radix_bits") {
        if (h->mode != 1) {
            set_error("radix_bits applies to radix mode only");
            return GB_ERR_INVALID;
        }
        gb_status s = radix_set_bits(h->plan, h->rplan, (int)value);
        if (s) {
            set_error("radix_bits must be 6..12 and fit the partition pass's shared memory");
            return s;
        }
    } else if (n == "radix_precombine") {
        if (h->mode != 1 || value < 0 || value > 1) {
            set_error("radix_precombine applies to radix mode only and is 0 or 1");
            return GB_ERR_INVALID;
        }
        h->rplan.p2_pre = (int)value;
    } else if (n == "hot_slots") {
        if (h->mode != 1 || value < 64 || value > h->rplan.HS || (value & (value - 1))) return GB_ERR_INVALID;
        h->rplan.HS = (int)value;
        h->rplan.nh = std::min<int>(h->rplan.nh, (int)value / 2);
        h->rplan.nsup = std::min<int>(h->rplan.nsup, h->rplan.nh);
    } else {
        set_error("unknown option '%s'", name);
        return GB_ERR_INVALID;
    }
    return GB_OK;
}

int32_t gb_agg_get_mode(const gb_agg *h) { return h ? h->mode : -1; }

gb_status gb_agg_set_profiling(gb_agg *h, int32_t on) {
    if (!h) return GB_ERR_INVALID;
    h->profiling = on != 0;
    if (!on) h->stats.clear();
    return GB_OK;
}

uint32_t gb_agg_profile(const gb_agg *h, gb_kernel_stat *out, uint32_t max) {
    if (!h) return 0;
    uint32_t n = (uint32_t)std::min<size_t>(max, h->stats.size());
    for (uint32_t i = 0; i < n; i++) out[i] = h->stats[i];
    return (uint32_t)h->stats.size();
}

gb_status gb_engine_hash_aggregate(const int32_t *keys, const int32_t *values, uint64_t n, int32_t *out_keys,
                                   int64_t *out_sums, int64_t *out_counts, uint64_t cap, uint64_t *n_out) {
    if ((!keys || !values) && n) return GB_ERR_INVALID;
    int32_t types[2] = {GB_T_INTEGER, GB_T_INTEGER};
    int32_t gcols[1] = {0};
    gb_agg_desc aggs[2] = {{GB_AGG_SUM, 1}, {GB_AGG_COUNT_STAR, -1}};
    gb_agg_spec spec{};
    spec.n_cols = 2;
    spec.col_types = types;
    spec.n_groups = 1;
    spec.group_cols = gcols;
    spec.n_aggs = 2;
    spec.aggs = aggs;
    gb_agg *h = nullptr;
    gb_status s = gb_agg_create(&spec, &h);
    if (s) return s;
    gb_col cols[2] = {{keys, nullptr, nullptr}, {values, nullptr, nullptr}};
    if (!(s = gb_agg_ingest(h, cols, n, GB_MEM_HOST, nullptr)) && !(s = gb_agg_finalize(h, nullptr))) {
        gb_result r;
        if (!(s = gb_agg_result(h, &r))) {
            if (r.n_rows > cap) {
                set_error("%llu groups exceed output capacity %llu", (unsigned long long)r.n_rows,
                          (unsigned long long)cap);
                s = GB_ERR_INVALID;
            } else {
                memcpy(out_keys, r.data[0], r.n_rows * 4);
                memcpy(out_sums, r.data[1], r.n_rows * 8);
                memcpy(out_counts, r.data[2], r.n_rows * 8);
                *n_out = r.n_rows;
            }
        }
    }
    gb_agg_destroy(h);
    return s;
}

gb_status gb_host_alloc(void **ptr, size_t bytes) {
    if (!ptr) return GB_ERR_INVALID;
    GB_CUDA(cudaMallocHost(ptr, bytes ? bytes : 1));
    return GB_OK;
}
gb_status gb_host_free(void *ptr) {
    GB_CUDA(cudaFreeHost(ptr));
    return GB_OK;
}
gb_status gb_device_alloc(void **ptr, size_t bytes) {
    if (!ptr) return GB_ERR_INVALID;
    GB_CUDA(cudaMalloc(ptr, bytes ? bytes : 1));
    return GB_OK;
}
gb_status gb_device_free(void *ptr) {
    GB_CUDA(cudaFree(ptr));
    return GB_OK;
}
gb_status gb_memcpy(void *dst, const void *src, size_t bytes, int32_t kind) {
    cudaMemcpyKind k = kind == 0 ? cudaMemcpyHostToDevice : (kind == 1 ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice);
    GB_CUDA(cudaMemcpy(dst, src, bytes, k));
    return GB_OK;
}
gb_status gb_device_sync(void) {
    GB_CUDA(cudaDeviceSynchronize());
    return GB_OK;
}

}  // extern "C"

// ------------------------------------------------------ Parquet ingest hooks
gb_status gb_agg_view(gb_agg *h, AggView *v) {
    if (!h || !v) return GB_ERR_INVALID;
    if (h->finalized) {
        set_error("ingest after finalize (call gb_agg_reset first)");
        return GB_ERR_STATE;
    }
    v->n_cols = (int)h->col_types.size();
    v->str_col = h->str_col;
    v->col_types = h->col_types.data();
    v->n_filters = h->plan.n_filters;
    for (int i = 0; i < h->plan.n_filters; i++) v->filters[i] = h->plan.filters[i];
    v->nullable_mask = h->nullable_mask;
    return GB_OK;
}

void gb_agg_count_launch(gb_agg *h, int n) { h->launches += (u64)n; }

void gb_agg_count_pruned(gb_agg *h, uint64_t n) { h->rg_pruned += n; }

gb_status gb_agg_ingest_prefiltered(gb_agg *h, const gb_col *cols, uint64_t nrows, void *stream) {
    const int nf = h->plan.n_filters;
    h->plan.n_filters = 0;
    const uint64_t saved_mask = h->nullable_mask;
    gb_status s = gb_agg_ingest(h, cols, nrows, GB_MEM_DEVICE, stream);
    h->plan.n_filters = nf;
    h->nullable_mask = saved_mask;
    return s;
}

gb_status gb_agg_ingest_prefiltered_ids(gb_agg *h, const gb_col *cols, uint64_t nrows, const int64_t *ids,
                                        void *stream) {
    if (!h || h->str_col < 0 || h->finalized) {
        set_error("string ids need a handle with a VARCHAR group key that is not finalised");
        return GB_ERR_STATE;
    }
    if (nrows == 0) return GB_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (gb_status s0 = apply_reset(h, st)) return s0;
    const int nc = (int)h->col_types.size();
    for (int c = 0; c < nc; c++) {
        if (cols[c].validity && !((h->nullable_mask >> c) & 1ull)) {
            set_error("column %d carries a validity mask but the spec declares it NOT NULL", c);
            return GB_ERR_INVALID;
        }
        h->plan.cols[c].data = cols[c].data;
        h->plan.cols[c].valid = c == h->str_col ? nullptr : cols[c].validity;  // a NULL key arrives as id -1
        h->plan.cols[c].offsets = cols[c].offsets;
    }
    h->plan.cols[nc].data = ids;
    h->plan.cols[nc].valid = nullptr;
    const int nf = h->plan.n_filters;
    h->plan.n_filters = 0;
    gb_status s = h->mode == 1 ? radix_ingest(h, nrows, st) : run_ingest(h, nrows, st);
    h->plan.n_filters = nf;
    h->rows_ingested += nrows;
    prof_collect(h);
    return s;
}

gb_status gb_agg_encode_strings(gb_agg *h, const uint8_t *bytes, const int64_t *offsets, uint64_t n,
                                uint64_t total_bytes, void *stream, const int64_t **ids) {
    if (!h || h->str_col < 0) {
        set_error("string encode needs a handle with a VARCHAR group key");
        return GB_ERR_STATE;
    }
    gb_status s = strdict_encode(h, bytes, offsets, 0, nullptr, n, total_bytes, (cudaStream_t)stream);
    if (s) return s;
    *ids = (const int64_t *)h->sd_ids.p;
    return GB_OK;
}

struct gb_prof_mark {
    int stat;
    cudaEvent_t a;
};

gb_prof_mark *gb_agg_prof_begin(gb_agg *h, const char *name, cudaStream_t st) {
    if (!h->profiling) return nullptr;
    gb_prof_mark *m = new gb_prof_mark{prof_stat(h, name), prof_event(h)};
    cudaEventRecord(m->a, st);
    return m;
}

void gb_agg_prof_end(gb_agg *h, gb_prof_mark *m, cudaStream_t st) {
    if (!m) return;
    cudaEvent_t b = prof_event(h);
    cudaEventRecord(b, st);
    h->prof_pending.push_back({m->stat, m->a, b});
    delete m;
}

// tuning hook (defaults here; the autotuner overrides per shape)
void gb_apply_tuning(gb_agg *h) {
    const int words = h->plan.words;
    // shared table: 2x the estimated groups, at most ~96 KB so two CTAs fit
    u64 est = h->est_groups ? h->est_groups : 4096;
    u64 S = next_pow2(est * 2);
    u64 max_s = (96 * 1024) / (8 * (1 + words));
    u64 max_p2 = 1;
    while (max_p2 * 2 <= max_s) max_p2 *= 2;
    if (S > max_p2) S = max_p2;
    if (S < 256) S = 256;
    h->smem_slots = (int)S;
    h->ctas_per_sm = 2;
    h->block = 512;
    // radix mode for high-cardinality keys
    h->mode = 0;
    bool want_radix = h->mode_option == 2 || (h->mode_option == 0 && h->est_groups >= (1u << 20));
    if (want_radix && radix_prepare(h->plan, h->rplan, std::max<u64>(h->est_groups, 1u << 16), h->nullable_mask) ==
                          GB_OK)
        h->mode = 1;
}

#include "gb_batch.cuh"
