// gb_radix.cu — the radix-partitioned GROUP BY for high-cardinality keys.
//
// GB300 restatement of the reference's radix aggregators
// (src/execution/radix_count_agg.cpp:17-106 RadixCountAgg: scatter rows by
// top hash bits, aggregate each radix partition in its own open-addressing
// map, src/execution/simple_i64_count_map.hpp:20-109) generalised to every
// aggregate of the plan, with a heavy-hitter stage in front:
//
//   S  sample:  a strided sample of the keys is counted; keys whose sample
//               count clears a threshold form the "hot" set (at most HS/2).
//   P1 scatter: persistent CTAs stream the rows (coalesced loads); a hot key
//               is folded into the CTA's shared-memory hot table; any other
//               row is scattered as a (key, values) tuple into partition
//               p = top bits of its hash.  Per tile, partition slots are
//               reserved with one global atomic per touched partition.
//   P2 agg:     one CTA per partition folds the partition's tuples into a
//               shared-memory open-addressing table and emits its groups.
//   P3 hot:     per-CTA hot partials are reduced in a fixed order and the
//               hot groups are emitted.
//
// A key is either hot for the whole query or never, and lives in exactly one
// partition, so every group is emitted exactly once.  Bounded probes fall
// back to the HBM hash table (whose groups are emitted by the compaction
// kernel), which keeps the result exact whatever the key distribution.
#include <algorithm>
#include <cstring>
#include <vector>

#include "gb_kernels.cuh"
#include "gb_radix.h"

namespace gb {

__device__ __forceinline__ u32 part_of(u64 h, int pbits) { return pbits ? (u32)(h >> (64 - pbits)) : 0u; }
__device__ __forceinline__ u32 hot_slot(u64 h, int HS) { return (u32)h & (u32)(HS - 1); }
__device__ __forceinline__ u32 agg_slot(u64 h, int SP) { return (u32)(h >> 20) & (u32)(SP - 1); }

// ------------------------------------------------------------- sampling
__global__ void k_sample_count(const __grid_constant__ Plan P, u64 n, u64 step, u64 m, u64 *skeys, u32 *scnt,
                               u64 scap) {
    for (u64 i = blockIdx.x * (u64)blockDim.x + threadIdx.x; i < m; i += (u64)gridDim.x * blockDim.x) {
        const u64 r = i * step;
        if (r >= n) continue;
        if (P.n_filters && !pass_filters(P, r)) continue;
        u64 pk;
        if (make_key(P, r, pk) != 0) continue;
        u64 s = mix64(pk) & (scap - 1);
        for (u64 p = 0; p < scap; p++) {
            u64 k = *(volatile u64 *)&skeys[s];
            if (k == EMPTY_KEY) {
                u64 old = atomicCAS(&skeys[s], EMPTY_KEY, pk);
                if (old == EMPTY_KEY || old == pk) k = pk;
            }
            if (k == pk) {
                atomicAdd(&scnt[s], 1u);
                break;
            }
            s = (s + 1) & (scap - 1);
        }
    }
}

__global__ void k_sample_hist(const u64 *skeys, const u32 *scnt, u64 scap, u32 *hist) {
    __shared__ u32 h[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (u64 s = blockIdx.x * (u64)blockDim.x + threadIdx.x; s < scap; s += (u64)gridDim.x * blockDim.x)
        if (skeys[s] != EMPTY_KEY) atomicAdd(&h[min(scnt[s], 255u)], 1u);
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[i], h[i]);
}

// Keys with sample count >= t (the smallest t >= min_count that admits at
// most hot_max keys) go into the hot table.  hist[256] += sampled rows
// covered by hot keys, for sizing the partitions.
__global__ void k_hot_build(const u64 *skeys, const u32 *scnt, u64 scap, u32 *hist, u32 min_count, u32 hot_max,
                            u64 *hot_keys, int HS) {
    __shared__ u32 s_t;
    __shared__ u32 s_rows;
    if (threadIdx.x == 0) {
        u32 cum = 0, t = 256;
        for (int c = 255; c >= (int)min_count; c--) {
            if (cum + hist[c] > hot_max) break;
            cum += hist[c];
            t = c;
        }
        s_t = t;
        s_rows = 0;
    }
    __syncthreads();
    const u32 t = s_t;
    for (u64 s = blockIdx.x * (u64)blockDim.x + threadIdx.x; s < scap; s += (u64)gridDim.x * blockDim.x) {
        u64 k = skeys[s];
        if (k == EMPTY_KEY || scnt[s] < t || t > 255) continue;
        atomicAdd(&s_rows, scnt[s]);
        u32 h = hot_slot(mix64(k), HS);
        for (int p = 0; p < HS; p++) {
            u64 old = atomicCAS(&hot_keys[h], EMPTY_KEY, k);
            if (old == EMPTY_KEY || old == k) break;
            h = (h + 1) & (u32)(HS - 1);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_rows) atomicAdd(&hist[256], s_rows);
}

// ------------------------------------------------------------- P1 scatter
__device__ __forceinline__ void tuple_vals(const Plan &P, const RadixPlan &R, u64 r, u64 *tv) {
#pragma unroll
    for (int j = 0; j < RADIX_MAX_V; j++) {
        if (j < R.V) {
            const DevCol &c = P.cols[R.vcol[j]];
            tv[j] = (c.type == GB_T_DOUBLE) ? (u64)__double_as_longlong(load_f64(c, r)) : (u64)load_int(c, r);
        }
    }
}

// Per-op contributions of one tuple (value columns are NOT NULL here).
__device__ __forceinline__ void tuple_contrib(const Plan &P, const RadixPlan &R, const u64 *tv, u64 *v) {
#pragma unroll
    for (int i = 0; i < GB_MAX_OPS; i++) {
        if (i < P.n_ops) {
            const u64 x = tv[R.op_v[i]];
            switch (P.ops[i].kind) {
            case OP_MIN_F:
            case OP_MAX_F: v[i] = (u64)enc_f64(__longlong_as_double((i64)x)); break;
            case OP_CNT_NN: v[i] = 1ull; break;
            default: v[i] = x; break;
            }
        }
    }
}

template <int ROWS, int VV>
__global__ void __launch_bounds__(1024, 1) k_partition(const __grid_constant__ Plan P, const __grid_constant__ RadixPlan R,
                                                       const RadixRef X, const TableRef T, const RadixTile A) {
    extern __shared__ u64 rsm[];
    const int HS = R.HS, W = P.words, NP = 1 << R.pbits;
    u64 *hk = rsm;                         // HS hot keys
    u64 *hs = rsm + HS;                    // HS * W hot states
    u32 *s_hist = (u32 *)(hs + (u64)HS * W);
    u32 *s_base = s_hist + NP;
    __shared__ u32 s_tile;
    for (int i = threadIdx.x; i < HS; i += blockDim.x) {
        hk[i] = X.hot_keys ? X.hot_keys[i] : EMPTY_KEY;
        for (int w = 0; w < W; w++) hs[(u64)i * W + w] = P.word_init[w];
    }
    for (int i = threadIdx.x; i < NP; i += blockDim.x) s_hist[i] = 0;
    __syncthreads();
    const int TV = 1 + R.V;
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
        const u32 tile = s_tile;
        __syncthreads();
        if (tile == ~0u) break;
        const u64 t0 = (u64)(A.first_tile + tile) * (u64)(ROWS * blockDim.x);
        const u64 t1 = min(A.n_rows, t0 + (u64)(ROWS * blockDim.x));
        u64 pk[ROWS];
        u64 tv[ROWS][VV];
        u32 pr[ROWS];  // partition << 16 | rank, ~0u = not a tail row
#pragma unroll
        for (int j = 0; j < ROWS; j++) {
            const u64 r = t0 + (u64)j * blockDim.x + threadIdx.x;
            pr[j] = ~0u;
            if (r >= t1) continue;
            if (P.n_filters && !pass_filters(P, r)) continue;
            const int kind = make_key(P, r, pk[j]);
            u64 tvf[RADIX_MAX_V];
            tuple_vals(P, R, r, tvf);
#pragma unroll
            for (int q = 0; q < VV; q++) tv[j][q] = tvf[q];
            u64 v[GB_MAX_OPS];
            tuple_contrib(P, R, tvf, v);
            if (kind != 0) {
                if (kind == 3) atomicOr(&T.ctl->err, (u32)ERR_NULL_IN_WIDE_KEY);
                else special_fold(P, T, kind, 1, v);
                continue;
            }
            const u64 h = mix64(pk[j]);
            bool hot = false;
            if (HS) {
                u32 s = hot_slot(h, HS);
                for (int p = 0; p < R.hot_probe; p++) {
                    const u64 k = hk[s];
                    if (k == pk[j]) {
                        apply_state(P, hs + (u64)s * W, 1, v);
                        hot = true;
                        break;
                    }
                    if (k == EMPTY_KEY) break;
                    s = (s + 1) & (u32)(HS - 1);
                }
            }
            if (!hot) {
                const u32 p = part_of(h, R.pbits);
                const u32 rank = atomicAdd(&s_hist[p], 1u);
                pr[j] = (p << 16) | rank;
            }
        }
        __syncthreads();
        for (int p = threadIdx.x; p < NP; p += blockDim.x) {
            const u32 c = s_hist[p];
            if (c) {
                s_base[p] = atomicAdd(&X.cursor[(u64)p * CURSOR_PAD], c);
                s_hist[p] = 0;
            }
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < ROWS; j++) {
            if (pr[j] == ~0u) continue;
            const u32 p = pr[j] >> 16;
            const u64 pos = (u64)s_base[p] + (pr[j] & 0xffffu);
            if (pos < X.cap_p) {
                u64 *dst = X.part + ((u64)p * X.cap_p + pos) * TV;
                dst[0] = pk[j];
#pragma unroll
                for (int q = 0; q < VV; q++) dst[1 + q] = tv[j][q];
            } else {
                const u32 o = atomicAdd(&T.ctl->aux0, 1u);
                if (o < X.ovf_cap) {
                    u64 *dst = X.ovf + (u64)o * (TV + 1);
                    dst[0] = p;
                    dst[1] = pk[j];
#pragma unroll
                    for (int q = 0; q < VV; q++) dst[2 + q] = tv[j][q];
                } else {
                    atomicOr(&T.ctl->err, (u32)ERR_SPILL_OVERFLOW);
                }
            }
        }
        if (threadIdx.x == 0 && *(volatile u32 *)&T.ctl->aux0 > X.ovf_threshold) atomicExch(&T.ctl->stop, 1u);
    }
    __syncthreads();
    // fold this CTA's hot partial states into its slice (launches of one
    // handle run in stream order, so the read-modify-write is race free)
    if (HS) {
        u64 *hp = X.hot_part + (u64)blockIdx.x * HS * W;
        for (u64 i = threadIdx.x; i < (u64)HS * W; i += blockDim.x) {
            const int w = (int)(i % W);
            const u64 a = hp[i], b = hs[i];
            hp[i] = (w == 0) ? a + b : op_combine(R.word_kind[w], a, b);
        }
    }
}

// Append overflow tuples to their (grown) partitions.
__global__ void k_part_drain(const RadixRef X, int V, u32 n) {
    const int TV = 1 + V;
    for (u64 i = blockIdx.x * (u64)blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
        const u64 *src = X.ovf + i * (TV + 1);
        const u32 p = (u32)src[0];
        const u64 pos = atomicAdd(&X.cursor[(u64)p * CURSOR_PAD], 1u);
        u64 *dst = X.part + ((u64)p * X.cap_p + pos) * TV;
        for (int q = 0; q < TV; q++) dst[q] = src[1 + q];
    }
}

// ------------------------------------------------------------- P2 aggregate
__global__ void __launch_bounds__(1024, 1) k_part_agg(const __grid_constant__ Plan P, const __grid_constant__ RadixPlan R,
                                                      const RadixRef X, const TableRef T,
                                                      const __grid_constant__ EmitArgs E, int SP) {
    extern __shared__ u64 rsm[];
    const int W = P.words, TV = 1 + R.V;
    u64 *keys = rsm;
    u64 *st = rsm + SP;
    __shared__ u32 s_new;
    for (int i = threadIdx.x; i < SP; i += blockDim.x) {
        keys[i] = EMPTY_KEY;
        for (int w = 0; w < W; w++) st[(u64)i * W + w] = P.word_init[w];
    }
    if (threadIdx.x == 0) s_new = 0;
    __syncthreads();
    const u32 p = blockIdx.x;
    const u64 n = min((u64)X.cursor[(u64)p * CURSOR_PAD], X.cap_p);
    const u64 *base = X.part + (u64)p * X.cap_p * TV;
    volatile u64 *vk = keys;
    for (u64 i = threadIdx.x; i < n; i += blockDim.x) {
        const u64 *tp = base + i * TV;
        const u64 pk = tp[0];
        u64 tv[RADIX_MAX_V];
#pragma unroll
        for (int q = 0; q < RADIX_MAX_V; q++)
            if (q < R.V) tv[q] = tp[1 + q];
        u64 v[GB_MAX_OPS];
        tuple_contrib(P, R, tv, v);
        const u64 h = mix64(pk);
        u32 s = agg_slot(h, SP);
        bool done = false;
        for (int q = 0; q < R.agg_probe; q++) {
            u64 k = vk[s];
            if (k == EMPTY_KEY) {
                u64 old = atomicCAS(&keys[s], EMPTY_KEY, pk);
                if (old == EMPTY_KEY || old == pk) k = pk;
                else k = old;
            }
            if (k == pk) {
                apply_state(P, st + (u64)s * W, 1, v);
                done = true;
                break;
            }
            s = (s + 1) & (u32)(SP - 1);
        }
        if (!done) global_fold(P, T, pk, 1, v, &s_new);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (int b = threadIdx.x - lane; b < SP; b += blockDim.x) {
        const int s = b + lane;
        const bool occ = keys[s] != EMPTY_KEY;
        const u64 o = warp_out_slot(T.ctl, occ, FULL);
        if (!occ) continue;
        if (o >= E.out_cap) {
            atomicOr(&T.ctl->err, (u32)ERR_OUT_OVERFLOW);
            continue;
        }
        emit_group(P, E, o, keys[s], false, st + (u64)s * W);
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_new) atomicAdd(&T.ctl->n_groups, s_new);
}

// ------------------------------------------------------------- P3 hot
__global__ void k_hot_emit(const __grid_constant__ Plan P, const __grid_constant__ RadixPlan R, const RadixRef X,
                           int G, Ctl *ctl, const __grid_constant__ EmitArgs E) {
    const int W = P.words, HS = R.HS;
    const int lane = threadIdx.x & 31;
    for (u64 b = blockIdx.x * (u64)blockDim.x + threadIdx.x - lane; b < (u64)HS;
         b += (u64)gridDim.x * blockDim.x) {
        const u64 s = b + lane;
        u64 w[GB_MAX_WORDS];
        bool occ = false;
        const u64 key = s < (u64)HS ? X.hot_keys[s] : EMPTY_KEY;
        if (key != EMPTY_KEY) {
            for (int q = 0; q < W; q++) w[q] = P.word_init[q];
            for (int g = 0; g < G; g++) {
                const u64 *hp = X.hot_part + ((u64)g * HS + s) * W;
                w[0] += hp[0];
                for (int q = 1; q < W; q++) w[q] = op_combine(R.word_kind[q], w[q], hp[q]);
            }
            occ = w[0] != 0;
        }
        const u64 o = warp_out_slot(ctl, occ, FULL);
        if (!occ) continue;
        if (o >= E.out_cap) {
            atomicOr(&ctl->err, (u32)ERR_OUT_OVERFLOW);
            continue;
        }
        emit_group(P, E, o, key, false, w);
    }
}

__global__ void k_fill_words(u64 *dst, u64 n, int W, const __grid_constant__ Plan P) {
    for (u64 i = blockIdx.x * (u64)blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x)
        dst[i] = P.word_init[i % W];
}

// ================================================================== host
static u64 pow2_at_least(u64 x) {
    u64 p = 1;
    while (p < x) p <<= 1;
    return p;
}

static int grid_of(u64 work, int block, int cap) {
    u64 g = (work + block - 1) / block;
    return (int)std::max<u64>(1, std::min<u64>(g, (u64)cap));
}

gb_status radix_prepare(const Plan &P, RadixPlan &R, u64 est_groups, u64 nullable_mask) {
    memset(&R, 0, sizeof R);
    if (P.key_mode == KEY_STRING) return GB_ERR_UNSUPPORTED;
    // tuple values: distinct NOT NULL op columns
    for (int i = 0; i < P.n_ops; i++) {
        const int c = P.ops[i].col;
        if ((nullable_mask >> c) & 1ull) return GB_ERR_UNSUPPORTED;
        int j = 0;
        while (j < R.V && R.vcol[j] != c) j++;
        if (j == R.V) {
            if (R.V >= RADIX_MAX_V) return GB_ERR_UNSUPPORTED;
            R.vcol[R.V++] = c;
        }
        R.op_v[i] = j;
        R.word_kind[P.ops[i].word] = P.ops[i].kind;
    }
    if (P.words > GB_MAX_WORDS) return GB_ERR_UNSUPPORTED;
    // partitions: ~3K groups each so a partition fits a shared table at
    // load <= 0.5
    u64 want = (est_groups + 3071) / 3072;
    u64 np = pow2_at_least(std::max<u64>(want, 64));
    np = std::min<u64>(np, 4096);
    int pb = 0;
    while ((1ull << pb) < np) pb++;
    R.pbits = pb;
    // hot table: as many slots as fit next to the partition counters
    const size_t budget = 200 * 1024 - 2 * np * 4;
    u64 hs = 1;
    while ((hs * 2) * 8 * (1 + (u64)P.words) <= budget) hs *= 2;
    R.HS = (int)std::min<u64>(hs, 8192);
    R.hot_probe = 8;
    R.agg_probe = 64;
    return GB_OK;
}

u32 radix_tile_rows(const RadixPlan &R) { return (u32)((R.V == 3 ? RADIX_ROWS / 2 : RADIX_ROWS) * RADIX_BLOCK); }

size_t radix_p1_smem(const Plan &P, const RadixPlan &R) {
    return (size_t)R.HS * 8 * (1 + P.words) + (size_t)2 * (1u << R.pbits) * 4;
}

int radix_sp(const Plan &P) {
    u64 sp = 1;
    while ((sp * 2) * 8 * (1 + (u64)P.words) <= 200 * 1024) sp *= 2;
    return (int)std::min<u64>(sp, 8192);
}

gb_status radix_launch_sample(const Plan &P, const RadixPlan &R, u64 n, u64 *skeys, u32 *scnt, u64 scap,
                              u32 *hist, u64 *hot_keys, cudaStream_t st, u64 *launches) {
    const u64 m = std::min<u64>(n, scap / 2);
    const u64 step = std::max<u64>(1, n / std::max<u64>(m, 1));
    const int sms = sm_count();
    k_sample_count<<<grid_of(m, 256, sms * 4), 256, 0, st>>>(P, n, step, m, skeys, scnt, scap);
    k_sample_hist<<<grid_of(scap, 256, sms * 2), 256, 0, st>>>(skeys, scnt, scap, hist);
    k_hot_build<<<grid_of(scap, 256, sms * 2), 256, 0, st>>>(skeys, scnt, scap, hist, 2, (u32)(R.HS / 2), hot_keys,
                                                            R.HS);
    *launches += 3;
    GB_CUDA(cudaGetLastError());
    return GB_OK;
}

gb_status radix_launch_p1(const Plan &P, const RadixPlan &R, const RadixRef &X, const TableRef &T,
                          const RadixTile &A, int grid, cudaStream_t st) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_partition<RADIX_ROWS, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
        cudaFuncSetAttribute(k_partition<RADIX_ROWS, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
        cudaFuncSetAttribute(k_partition<RADIX_ROWS / 2, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             220 * 1024);
        cudaFuncSetAttribute(k_part_agg, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
        attr = true;
    }
    const size_t smem = radix_p1_smem(P, R);
    if (R.V == 1) k_partition<RADIX_ROWS, 1><<<grid, RADIX_BLOCK, smem, st>>>(P, R, X, T, A);
    else if (R.V == 2) k_partition<RADIX_ROWS, 2><<<grid, RADIX_BLOCK, smem, st>>>(P, R, X, T, A);
    else k_partition<RADIX_ROWS / 2, 3><<<grid, RADIX_BLOCK, smem, st>>>(P, R, X, T, A);
    GB_CUDA(cudaGetLastError());
    return GB_OK;
}

gb_status radix_launch_drain(const RadixRef &X, int V, u32 n, cudaStream_t st) {
    k_part_drain<<<grid_of(n, 256, sm_count() * 4), 256, 0, st>>>(X, V, n);
    GB_CUDA(cudaGetLastError());
    return GB_OK;
}

gb_status radix_launch_p2(const Plan &P, const RadixPlan &R, const RadixRef &X, const TableRef &T, const EmitArgs &E,
                          cudaStream_t st) {
    const int SP = radix_sp(P);
    const size_t smem = (size_t)SP * 8 * (1 + P.words);
    k_part_agg<<<1 << R.pbits, RADIX_BLOCK, smem, st>>>(P, R, X, T, E, SP);
    GB_CUDA(cudaGetLastError());
    return GB_OK;
}

gb_status radix_launch_p3(const Plan &P, const RadixPlan &R, const RadixRef &X, int G, Ctl *ctl, const EmitArgs &E,
                          cudaStream_t st) {
    if (R.HS == 0) return GB_OK;
    k_hot_emit<<<grid_of(R.HS, 256, sm_count() * 2), 256, 0, st>>>(P, R, X, G, ctl, E);
    GB_CUDA(cudaGetLastError());
    return GB_OK;
}

gb_status radix_fill_identity(u64 *dst, u64 n, int W, const Plan &P, cudaStream_t st) {
    k_fill_words<<<grid_of(n, 256, sm_count() * 8), 256, 0, st>>>(dst, n, W, P);
    GB_CUDA(cudaGetLastError());
    return GB_OK;
}

}  // namespace gb
