// gb_radix.cu — the radix-partitioned GROUP BY for high-cardinality keys.
//
// GB300 restatement of the reference's radix aggregators
// (src/execution/radix_count_agg.cpp:17-106 RadixCountAgg: scatter rows by
// top hash bits, aggregate each radix partition in its own open-addressing
// map, src/execution/simple_i64_count_map.hpp:20-109) generalised to every
// aggregate of the plan, with a heavy-hitter stage in front:
//
//   S  sample:  a strided sample of the keys is counted; the NH most frequent
//               keys become "hot" (dense hot index), the NSUP most frequent of
//               them "super-hot".
//   P1 scatter: persistent CTAs (32 warps, 4 rows per thread per tile) stream
//               the rows.  A row of one of the REG_HOT hottest keys is folded
//               into per-lane registers; a super-hot row into its warp's
//               private shared state; another hot row into the CTA's shared
//               state (shared atomics); any other row is appended as a (key,
//               values) tuple to partition p = top hash bits through a
//               per-CTA write-combining buffer of wcb tuples per partition,
//               flushed in aligned groups (one global atomic per flush).
//               The specialised instance (one non-NULL BIGINT key, one SUM,
//               no predicates) keeps only the hot counts in registers and
//               shared memory; every hot row's sum is a fire-and-forget L2
//               reduction into the CTA's hot slice.
//               Partition regions have per-partition capacities; a region
//               that overflows is grown (and its tuples moved) by the host,
//               and a re-execution keeps the grown capacities.
//   P2 agg:     one CTA per partition: a shared open-addressing table (keys,
//               32-bit counts) with either the state words beside it and a
//               warp pre-combine of equal keys (32-bit hash match checked on
//               the full key), or, when every op is a DOUBLE SUM, the words
//               in the partition's L2 slice folded tuple by tuple as L2
//               reductions; a table that overflows folds the rest into the
//               HBM hash table.
//   P3 hot:     per-CTA hot partials are reduced in a fixed order and
//               emitted.  (DOUBLE sums are exact to rounding but, as with any
//               atomic accumulation, their last bits depend on the order the
//               rows arrive in.)
//
// A key is hot for the whole query or never, and lives in exactly one
// partition, so every group is emitted exactly once.  Bounded probes fall
// back to the HBM hash table (emitted by the compaction kernel), which keeps
// the result exact for any key distribution.
#include <algorithm>
#include <cstring>
#include <vector>

#include "gb_kernels.cuh"
#include "gb_radix.h"

namespace gb {

// P1 hash of a group key: the high half folded into the low half, then one
// multiplicative (Fibonacci) step.  Its top bits pick the partition, bits
// 32.. the hot bucket.  (P2 hashes the keys of a partition with mix64.)
__device__ __forceinline__ u64 p1_hash(u64 k) { return (k ^ (k >> 32)) * 0x9E3779B97F4A7C15ull; }
__device__ __forceinline__ u32 part_of(u64 h, int pbits) { return pbits ? (u32)(h >> (64 - pbits)) : 0u; }
__device__ __forceinline__ u32 hot_bucket(u64 h, int HB) { return (u32)(h >> 32) & (u32)(HB - 1); }
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
    __shared__ u32 h[HIST_BINS];
    for (int i = threadIdx.x; i < HIST_BINS; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (u64 s = blockIdx.x * (u64)blockDim.x + threadIdx.x; s < scap; s += (u64)gridDim.x * blockDim.x)
        if (skeys[s] != EMPTY_KEY) atomicAdd(&h[min(scnt[s], (u32)(HIST_BINS - 1))], 1u);
    __syncthreads();
    for (int i = threadIdx.x; i < HIST_BINS; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[i], h[i]);
}

// The smallest t >= floor_t admitting at most `cap` keys with sample count
// >= t (HIST_BINS = none), computed by a whole block: the histogram is
// loaded into shared memory and suffix-summed by one warp's scan (one thread
// walking 1024 bins in global memory took tens of microseconds).  `hs` holds
// HIST_BINS u32; every thread gets the result.
__device__ u32 block_count_threshold(const u32 *hist, u32 cap, u32 floor_t, u32 *hs) {
    __shared__ u32 s_t;
    const int lane = threadIdx.x & 31;
    for (int c = threadIdx.x; c < HIST_BINS; c += blockDim.x) hs[c] = hist[c];
    if (threadIdx.x == 0) s_t = HIST_BINS;
    __syncthreads();
    if (threadIdx.x < 32) {
        // lane L sums the chunk [c1 - per, c1) of bins, chunks from the top
        const int per = HIST_BINS / 32;
        const int c1 = HIST_BINS - lane * per;
        u32 sum = 0;
        for (int c = c1 - 1; c >= c1 - per; c--) sum += hs[c];
        u32 incl = sum;
        for (int o = 1; o < 32; o <<= 1) {
            const u32 y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        u32 run = incl - sum;  // keys with count >= c1
        for (int c = c1 - 1; c >= c1 - per; c--) {
            run += hs[c];
            hs[c] = run;  // keys with count >= c
        }
    }
    __syncthreads();
    // hs is non-increasing: t = max(floor_t, the first c with hs[c] <= cap)
    for (int c = threadIdx.x; c < HIST_BINS; c += blockDim.x)
        if (c >= (int)floor_t && hs[c] <= cap && (c == (int)floor_t || hs[c - 1] > cap)) atomicMin(&s_t, (u32)c);
    __syncthreads();
    return s_t;
}

// Hot-set candidates: every sampled key whose count reaches the threshold
// that admits at most NH keys (hstate[3] = candidates found).
__global__ void k_hot_collect(const u64 *skeys, const u32 *scnt, u64 scap, const u32 *hist, u32 *hstate, int NH,
                              u64 *cand_key, u32 *cand_cnt) {
    __shared__ u32 hs[HIST_BINS];
    const u32 t = block_count_threshold(hist, (u32)NH, 2, hs);
    if (t >= HIST_BINS) return;
    for (u64 s = blockIdx.x * (u64)blockDim.x + threadIdx.x; s < scap; s += (u64)gridDim.x * blockDim.x) {
        const u64 k = skeys[s];
        if (k == EMPTY_KEY) continue;
        const u32 c = min(scnt[s], (u32)(HIST_BINS - 1));
        if (c < t) continue;
        const u32 i = atomicAdd(&hstate[3], 1u);
        if (i < (u32)NH) {
            cand_key[i] = k;
            cand_cnt[i] = scnt[s];
        }
    }
}

// Rank the candidates (sampled count descending, equal counts by candidate
// slot: rank 0 is the hottest key) and place them into the 2-way bucket
// table: each bucket b = hot_bucket(key) takes its two best-ranked keys
// (slots 2b, 2b + 1), so the hottest keys always get a slot and a lookup is
// one 16-byte shared load.  A key whose bucket holds two better-ranked keys
// is not hot (its rows take the partitioned path).  hot_list[rank] = key for
// every candidate; hstate[0] = candidates among the NSUP hottest, hstate[1]
// = the others, hstate[2] = sampled rows of the placed keys.  One block of
// 1024 threads, HOT_RANK_SMEM bytes of dynamic shared memory; NH <= 4096,
// HB <= 4096.
#define HOT_RANK_SMEM (4096 * 8 + 4096 * 4 * 2)
__global__ void __launch_bounds__(1024) k_hot_rank(const u64 *cand_key, const u32 *cand_cnt, u32 *hstate, int NSUP,
                                                   int NH, int HB, u64 *hot_keys, uint16_t *hot_rank,
                                                   u64 *hot_list) {
    extern __shared__ u64 hrsm[];
    u64 *sv = hrsm;                // [4096] sort values: (~count << 32) | candidate slot
    u32 *b1 = (u32 *)(sv + 4096);  // [4096] best rank of each bucket
    u32 *b2 = b1 + 4096;           // [4096] second-best rank
    __shared__ u32 s_rows;
    const u32 n = min(hstate[3], (u32)min(NH, 4096));
    u32 n2 = 1;
    while (n2 < n) n2 <<= 1;
    for (u32 i = threadIdx.x; i < n2; i += blockDim.x) sv[i] = i < n ? ((u64)(~cand_cnt[i]) << 32) | i : ~0ull;
    for (int i = threadIdx.x; i < HB; i += blockDim.x) {
        b1[i] = ~0u;
        b2[i] = ~0u;
    }
    if (threadIdx.x == 0) s_rows = 0;
    __syncthreads();
    // bitonic sort, ascending: larger count first, then the lower candidate slot
    for (u32 size = 2; size <= n2; size <<= 1) {
        for (u32 stride = size >> 1; stride > 0; stride >>= 1) {
            for (u32 i = threadIdx.x; i < n2 / 2; i += blockDim.x) {
                const u32 lo = 2 * i - (i & (stride - 1));
                const u32 hi = lo + stride;
                const u64 a = sv[lo], b = sv[hi];
                if ((b < a) == ((lo & size) == 0)) {
                    sv[lo] = b;
                    sv[hi] = a;
                }
            }
            __syncthreads();
        }
    }
    // each bucket keeps its two best ranks
    for (u32 r = threadIdx.x; r < n; r += blockDim.x) {
        const u64 k = cand_key[(u32)sv[r]];
        hot_list[r] = k;
        atomicMin(&b1[hot_bucket(p1_hash(k), HB)], r);
    }
    __syncthreads();
    for (u32 r = threadIdx.x; r < n; r += blockDim.x) {
        const u32 b = hot_bucket(p1_hash(hot_list[r]), HB);
        if (b1[b] != r) atomicMin(&b2[b], r);
    }
    __syncthreads();
    for (u32 r = threadIdx.x; r < n; r += blockDim.x) {
        const u32 ci = (u32)sv[r];
        const u64 k = cand_key[ci];
        const u32 b = hot_bucket(p1_hash(k), HB);
        const int way = b1[b] == r ? 0 : (b2[b] == r ? 1 : -1);
        if (way >= 0) {
            hot_keys[2 * b + way] = k;
            hot_rank[2 * b + way] = (uint16_t)r;
            atomicAdd(&s_rows, cand_cnt[ci]);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        hstate[0] = min(n, (u32)NSUP);
        hstate[1] = n - min(n, (u32)NSUP);
        hstate[2] = s_rows;
    }
}

// ------------------------------------------------------------- helpers
template <int VV>
__device__ __forceinline__ void tuple_vals(const Plan &P, const RadixPlan &R, u64 r, u64 *tv) {
#pragma unroll
    for (int j = 0; j < VV; j++) {
        const DevCol &c = P.cols[R.vcol[j]];
        tv[j] = (c.type == GB_T_DOUBLE) ? (u64)__double_as_longlong(load_f64(c, r)) : (u64)load_int(c, r);
    }
}

template <int VV>
__device__ __forceinline__ u64 tv_pick(const u64 *tv, int j) {
    if (VV == 1) return tv[0];
    if (VV == 2) return j == 0 ? tv[0] : tv[1];
    return j == 0 ? tv[0] : (j == 1 ? tv[1] : tv[2]);
}

// Per-op contributions of one tuple (value columns are NOT NULL here).
template <int VV, int NOPS>
__device__ __forceinline__ void tuple_contrib(const Plan &P, const RadixPlan &R, const u64 *tv, u64 *v) {
#pragma unroll
    for (int i = 0; i < NOPS; i++) {
        const u64 x = tv_pick<VV>(tv, R.op_v[i]);
        switch (P.ops[i].kind) {
        case OP_MIN_F:
        case OP_MAX_F: v[i] = (u64)enc_f64(__longlong_as_double((i64)x)); break;
        case OP_CNT_NN: v[i] = 1ull; break;
        default: v[i] = x; break;
        }
    }
}

// Plain (non-atomic) fold of a combined partial into state words owned by
// the calling lane.
template <int NOPS>
__device__ __forceinline__ void fold_plain(const Plan &P, u64 *w, u64 cnt, const u64 *v) {
    w[0] += cnt;
#pragma unroll
    for (int i = 0; i < NOPS; i++) w[P.ops[i].word] = op_combine(P.ops[i].kind, w[P.ops[i].word], v[i]);
}

template <int NOPS>
__device__ __forceinline__ void fold_atomic(const Plan &P, u64 *w, u64 cnt, const u64 *v) {
    atomicAdd(w, cnt);
#pragma unroll
    for (int i = 0; i < NOPS; i++) op_apply(P.ops[i].kind, w + P.ops[i].word, v[i], P.word_init[P.ops[i].word]);
}

template <int NOPS>
__device__ __forceinline__ void global_fold_n(const Plan &P, const TableRef &T, u64 pk, u64 cnt, const u64 *v,
                                              u32 *new_groups) {
    u64 vv[GB_MAX_OPS];
#pragma unroll
    for (int i = 0; i < GB_MAX_OPS; i++) vv[i] = i < NOPS ? v[i < NOPS ? i : 0] : 0;
    global_fold(P, T, pk, cnt, vv, new_groups);
}

// Warp segmented combine: lanes with equal `id` (among `act` lanes) fold
// their partials into the lowest such lane (the leader).  Returns the leader
// flag; cnt = group size.
template <int NOPS>
__device__ __forceinline__ bool warp_combine(const Plan &P, bool act, u64 id, u64 *v, u64 &cnt) {
    const int lane = threadIdx.x & 31;
    const unsigned am = __ballot_sync(FULL, act);
    const unsigned peers = __match_any_sync(FULL, id) & am;
    const bool leader = act && ((__ffs(peers) - 1) == lane);
    unsigned rem = leader ? (peers & ~(1u << lane)) : 0u;
    const int maxit = __reduce_max_sync(FULL, (unsigned)__popc(rem));
    for (int it = 0; it < maxit; it++) {
        const int src = rem ? (__ffs(rem) - 1) : lane;
        rem &= rem - 1u;
#pragma unroll
        for (int q = 0; q < NOPS; q++) {
            const u64 o = __shfl_sync(FULL, v[q], src);
            if (src != lane) v[q] = op_combine(P.ops[q].kind, v[q], o);
        }
    }
    cnt = __popc(peers);
    return leader;
}

template <int VV>
__device__ __forceinline__ void put_tuple(u64 *dst, u64 pk, const u64 *tv) {
    dst[0] = pk;
#pragma unroll
    for (int q = 0; q < VV; q++) dst[1 + q] = tv[q];
}

template <int VV>
__device__ __forceinline__ void put_overflow(const RadixRef &X, const TableRef &T, u32 p, u64 pk, const u64 *tv) {
    const u32 o = atomicAdd(&T.ctl->aux0, 1u);
    if (o < X.ovf_cap) {
        u64 *od = X.ovf + (u64)o * (VV + 2);
        od[0] = p;
        put_tuple<VV>(od + 1, pk, tv);
    } else {
        atomicOr(&T.ctl->err, (u32)ERR_SPILL_OVERFLOW);
    }
}

// Write one tuple at region position `pos` of partition p (or overflow).
template <int VV>
__device__ __forceinline__ void store_at(const RadixRef &X, const TableRef &T, u32 p, u32 pos, u64 pk, const u64 *tv) {
    if (pos < __ldg(&X.part_cap[p])) put_tuple<VV>(X.part + ((u64)__ldg(&X.part_off[p]) + pos) * (1 + VV), pk, tv);
    else put_overflow<VV>(X, T, p, pk, tv);
}

// ------------------------------------------------------------- P1 scatter
// Generic plans.  Block: P1_WARPS warps, ROWS rows per thread per tile.  The
// REG_HOT hottest keys accumulate in per-lane registers; the next NPRIV -
// REG_HOT have a private state per warp (u32 count + W-1 words; only this
// warp's lanes contend on its atomics); the other hot keys share one state
// per CTA.  Cold tuples go through per-CTA write-combining buffers.
template <int ROWS, int VV, int NOPS>
__global__ void __launch_bounds__(P1_WARPS * 32, 1)
    k_partition(const __grid_constant__ Plan P, const __grid_constant__ RadixPlan R, const RadixRef X,
                const TableRef T, const RadixTile A) {
    extern __shared__ u64 rsm[];
    constexpr int TV = 1 + VV;
    constexpr int NT = P1_WARPS * 32;
    const int HS = R.HS, W = P.words, NP = 1 << R.pbits, NH = R.nh, NPRIV = R.nsup, NWARM = R.nh - R.nsup;
    const int B = R.wcb;
    const int WM = W - 1;  // state words besides the count
    const int warp = threadIdx.x >> 5;
    u64 *hk = rsm;                                        // [HS] hot keys
    u64 *pw = hk + HS;                                    // [P1_WARPS][NPRIV][WM] private words
    u64 *sw = pw + (size_t)P1_WARPS * NPRIV * WM;         // [NWARM][WM] shared words
    u64 *wbuf = sw + (size_t)NWARM * WM;                  // [NP][B][TV] write-combining buffers
    u32 *pc = (u32 *)(wbuf + (size_t)NP * B * TV);        // [P1_WARPS][NPRIV] private counts
    u32 *sc = pc + P1_WARPS * NPRIV;                      // [NWARM] shared counts
    u32 *bcnt = sc + NWARM;                               // [NP] buffered tuples
    u32 *sbase = bcnt + NP;                               // [NP] flush base this tile
    u32 *snf = sbase + NP;                                // [NP] tuples flushed this tile
    uint16_t *hix = (uint16_t *)(snf + NP);               // [HS] hot rank of each bucket slot
    const int HB = HS >> 1;
    __shared__ u32 s_tile;
    for (int i = threadIdx.x; i < HS; i += NT) {
        hk[i] = X.hot_keys[i];
        hix[i] = X.hot_idx[i];
    }
    for (int i = threadIdx.x; i < P1_WARPS * NPRIV; i += NT) {
        pc[i] = 0;
        for (int w = 0; w < WM; w++) pw[(size_t)i * WM + w] = P.word_init[1 + w];
    }
    for (int i = threadIdx.x; i < NWARM; i += NT) {
        sc[i] = 0;
        for (int w = 0; w < WM; w++) sw[(size_t)i * WM + w] = P.word_init[1 + w];
    }
    for (int i = threadIdx.x; i < NP; i += NT) bcnt[i] = 0;
    __syncthreads();
    u32 *mypc = pc + warp * NPRIV;
    u64 *mypw = pw + (size_t)warp * NPRIV * WM;
    u64 *hpart = X.hot_part + (u64)blockIdx.x * NH * W;  // this CTA's hot slice (identity-initialised)
    // the REG_HOT hottest keys accumulate in this lane's registers: no
    // conflicts, no warp collectives
    constexpr int NV = NOPS > 0 ? NOPS : 1;
    u32 rc[REG_HOT];
    u64 rw[REG_HOT][NV];
#pragma unroll
    for (int k = 0; k < REG_HOT; k++) {
        rc[k] = 0;
#pragma unroll
        for (int i = 0; i < NV; i++) rw[k][i] = i < NOPS ? P.word_init[P.ops[i < NOPS ? i : 0].word] : 0;
    }
    // the next tile is claimed one tile ahead so the claim's latency overlaps work
    if (threadIdx.x == 0) {
        u32 c = atomicAdd(&T.ctl->tile_counter, 1u);
        s_tile = c < A.n_tiles ? c : ~0u;
    }
    __syncthreads();
    u32 tile = s_tile;
    __syncthreads();
    while (tile != ~0u) {
        if (threadIdx.x == 0) {
            u32 t = ~0u;
            if (*(volatile u32 *)&T.ctl->stop == 0) {
                u32 c = atomicAdd(&T.ctl->tile_counter, 1u);
                if (c < A.n_tiles) t = c;
            }
            s_tile = t;
        }
        const u64 t0 = (u64)(A.first_tile + tile) * (u64)(ROWS * NT);
        const u64 t1 = min(A.n_rows, t0 + (u64)(ROWS * NT));
        u64 pk[ROWS];
        u64 tv[ROWS][VV];
        u32 pend[ROWS];  // partition + 1 of a tuple that did not fit the buffer
        u32 pslot[ROWS];
        int kinds[ROWS];
        bool acts[ROWS];
        // issue every load of the tile before any dependent work
#pragma unroll
        for (int j = 0; j < ROWS; j++) {
            const u64 r = t0 + (u64)j * NT + threadIdx.x;
            acts[j] = r < t1;
            kinds[j] = 0;
            pk[j] = 0;
            if (acts[j]) {
                kinds[j] = make_key(P, r, pk[j]);
                tuple_vals<VV>(P, R, r, tv[j]);
            }
        }
#pragma unroll
        for (int j = 0; j < ROWS; j++) {
            const u64 r = t0 + (u64)j * NT + threadIdx.x;
            pend[j] = 0;
            pslot[j] = 0;
            bool act = acts[j];
            if (act && P.n_filters) act = pass_filters(P, r);
            u32 hidx = 0;
            u64 v[NOPS > 0 ? NOPS : 1];
#pragma unroll
            for (int q = 0; q < (NOPS > 0 ? NOPS : 1); q++) v[q] = 0;
            if (act) {
                const int kind = kinds[j];
                tuple_contrib<VV, NOPS>(P, R, tv[j], v);
                if (kind != 0) {
                    if (kind == 3) {
                        atomicOr(&T.ctl->err, (u32)ERR_NULL_IN_WIDE_KEY);
                    } else {
                        u64 *w = T.slots + (T.cap + (u64)(kind - 1)) * (u64)T.stride + 1;
                        fold_atomic<NOPS>(P, w, 1, v);
                    }
                } else {
                    const u64 h = p1_hash(pk[j]);
                    bool hot = false;
                    if (HS) {
                        // the key's 2-way bucket: one 16-byte shared load
                        const u32 b = hot_bucket(h, HB);
                        const ulonglong2 kk = *(const ulonglong2 *)(hk + 2 * b);
                        if (kk.x == pk[j]) {
                            hidx = hix[2 * b];
                            hot = true;
                        } else if (kk.y == pk[j]) {
                            hidx = hix[2 * b + 1];
                            hot = true;
                        }
                    }
                    if (hot) {
                        if (hidx < (u32)REG_HOT) {
#pragma unroll
                            for (int k = 0; k < REG_HOT; k++) {
                                if (hidx == (u32)k) {
                                    rc[k]++;
#pragma unroll
                                    for (int i = 0; i < NOPS; i++)
                                        rw[k][i] = op_combine(P.ops[i].kind, rw[k][i], v[i]);
                                }
                            }
                        } else if ((int)hidx < NPRIV) {
                            // warp-private state: only lanes of this warp contend
                            atomicAdd(&mypc[hidx], 1u);
#pragma unroll
                            for (int i = 0; i < NOPS; i++)
                                op_apply(P.ops[i].kind, mypw + (size_t)hidx * WM + (P.ops[i].word - 1), v[i],
                                         P.word_init[P.ops[i].word]);
                        } else {
                            const u32 wi = hidx - NPRIV;
                            atomicAdd(&sc[wi], 1u);
#pragma unroll
                            for (int i = 0; i < NOPS; i++)
                                op_apply(P.ops[i].kind, sw + (size_t)wi * WM + (P.ops[i].word - 1), v[i],
                                         P.word_init[P.ops[i].word]);
                        }
                    } else {
                        const u32 p = part_of(h, R.pbits);
                        const u32 slot = atomicAdd(&bcnt[p], 1u);
                        if (slot < (u32)B) {
                            put_tuple<VV>(wbuf + ((size_t)p * B + slot) * TV, pk[j], tv[j]);
                        } else {
                            pend[j] = p + 1;
                            pslot[j] = slot;
                        }
                    }
                }
            }
        }
        __syncthreads();
        // flush full buffers: whole multiples of B tuples, aligned
        for (int p = threadIdx.x; p < NP; p += NT) {
            const u32 c = bcnt[p];
            if (c >= (u32)B) {
                const u32 nf = (c / (u32)B) * (u32)B;
                const u32 base = atomicAdd(&X.cursor[(u64)p * CURSOR_PAD], nf);
                sbase[p] = base;
                snf[p] = nf;
                bcnt[p] = c - nf;
                const u64 *src = wbuf + (size_t)p * B * TV;
                if (base + (u32)B <= __ldg(&X.part_cap[p])) {
                    u64 *dst = X.part + ((u64)__ldg(&X.part_off[p]) + base) * TV;
                    for (int q = 0; q < B * TV; q += 2)
                        *(ulonglong2 *)(dst + q) = *(const ulonglong2 *)(src + q);
                } else {
                    for (int q = 0; q < B; q++) store_at<VV>(X, T, p, base + q, src[q * TV], src + q * TV + 1);
                }
            }
        }
        __syncthreads();
        // tuples beyond the buffer: inside the flushed range they go straight
        // to HBM, the rest become the buffer's new head
#pragma unroll
        for (int j = 0; j < ROWS; j++) {
            if (!pend[j]) continue;
            const u32 p = pend[j] - 1;
            const u32 slot = pslot[j];
            if (slot < snf[p]) store_at<VV>(X, T, p, sbase[p] + slot, pk[j], tv[j]);
            else put_tuple<VV>(wbuf + ((size_t)p * B + (slot - snf[p])) * TV, pk[j], tv[j]);
        }
        if (threadIdx.x == 0 && *(volatile u32 *)&T.ctl->aux0 > X.ovf_threshold) atomicExch(&T.ctl->stop, 1u);
        __syncthreads();
        tile = s_tile;
        __syncthreads();
    }
    // final partial buffers: padded to B with holes (EMPTY_KEY) so every
    // flush stays aligned; P2 skips the holes
    for (int p = threadIdx.x; p < NP; p += NT) {
        const u32 c = bcnt[p];
        if (c == 0) continue;
        const u32 base = atomicAdd(&X.cursor[(u64)p * CURSOR_PAD], (u32)B);
        u64 *src = wbuf + (size_t)p * B * TV;
        for (u32 q = c; q < (u32)B; q++) src[q * TV] = EMPTY_KEY;
        for (int q = 0; q < B; q++) {
            const u32 pos = base + q;
            if (pos < __ldg(&X.part_cap[p]))
                put_tuple<VV>(X.part + ((u64)__ldg(&X.part_off[p]) + pos) * TV, src[q * TV], src + q * TV + 1);
            else if (q < (int)c)
                put_overflow<VV>(X, T, p, src[q * TV], src + q * TV + 1);
        }
    }
    // this lane's register accumulators join its warp's private states
#pragma unroll
    for (int k = 0; k < REG_HOT; k++) {
        if (k < NPRIV && rc[k]) {
            atomicAdd(&mypc[k], rc[k]);
#pragma unroll
            for (int i = 0; i < NOPS; i++)
                op_apply(P.ops[i].kind, mypw + (size_t)k * WM + (P.ops[i].word - 1), rw[k][i],
                         P.word_init[P.ops[i].word]);
        }
    }
    __syncthreads();
    // fold private and shared hot states into this CTA's slice
    u64 *hp = hpart;
    for (int i = threadIdx.x; i < NH; i += NT) {
        u64 acc[GB_MAX_WORDS];
        for (int w = 0; w < W; w++) acc[w] = hp[(size_t)i * W + w];
        if (i < NPRIV) {
            for (int wp = 0; wp < P1_WARPS; wp++) {
                acc[0] += pc[wp * NPRIV + i];
                const u64 *s = pw + ((size_t)wp * NPRIV + i) * WM;
                for (int w = 1; w < W; w++) acc[w] = op_combine(R.word_kind[w], acc[w], s[w - 1]);
            }
        } else {
            acc[0] += sc[i - NPRIV];
            const u64 *s = sw + (size_t)(i - NPRIV) * WM;
            for (int w = 1; w < W; w++) acc[w] = op_combine(R.word_kind[w], acc[w], s[w - 1]);
        }
        for (int w = 0; w < W; w++) hp[(size_t)i * W + w] = acc[w];
    }
}

// ------------------------------------------------------------- P1, one key + one SUM
// The specialised P1 for the plan "one non-NULL BIGINT key, one non-NULL
// value column, one SUM (DOUBLE: OPK = OP_ADD_F, BIGINT: OP_ADD_I), at most
// one numeric predicate on the value column (FILT)".  A row that fails the
// predicate is dropped before its hot-table probe.  Nothing in its row loop waits on other warps: each warp
// claims P1D_CLAIM steps of P1D_RUN rows at a time and streams them with
// 128-bit loads (4 rows per lane).  A hot row (its key in the 2-way bucket
// table) counts in registers (the REG_HOT hottest keys) or in a shared u32
// counter, and adds its value to this CTA's hot slice with one
// fire-and-forget L2 reduction (no FP64 arithmetic on the SM).  A cold row
// reserves its slot with one atomic on its partition's cursor and writes its
// 16-byte tuple straight to the partition region: the regions' write
// frontiers stay in L2, so every 32-byte sector is complete before it is
// written back.  A tuple beyond its region's capacity goes to the overflow
// list (the host grows the region and re-runs the rest).
#define P1D_RUN 128   // rows per warp step: lane l owns rows 64j + 2l, 64j + 2l + 1 (j = 0, 1)
#define P1D_CLAIM 8   // steps per claim (1024 rows)

size_t radix_p1d_smem(const RadixPlan &R) {
    const size_t HB = (size_t)R.HS / 2, NP = (size_t)1 << R.pbits;
    return HB * 16 + NP * 8 + HB * 4 + NP * 4 + (size_t)R.nh * 4;
}

template <int OPK, bool FILT>
__global__ void __launch_bounds__(P1_WARPS * 32, 1)
    k_partition_direct(const __grid_constant__ Plan P, const __grid_constant__ RadixPlan R, const RadixRef X,
                       const TableRef T, const RadixTile A) {
    extern __shared__ u64 rsm[];
    const int HB = R.HS >> 1, NH = R.nh, NP = 1 << R.pbits, W = P.words;
    const int lane = threadIdx.x & 31;
    ulonglong2 *hb = (ulonglong2 *)rsm;  // [HB] bucket keys (way 0, way 1)
    u64 *pbase = (u64 *)(hb + HB);       // [NP] first tuple of each partition region
    u32 *hr = (u32 *)(pbase + NP);       // [HB] bucket ranks: way 0 in the low half, way 1 in the high half
    u32 *pcap = hr + HB;                 // [NP] tuples each region holds
    u32 *sc = pcap + NP;                 // [NH] hot counts (ranks >= REG_HOT)
    for (int i = threadIdx.x; i < HB; i += blockDim.x) {
        hb[i] = ((const ulonglong2 *)X.hot_keys)[i];
        hr[i] = ((const u32 *)X.hot_idx)[i];
    }
    for (int p = threadIdx.x; p < NP; p += blockDim.x) {
        pbase[p] = X.part_off[p];
        pcap[p] = X.part_cap[p];
    }
    for (int i = threadIdx.x; i < NH; i += blockDim.x) sc[i] = 0;
    __syncthreads();
    const u64 *kcol = (const u64 *)P.cols[P.key_col[0]].data;
    const u64 *vcol = (const u64 *)P.cols[R.vcol[0]].data;
    const bool vec = ((((u64)kcol) | ((u64)vcol)) & 15) == 0;
    u64 *hsum = X.hot_part + (u64)blockIdx.x * NH * W + P.ops[0].word;  // this CTA's hot slice, SUM word
    u64 *oob = T.slots + T.cap * (u64)T.stride + 1;  // state words of the key equal to EMPTY_KEY
    const u64 n = A.n_rows;
    const int fop = FILT ? P.filters[0].op : 0;
    const double fdc = FILT ? P.filters[0].dc : 0.0;
    const i64 fic = FILT ? P.filters[0].ic : 0;
    u32 rc[REG_HOT];
#pragma unroll
    for (int q = 0; q < REG_HOT; q++) rc[q] = 0;
    for (;;) {
        u32 c = ~0u;
        if (lane == 0 && *(volatile u32 *)&T.ctl->stop == 0) {
            const u32 t = atomicAdd(&T.ctl->tile_counter, 1u);
            if (t < A.n_tiles) c = t;
        }
        c = __shfl_sync(FULL, c, 0);
        if (c == ~0u) break;
        const u64 c0 = ((u64)A.first_tile + c) * (u64)(P1D_RUN * P1D_CLAIM);
        for (int stp = 0; stp < P1D_CLAIM; stp++) {
            const u64 r0 = c0 + (u64)stp * P1D_RUN;
            if (r0 >= n) break;
            u64 k[4], v[4];
            u32 live = 0xfu;
            if (vec && r0 + P1D_RUN <= n) {
#pragma unroll
                for (int j = 0; j < 2; j++) {
                    const ulonglong2 a = __ldcs((const ulonglong2 *)(kcol + r0 + 64 * j + 2 * lane));
                    const ulonglong2 b = __ldcs((const ulonglong2 *)(vcol + r0 + 64 * j + 2 * lane));
                    k[2 * j] = a.x;
                    k[2 * j + 1] = a.y;
                    v[2 * j] = b.x;
                    v[2 * j + 1] = b.y;
                }
            } else {
                live = 0;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const u64 r = r0 + 64 * (j >> 1) + 2 * lane + (j & 1);
                    k[j] = 0;
                    v[j] = 0;
                    if (r < n) {
                        k[j] = kcol[r];
                        v[j] = vcol[r];
                        live |= 1u << j;
                    }
                }
            }
            if (FILT) {
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const bool pass = OPK == OP_ADD_F ? cmp_f(fop, __longlong_as_double((i64)v[j]), fdc)
                                                      : cmp_i(fop, (i64)v[j], fic);
                    if (!pass) live &= ~(1u << j);
                }
            }
            u32 cp[4];  // partition + 1 of a cold row, 0 otherwise
#pragma unroll
            for (int j = 0; j < 4; j++) {
                cp[j] = 0;
                if (!((live >> j) & 1u)) continue;
                const u64 key = k[j];
                if (key == EMPTY_KEY) {  // out-of-band slot of the HBM table
                    fold_atomic<1>(P, oob, 1, &v[j]);
                    continue;
                }
                const u64 h = p1_hash(key);
                const u32 b = hot_bucket(h, HB);
                const ulonglong2 kk = hb[b];
                const u32 rr = hr[b];
                const int rank = kk.x == key ? (int)(rr & 0xffffu) : (kk.y == key ? (int)(rr >> 16) : -1);
                if (rank >= 0) {
#pragma unroll
                    for (int q = 0; q < REG_HOT; q++) rc[q] += rank == q ? 1u : 0u;
                    if (rank >= REG_HOT) atomicAdd(&sc[rank], 1u);
                    u64 *w = hsum + (size_t)rank * W;
                    if (OPK == OP_ADD_F) atomicAdd((double *)w, __longlong_as_double((i64)v[j]));
                    else atomicAdd((unsigned long long *)w, (unsigned long long)v[j]);
                } else {
                    cp[j] = part_of(h, R.pbits) + 1;
                }
            }
            // every reservation of the step is issued before its stores
            u32 pos[4];
#pragma unroll
            for (int j = 0; j < 4; j++)
                pos[j] = cp[j] ? atomicAdd(&X.cursor[(u64)(cp[j] - 1) * CURSOR_PAD], 1u) : 0u;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                if (!cp[j]) continue;
                const u32 p = cp[j] - 1;
                if (pos[j] < pcap[p]) {
                    *(ulonglong2 *)(X.part + (pbase[p] + pos[j]) * 2) = make_ulonglong2(k[j], v[j]);
                } else {
                    put_overflow<1>(X, T, p, k[j], &v[j]);
                    if (*(volatile u32 *)&T.ctl->aux0 > X.ovf_threshold) atomicExch(&T.ctl->stop, 1u);
                }
            }
        }
    }
    // register counts (summed over the warp) join the shared counts
#pragma unroll
    for (int q = 0; q < REG_HOT; q++) {
        const u32 t = __reduce_add_sync(FULL, rc[q]);
        if (lane == 0 && t && q < NH) atomicAdd(&sc[q], t);
    }
    __syncthreads();
    // counts into word 0 of this CTA's hot slice (only this CTA writes it)
    u64 *hcnt = X.hot_part + (u64)blockIdx.x * NH * W;
    for (int i = threadIdx.x; i < NH; i += blockDim.x)
        if (sc[i]) hcnt[(size_t)i * W] += sc[i];
}

// Append overflow tuples to their (grown) partitions.
__global__ void k_part_drain(const RadixRef X, int V, u32 n) {
    const int TV = 1 + V;
    for (u64 i = blockIdx.x * (u64)blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
        const u64 *src = X.ovf + i * (TV + 1);
        const u32 p = (u32)src[0];
        const u64 pos = atomicAdd(&X.cursor[(u64)p * CURSOR_PAD], 1u);
        u64 *dst = X.part + (X.part_off[p] + pos) * TV;
        for (int q = 0; q < TV; q++) dst[q] = src[1 + q];
    }
}

// Copy each partition's filled prefix into the (larger) regions of `to`.
__global__ void k_part_move(const RadixRef from, const RadixRef to, int V) {
    const int TV = 1 + V;
    const u32 p = blockIdx.x;
    const u64 n = (u64)min(from.cursor[(u64)p * CURSOR_PAD], from.part_cap[p]) * TV;
    const u64 *src = from.part + from.part_off[p] * TV;
    u64 *dst = to.part + to.part_off[p] * TV;
    for (u64 i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

__global__ void k_fill_u64(u64 *dst, u64 n, u64 value) {
    for (u64 i = blockIdx.x * (u64)blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) dst[i] = value;
}

// ------------------------------------------------------------- P2 aggregate
// One CTA per partition: a shared open-addressing table (u64 keys, u32
// counts, W-1 state words).  Warps pre-combine duplicate keys, then fold with
// native u32 count atomics and (rarely contended) word atomics; no barriers
// in the main loop.  (Plans whose ops are all DOUBLE SUMs take
// k_part_agg_sum, whose words fold in L2.)
template <int VV, int NOPS>
__global__ void __launch_bounds__(RADIX_BLOCK, 1)
    k_part_agg(const __grid_constant__ Plan P, const __grid_constant__ RadixPlan R, const RadixRef X,
               const TableRef T, const __grid_constant__ EmitArgs E, int SP) {
    extern __shared__ u64 rsm[];
    constexpr int TV = 1 + VV;
    constexpr int NV = NOPS > 0 ? NOPS : 1;
    const int W = P.words, WM = W - 1;
    const int lane = threadIdx.x & 31;
    u64 *keys = rsm;  // [SP]
    u64 *wd = keys + SP;                        // [SP][WM]
    u32 *cn = (u32 *)(wd + (size_t)SP * WM);    // [SP]
    __shared__ u32 s_new;
    for (int i = threadIdx.x; i < SP; i += blockDim.x) {
        keys[i] = EMPTY_KEY;
        cn[i] = 0;
        for (int w = 0; w < WM; w++) wd[(size_t)i * WM + w] = P.word_init[1 + w];
    }
    if (threadIdx.x == 0) s_new = 0;
    const u32 p = blockIdx.x;
    const u64 n = min((u64)X.cursor[(u64)p * CURSOR_PAD], (u64)X.part_cap[p]);
    const u64 *base = X.part + X.part_off[p] * TV;
    if (threadIdx.x < 32) {
        // the partition's tuples head for L2 in 32 KB pieces, one per lane
        const u64 bytes = n * TV * 8, piece = 32768;
        for (u64 o = (u64)threadIdx.x * piece; o < bytes; o += 32 * piece)
            l2_prefetch((const char *)base + o, min(piece, bytes - o));
    }
    __syncthreads();
    volatile u64 *vk = keys;
    for (u64 b0 = threadIdx.x - lane; b0 < n; b0 += blockDim.x) {
        const u64 i = b0 + lane;
        bool act = false;
        u64 pk = EMPTY_KEY ^ (u64)(lane + 1);
        u64 v[NV];
#pragma unroll
        for (int q = 0; q < NV; q++) v[q] = 0;
        if (i < n) {
            const u64 *tp = base + i * TV;
            const u64 k = tp[0];
            if (k != EMPTY_KEY) {
                u64 tv[VV];
#pragma unroll
                for (int q = 0; q < VV; q++) tv[q] = tp[1 + q];
                tuple_contrib<VV, NOPS>(P, R, tv, v);
                pk = k;
                act = true;
            }
        }
        const u64 hh = mix64(pk);
        if (!R.p2_pre) {
            // tail keys rarely repeat within 32 consecutive tuples: fold each
            // tuple on its own
            if (!act) continue;
            const u64 cnt = 1;
            u32 s = agg_slot(hh, SP);
            bool done = false;
            for (int q = 0; q < R.agg_probe; q++) {
                u64 k = vk[s];
                if (k == EMPTY_KEY) {
                    const u64 old = atomicCAS(&keys[s], EMPTY_KEY, pk);
                    k = (old == EMPTY_KEY) ? pk : old;
                }
                if (k == pk) {
                    atomicAdd(&cn[s], (u32)cnt);
#pragma unroll
                    for (int o = 0; o < NOPS; o++)
                        op_apply(P.ops[o].kind, wd + (size_t)s * WM + (P.ops[o].word - 1), v[o],
                                 P.word_init[P.ops[o].word]);
                    done = true;
                    break;
                }
                s = (s + 1) & (u32)(SP - 1);
            }
            if (!done) global_fold_n<NOPS>(P, T, pk, cnt, v, &s_new);
            continue;
        }
        // pre-combine lanes with equal keys: match on 32 hash bits (cheaper
        // than a 64-bit match), then keep only lanes whose full key equals
        // their group leader's; the others stay leaders of themselves
        const unsigned am = __ballot_sync(FULL, act);
        unsigned peers = __match_any_sync(FULL, (unsigned)hh) & am;
        const int ldr = __ffs(peers) - 1;
        const u64 lkey = __shfl_sync(FULL, pk, ldr < 0 ? lane : ldr);
        const bool same = act && lkey == pk;
        peers &= __ballot_sync(FULL, same);
        const bool leader = act && (!same || ldr == lane);
        if (!same) peers = act ? (1u << lane) : 0u;
        unsigned rem = (leader && same) ? (peers & ~(1u << lane)) : 0u;
        const int maxit = __reduce_max_sync(FULL, (unsigned)__popc(rem));
        for (int it = 0; it < maxit; it++) {
            const int src = rem ? (__ffs(rem) - 1) : lane;
            rem &= rem - 1u;
#pragma unroll
            for (int q = 0; q < NOPS; q++) {
                const u64 o = __shfl_sync(FULL, v[q], src);
                if (src != lane) v[q] = op_combine(P.ops[q].kind, v[q], o);
            }
        }
        if (!leader) continue;
        const u64 cnt = __popc(peers);
        u32 s = agg_slot(hh, SP);
        bool done = false;
        for (int q = 0; q < R.agg_probe; q++) {
            u64 k = vk[s];
            if (k == EMPTY_KEY) {
                const u64 old = atomicCAS(&keys[s], EMPTY_KEY, pk);
                k = (old == EMPTY_KEY) ? pk : old;
            }
            if (k == pk) {
                atomicAdd(&cn[s], (u32)cnt);
#pragma unroll
                for (int o = 0; o < NOPS; o++)
                    op_apply(P.ops[o].kind, wd + (size_t)s * WM + (P.ops[o].word - 1), v[o],
                             P.word_init[P.ops[o].word]);
                done = true;
                break;
            }
            s = (s + 1) & (u32)(SP - 1);
        }
        if (!done) global_fold_n<NOPS>(P, T, pk, cnt, v, &s_new);
    }
    __syncthreads();
    // emit: one output reservation per CTA
    u32 mine = 0;
    for (int s = threadIdx.x; s < SP; s += blockDim.x) mine += keys[s] != EMPTY_KEY;
    u64 o = block_out_base(T.ctl, mine);
    for (int s = threadIdx.x; s < SP; s += blockDim.x) {
        if (keys[s] == EMPTY_KEY) continue;
        if (o >= E.out_cap) {
            atomicOr(&T.ctl->err, (u32)ERR_OUT_OVERFLOW);
            continue;
        }
        u64 w[GB_MAX_WORDS];
        w[0] = cn[s];
        for (int q = 0; q < WM; q++) w[1 + q] = wd[(size_t)s * WM + q];
        emit_group(P, E, o, keys[s], false, w);
        o++;
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_new) atomicAdd(&T.ctl->n_groups, s_new);
}

// P2 for plans whose ops are all DOUBLE SUMs of the one value column (the
// COUNT / SUM / AVG(DOUBLE) shape): shared memory holds only keys and u32
// counts; the sum words of this partition live in its slice of p2_words and
// fold as fire-and-forget L2 reductions.  The CTA zeroes its slice first:
// full-line stores allocate the lines in L2 without a DRAM read, so the
// reductions that follow hit L2 (a slice left zero between runs instead made
// every first reduction of a line miss).  One 128-bit load per tuple, no
// per-op switch; the slot comes from bits 20.. of the P1 hash (the partition
// took its top bits).
template <int NOPS>
__global__ void __launch_bounds__(RADIX_BLOCK, 1)
    k_part_agg_sum(const __grid_constant__ Plan P, const __grid_constant__ RadixPlan R, const RadixRef X,
                   const TableRef T, const __grid_constant__ EmitArgs E, int SP) {
    extern __shared__ u64 rsm[];
    const int WM = P.words - 1;
    u64 *keys = rsm;               // [SP]
    u32 *cn = (u32 *)(keys + SP);  // [SP]
    u64 *wd = X.p2_words + (size_t)blockIdx.x * SP * WM;  // [SP][WM]
    __shared__ u32 s_new;
    for (int i = threadIdx.x; i < SP; i += blockDim.x) {
        keys[i] = EMPTY_KEY;
        cn[i] = 0;
    }
    for (int i = threadIdx.x; i < SP * WM; i += blockDim.x) wd[i] = 0ull;  // DOUBLE SUM identity
    if (threadIdx.x == 0) s_new = 0;
    const u32 p = blockIdx.x;
    const u64 n = min((u64)X.cursor[(u64)p * CURSOR_PAD], (u64)X.part_cap[p]);
    const ulonglong2 *base = (const ulonglong2 *)(X.part + X.part_off[p] * 2);
    if (threadIdx.x < 32) {
        const u64 bytes = n * 16, piece = 32768;
        for (u64 o = (u64)threadIdx.x * piece; o < bytes; o += 32 * piece)
            l2_prefetch((const char *)base + o, min(piece, bytes - o));
    }
    int wo[NOPS];
#pragma unroll
    for (int o = 0; o < NOPS; o++) wo[o] = P.ops[o].word - 1;
    __syncthreads();
    volatile u64 *vk = keys;
    for (u64 i = threadIdx.x; i < n; i += blockDim.x) {
        const ulonglong2 t = __ldcs(base + i);
        const u64 pk = t.x;
        if (pk == EMPTY_KEY) continue;  // a padding hole of the write-combining P1
        u32 s = agg_slot(p1_hash(pk), SP);
        bool done = false;
        for (int q = 0; q < R.agg_probe; q++) {
            u64 k = vk[s];
            if (k == EMPTY_KEY) {
                const u64 old = atomicCAS(&keys[s], EMPTY_KEY, pk);
                k = (old == EMPTY_KEY) ? pk : old;
            }
            if (k == pk) {
                atomicAdd(&cn[s], 1u);
#pragma unroll
                for (int o = 0; o < NOPS; o++)
                    atomicAdd((double *)(wd + (size_t)s * WM + wo[o]), __longlong_as_double((i64)t.y));
                done = true;
                break;
            }
            s = (s + 1) & (u32)(SP - 1);
        }
        if (!done) {
            u64 v[NOPS];
#pragma unroll
            for (int o = 0; o < NOPS; o++) v[o] = t.y;
            global_fold_n<NOPS>(P, T, pk, 1, v, &s_new);
        }
    }
    __threadfence();  // the reductions reach L2 before the emit reads them
    __syncthreads();
    u32 mine = 0;
    for (int s = threadIdx.x; s < SP; s += blockDim.x) mine += keys[s] != EMPTY_KEY;
    u64 o = block_out_base(T.ctl, mine);
    for (int s = threadIdx.x; s < SP; s += blockDim.x) {
        if (keys[s] == EMPTY_KEY) continue;
        if (o >= E.out_cap) {
            atomicOr(&T.ctl->err, (u32)ERR_OUT_OVERFLOW);
            continue;
        }
        u64 w[GB_MAX_WORDS];
        w[0] = cn[s];
        for (int q = 0; q < WM; q++) w[1 + q] = __ldcg(wd + (size_t)s * WM + q);
        emit_group(P, E, o, keys[s], false, w);
        o++;
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_new) atomicAdd(&T.ctl->n_groups, s_new);
}

// ------------------------------------------------------------- P3 hot
// One warp per hot key: lanes fold the per-CTA slices lane, lane+32, ... and
// a fixed shuffle tree combines them (deterministic order).  Output rows are
// reserved per block.
__global__ void k_hot_emit(const __grid_constant__ Plan P, const __grid_constant__ RadixPlan R, const RadixRef X,
                           int G, const u32 *hstate, Ctl *ctl, const __grid_constant__ EmitArgs E) {
    const int W = P.words, NH = R.nh, NSUP = R.nsup;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const u32 nsup = min(hstate[0], (u32)NSUP), nwarm = min(hstate[1], (u32)(NH - NSUP));
    for (u64 k0 = (u64)blockIdx.x * nwarps; k0 < (u64)NH; k0 += (u64)gridDim.x * nwarps) {
        const u64 s = k0 + warp;
        const bool used = s < (u64)NH && (s < nsup || (s >= (u64)NSUP && s < (u64)NSUP + nwarm));
        u64 w[GB_MAX_WORDS];
        for (int q = 0; q < W; q++) w[q] = P.word_init[q];
        if (used) {
            for (int g = lane; g < G; g += 32) {
                const u64 *hp = X.hot_part + ((u64)g * NH + s) * W;
                w[0] += hp[0];
                for (int q = 1; q < W; q++) w[q] = op_combine(R.word_kind[q], w[q], hp[q]);
            }
            for (int o = 16; o > 0; o >>= 1) {
                w[0] += __shfl_xor_sync(FULL, w[0], o);
                for (int q = 1; q < W; q++) w[q] = op_combine(R.word_kind[q], w[q], __shfl_xor_sync(FULL, w[q], o));
            }
        }
        const bool occ = used && w[0] != 0 && lane == 0;
        u64 o = block_out_base(ctl, occ ? 1u : 0u);
        if (!occ) continue;
        if (o >= E.out_cap) {
            atomicOr(&ctl->err, (u32)ERR_OUT_OVERFLOW);
            continue;
        }
        emit_group(P, E, o, X.hot_list[s], false, w);
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

size_t radix_p1_smem(const Plan &P, const RadixPlan &R) {
    const size_t WM = P.words - 1, NP = (size_t)1 << R.pbits, V = R.V;
    const size_t NWARM = R.nh - R.nsup;
    return (size_t)R.HS * 8 + (size_t)P1_WARPS * R.nsup * WM * 8 + NWARM * WM * 8 + NP * R.wcb * (1 + V) * 8 +
           (size_t)P1_WARPS * R.nsup * 4 + NWARM * 4 + 3 * NP * 4 + (size_t)R.HS * 2;
}

size_t radix_p2_smem(const Plan &P, const RadixPlan &R) {
    const size_t WM = P.words - 1, SP = (size_t)R.sub;
    return SP * 8 + SP * WM * 8 + SP * 4;
}

bool radix_p2_global_words(const Plan &P, const RadixPlan &R) {
    if (P.n_ops < 1 || P.n_ops > 2 || R.V != 1) return false;
    for (int i = 0; i < P.n_ops; i++)
        if (P.ops[i].kind != OP_ADD_F) return false;
    return true;
}

// Rows of one claim of the P1 kernel that runs (a CTA tile of the generic
// kernel, a warp claim of the specialised one) and the rows that can still be
// in flight when the kernel is told to stop (every claim is finished).
u32 radix_tile_rows(const RadixPlan &R) {
    if (R.spec) return (u32)(P1D_RUN * P1D_CLAIM);
    return (u32)((R.V == 3 ? RADIX_ROWS / 2 : RADIX_ROWS) * P1_WARPS * 32);
}
u64 radix_inflight_rows(const RadixPlan &R, int grid) {
    return (u64)grid * radix_tile_rows(R) * (R.spec ? P1_WARPS : 1);
}

// The specialised P1 applies (decided when the plan is made: the columns'
// NOT NULL declarations hold for every ingest): one non-NULL BIGINT key, one
// non-NULL value column, one ADD op, no predicates.
static int p1_spec(const Plan &P, const RadixPlan &R, u64 nullable_mask) {
    if (P.key_mode != KEY_SINGLE || P.cols[P.key_col[0]].type != GB_T_BIGINT) return 0;
    if ((nullable_mask >> P.key_col[0]) & 1ull) return 0;
    if (R.V != 1 || P.n_ops != 1 || P.n_filters > 1 || ((nullable_mask >> R.vcol[0]) & 1ull)) return 0;
    // one compare on the value column itself (its type is the op's)
    if (P.n_filters && (P.filters[0].col != R.vcol[0] || P.filters[0].op > GB_CMP_GE)) return 0;
    const int t = P.cols[R.vcol[0]].type;
    if (P.ops[0].kind == OP_ADD_F && t == GB_T_DOUBLE) return OP_ADD_F;
    if (P.ops[0].kind == OP_ADD_I && t == GB_T_BIGINT) return OP_ADD_I;
    return 0;
}

int radix_spec_of(const Plan &P, const RadixPlan &R, u64 nullable_mask) { return p1_spec(P, R, nullable_mask); }

static const size_t kSmemBudget = 224 * 1024;  // <= the 227 KiB opt-in minus static shared memory

gb_status radix_prepare(const Plan &P, RadixPlan &R, u64 est_groups, u64 nullable_mask) {
    memset(&R, 0, sizeof R);
    if (P.key_mode == KEY_STRING || P.n_dist) return GB_ERR_UNSUPPORTED;
    if (P.n_ops > RADIX_MAX_OPS) return GB_ERR_UNSUPPORTED;
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
    if (R.V == 0) {  // COUNT(*) only: the tuple carries one unused value
        R.vcol[0] = P.key_col[0];
        R.V = 1;
    }
    if (P.words > GB_MAX_WORDS) return GB_ERR_UNSUPPORTED;
    R.spec = p1_spec(P, R, nullable_mask);
    // P2: one shared table of `sub` slots per partition (keys + counts only,
    // 12 bytes a slot, when the state words fold in L2)
    int sp = 8192;
    R.sub = sp;
    if (radix_p2_global_words(P, R) && (size_t)16384 * 12 <= kSmemBudget) {
        sp = 16384;
        R.sub = sp;
    }
    while (sp > 512 && !radix_p2_global_words(P, R) && radix_p2_smem(P, R) > kSmemBudget) {
        sp /= 2;
        R.sub = sp;
    }
    R.agg_probe = 64;
    // a table whose words fold in L2 takes repeated keys cheaply: no pre-combine
    R.p2_pre = radix_p2_global_words(P, R) ? 0 : 1;
    // partitions so that a partition's groups fill its table to <= ~0.7
    const u64 per_part = (u64)sp * 7 / 10;
    u64 np = pow2_at_least(std::max<u64>((est_groups + per_part - 1) / per_part, 64));
    np = std::min<u64>(np, 4096);
    int pb = 0;
    while ((1ull << pb) < np) pb++;
    R.pbits = pb;
    R.wcb = 4;  // write-combining tuples per partition per flush
    // P1: hot set of nh keys, the nsup hottest private per warp; shrink to fit
    R.HS = 8192;
    R.nh = 4096;
    R.nsup = 64;
    R.hot_probe = 8;
    if (R.spec) return radix_p1d_smem(R) <= kSmemBudget ? GB_OK : GB_ERR_UNSUPPORTED;
    while (radix_p1_smem(P, R) > kSmemBudget) {
        // keep the hot set large (a key left out of it lands in P2, where its
        // repeats contend): shrink the warp-private tier first
        if (R.pbits > 10) R.pbits--;
        else if (R.nsup > 32) R.nsup -= 16;
        else if (R.nh > 1024) {
            R.nh /= 2;
            R.HS /= 2;
        } else if (R.pbits > 8) R.pbits--;
        else if (R.nsup > 16) R.nsup /= 2;
        else if (R.nh > 64) {
            R.nh /= 2;
            R.HS /= 2;
        } else if (R.pbits > 6) R.pbits--;
        else return GB_ERR_UNSUPPORTED;
    }
    return GB_OK;
}

// Override the partition count (2^bits partitions) chosen by radix_prepare.
gb_status radix_set_bits(const Plan &P, RadixPlan &R, int bits) {
    if (bits < 6 || bits > 12) return GB_ERR_INVALID;
    RadixPlan t = R;
    t.pbits = bits;
    if ((t.spec ? radix_p1d_smem(t) : radix_p1_smem(P, t)) > kSmemBudget) return GB_ERR_UNSUPPORTED;
    R = t;
    return GB_OK;
}

static gb_status radix_set_attributes();

gb_status radix_launch_sample(const Plan &P, const RadixPlan &R, u64 n, u64 *skeys, u32 *scnt, u64 scap,
                              u32 *hist, u32 *hstate, u64 *cand_key, u32 *cand_cnt, u64 *hot_keys,
                              uint16_t *hot_idx, u64 *hot_list, cudaStream_t st, u64 *launches) {
    if (R.nh > 4096 || R.HS != 2 * R.nh) {
        set_error("radix plan: the hot set holds at most 4096 keys in twice as many bucket slots");
        return GB_ERR_INVALID;
    }
    if (gb_status s = radix_set_attributes()) return s;
    const u64 m = std::min<u64>(n, scap / 2);
    const u64 step = std::max<u64>(1, n / std::max<u64>(m, 1));
    const int sms = sm_count();
    k_sample_count<<<grid_of(m, 256, sms * 4), 256, 0, st>>>(P, n, step, m, skeys, scnt, scap);
    k_sample_hist<<<grid_of(scap, 256, sms * 2), 256, 0, st>>>(skeys, scnt, scap, hist);
    k_hot_collect<<<grid_of(scap, 256, sms * 2), 256, 0, st>>>(skeys, scnt, scap, hist, hstate, R.nh, cand_key,
                                                              cand_cnt);
    k_hot_rank<<<1, 1024, HOT_RANK_SMEM, st>>>(cand_key, cand_cnt, hstate, R.nsup, R.nh, R.HS / 2, hot_keys, hot_idx,
                                               hot_list);
    *launches += 4;
    GB_CUDA(cudaGetLastError());
    return GB_OK;
}

// Raise a kernel's dynamic shared-memory limit to what the device allows
// next to the kernel's static shared memory.
template <typename F>
static gb_status allow_max_smem(F f) {
    int dev = 0, optin = 0;
    GB_CUDA(cudaGetDevice(&dev));
    GB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes a;
    GB_CUDA(cudaFuncGetAttributes(&a, f));
    GB_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)a.sharedSizeBytes));
    return GB_OK;
}

typedef void (*P1Fn)(Plan, RadixPlan, RadixRef, TableRef, RadixTile);
typedef void (*P2Fn)(Plan, RadixPlan, RadixRef, TableRef, EmitArgs, int);

template <int VV, int NOPS>
static void p1_table(P1Fn *t) {
    t[VV * (RADIX_MAX_OPS + 1) + NOPS] = (P1Fn)k_partition<(VV == 3 ? RADIX_ROWS / 2 : RADIX_ROWS), VV, NOPS>;
}
template <int VV, int NOPS>
static void p2_table(P2Fn *t) {
    t[VV * (RADIX_MAX_OPS + 1) + NOPS] = (P2Fn)k_part_agg<VV, NOPS>;
}

template <int VV>
static void fill_tables(P1Fn *t1, P2Fn *t2) {
    p1_table<VV, 0>(t1); p1_table<VV, 1>(t1); p1_table<VV, 2>(t1); p1_table<VV, 3>(t1); p1_table<VV, 4>(t1);
    p2_table<VV, 0>(t2); p2_table<VV, 1>(t2); p2_table<VV, 2>(t2); p2_table<VV, 3>(t2); p2_table<VV, 4>(t2);
}

static P1Fn g_p1[4 * (RADIX_MAX_OPS + 1)];
static P2Fn g_p2[4 * (RADIX_MAX_OPS + 1)];
static P1Fn g_p1_spec[2][2];  // specialised P1: BIGINT key, one SUM [integer, DOUBLE][predicate]
static P2Fn g_p2_gw[RADIX_MAX_OPS + 1];  // P2 with the state words in L2 (ops all DOUBLE SUM), one value column

static gb_status radix_set_attributes() {
    static bool done = false;
    if (done) return GB_OK;
    fill_tables<1>(g_p1, g_p2);
    fill_tables<2>(g_p1, g_p2);
    fill_tables<3>(g_p1, g_p2);
    g_p1_spec[0][0] = (P1Fn)k_partition_direct<OP_ADD_I, false>;
    g_p1_spec[0][1] = (P1Fn)k_partition_direct<OP_ADD_I, true>;
    g_p1_spec[1][0] = (P1Fn)k_partition_direct<OP_ADD_F, false>;
    g_p1_spec[1][1] = (P1Fn)k_partition_direct<OP_ADD_F, true>;
    g_p2_gw[1] = (P2Fn)k_part_agg_sum<1>;
    g_p2_gw[2] = (P2Fn)k_part_agg_sum<2>;
    for (P1Fn f : {g_p1_spec[0][0], g_p1_spec[0][1], g_p1_spec[1][0], g_p1_spec[1][1]})
        if (gb_status s = allow_max_smem(f)) return s;
    if (gb_status s = allow_max_smem(k_hot_rank)) return s;
    for (int o = 1; o <= 2; o++)
        if (gb_status s = allow_max_smem(g_p2_gw[o])) return s;
    for (int v = 1; v <= 3; v++)
        for (int o = 0; o <= RADIX_MAX_OPS; o++) {
            gb_status s;
            if ((s = allow_max_smem(g_p1[v * (RADIX_MAX_OPS + 1) + o]))) return s;
            if ((s = allow_max_smem(g_p2[v * (RADIX_MAX_OPS + 1) + o]))) return s;
        }
    done = true;
    return GB_OK;
}

gb_status radix_launch_p1(const Plan &P, const RadixPlan &R, const RadixRef &X, const TableRef &T,
                          const RadixTile &A, int grid, cudaStream_t st) {
    gb_status s = radix_set_attributes();
    if (s) return s;
    size_t smem = radix_p1_smem(P, R);
    P1Fn f = g_p1[R.V * (RADIX_MAX_OPS + 1) + P.n_ops];
    if (R.spec) {
        // the plan's NOT NULL declarations were checked against every column
        if (P.cols[P.key_col[0]].valid || P.cols[R.vcol[0]].valid) {
            set_error("radix plan: a NOT NULL column carries a validity mask");
            return GB_ERR_INVALID;
        }
        f = g_p1_spec[R.spec == OP_ADD_F ? 1 : 0][P.n_filters ? 1 : 0];
        smem = radix_p1d_smem(R);
    }
    f<<<grid, P1_WARPS * 32, smem, st>>>(P, R, X, T, A);
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
    gb_status s = radix_set_attributes();
    if (s) return s;
    size_t smem = radix_p2_smem(P, R);
    const int np = 1 << R.pbits;
    P2Fn f = g_p2[R.V * (RADIX_MAX_OPS + 1) + P.n_ops];
    if (X.p2_words && radix_p2_global_words(P, R)) {
        f = g_p2_gw[P.n_ops];
        smem = (size_t)R.sub * 12;
    }
    f<<<np, RADIX_BLOCK, smem, st>>>(P, R, X, T, E, R.sub);
    GB_CUDA(cudaGetLastError());
    return GB_OK;
}

gb_status radix_launch_p3(const Plan &P, const RadixPlan &R, const RadixRef &X, int G, const u32 *hstate, Ctl *ctl,
                          const EmitArgs &E, cudaStream_t st) {
    if (R.nh == 0) return GB_OK;
    k_hot_emit<<<grid_of((u64)R.nh * 32, 256, sm_count() * 4), 256, 0, st>>>(P, R, X, G, hstate, ctl, E);
    GB_CUDA(cudaGetLastError());
    return GB_OK;
}

gb_status radix_launch_move(const RadixRef &from, const RadixRef &to, int V, int np, cudaStream_t st) {
    k_part_move<<<np, 256, 0, st>>>(from, to, V);
    GB_CUDA(cudaGetLastError());
    return GB_OK;
}

gb_status radix_fill_u64(u64 *dst, u64 n, u64 value, cudaStream_t st) {
    k_fill_u64<<<grid_of(n, 256, sm_count() * 8), 256, 0, st>>>(dst, n, value);
    GB_CUDA(cudaGetLastError());
    return GB_OK;
}

gb_status radix_fill_identity(u64 *dst, u64 n, int W, const Plan &P, cudaStream_t st) {
    k_fill_words<<<grid_of(n, 256, sm_count() * 8), 256, 0, st>>>(dst, n, W, P);
    GB_CUDA(cudaGetLastError());
    return GB_OK;
}

}  // namespace gb
