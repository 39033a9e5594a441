// gb_kernels.cuh — the hash-aggregation device code shared by the single
// query path (gb_agg.cu) and the batched persistent path (gb_batch.cu).
//
// Row pipeline per warp (32 consecutive rows, coalesced column loads):
//   filter predicates → packed 64-bit group key → __match_any_sync groups the
//   lanes holding the same key → segmented shuffle reduction combines their
//   partial states into the lowest lane (the "leader") → the leader folds
//   the combined partial into the CTA's shared-memory open-addressing table
//   with shared-memory atomics → if the shared table has no room the partial
//   goes to the HBM table with global atomics → if the HBM table is too full
//   (probe bound) the partial is spilled as a record and merged after the
//   host grows the table.  At CTA exit the shared table is flushed into the
//   HBM table.
//
// This restates the reference's per-row probe + AggState update
// (src/execution/physical_planner.cpp:7933-8021 in-memory loop, 7698-7820
// fused Parquet loop) with a three-level GPU memory hierarchy in place of
// the per-thread ankerl maps and their shard merge (7871-7908).
#pragma once

#include "gb_internal.cuh"

namespace gb {

struct Ctl {
    u32 n_groups;      // groups inserted in the HBM table
    u32 spill_count;   // spill records written
    u32 tile_counter;  // tiles claimed by persistent CTAs
    u32 stop;          // set when the spill buffer nears its threshold
    u32 err;           // ErrFlag bits
    u32 out_count;     // rows written by compaction
    u32 aux0, aux1;
};

struct TableRef {
    u64 *slots;        // (cap + 2) * stride words
    u64 cap;           // power of two
    int32_t stride;
    int32_t gmax_probe;
    Ctl *ctl;
    u64 *spill;        // spill_cap records of (1 + words) words
    u32 spill_cap;
    u32 spill_threshold;
};

// ----------------------------------------------------------------- keys
// Returns 0 = ordinary key in pk, 1 = pk equals EMPTY_KEY (out-of-band slot
// cap+0), 2 = NULL key (slot cap+1), 3 = NULL in a full-width pair key
// (unsupported; flagged).
__device__ __forceinline__ int make_key(const Plan &P, u64 r, u64 &pk) {
    if (P.key_mode == KEY_SINGLE || P.key_mode == KEY_STRING) {
        const DevCol &c = P.cols[P.key_col[0]];
        if (!row_valid(c.valid, r)) { pk = 0; return 2; }
        pk = (u64)load_int(c, r);
        if (P.key_mode == KEY_STRING && (i64)pk < 0) { pk = 0; return 2; }  // NULL string → id -1
        return pk == EMPTY_KEY ? 1 : 0;
    }
    const DevCol &ca = P.cols[P.key_col[0]];
    const DevCol &cb = P.cols[P.key_col[1]];
    bool va = row_valid(ca.valid, r), vb = row_valid(cb.valid, r);
    u64 a = va ? (u64)load_int(ca, r) : 0ull;
    u64 b = vb ? (u64)load_int(cb, r) : 0ull;
    if (P.key_mode == KEY_PACKED) {
        const int bb = P.key_bits_b, ba = P.key_bits_a;
        const u64 mb = (bb >= 64) ? ~0ull : ((1ull << bb) - 1ull);
        const u64 ma = (ba >= 64) ? ~0ull : ((1ull << ba) - 1ull);
        pk = ((a & ma) << bb) | (b & mb) | ((u64)(!va) << (ba + bb)) | ((u64)(!vb) << (ba + bb + 1));
        return 0;
    }
    if (!va || !vb) { pk = 0; return 3; }
    pk = ((a & 0xffffffffull) << 32) | (b & 0xffffffffull);
    return pk == EMPTY_KEY ? 1 : 0;
}

__device__ __forceinline__ bool pass_filters(const Plan &P, u64 r) {
    for (int i = 0; i < P.n_filters; i++) {
        const Filter &f = P.filters[i];
        const DevCol &c = P.cols[f.col];
        if (!row_valid(c.valid, r)) return false;
        if (c.type == GB_T_VARCHAR) {
            const i64 b = c.offsets[r], e = c.offsets[r + 1];
            if (!str_pred(f.op, (const uint8_t *)c.data + b, (u64)(e - b), f.ptr, f.n)) return false;
        } else if (f.op == GB_CMP_IN) {
            if (!in_set(f.ptr, f.n, load_int(c, r))) return false;
        } else if (c.type == GB_T_DOUBLE) {
            if (!cmp_f(f.op, load_f64(c, r), f.dc)) return false;
        } else {
            if (!cmp_i(f.op, load_int(c, r), f.ic)) return false;
        }
    }
    return true;
}

// Per-op partial contributions of row r (identity where the input is NULL).
__device__ __forceinline__ void load_vals(const Plan &P, u64 r, u64 *v) {
#pragma unroll
    for (int i = 0; i < GB_MAX_OPS; i++) {
        if (i < P.n_ops) {
            const Op o = P.ops[i];
            const DevCol &c = P.cols[o.col];
            const bool ok = row_valid(c.valid, r);
            u64 x = P.word_init[o.word];
            if (ok) {
                switch (o.kind) {
                case OP_ADD_F: x = (u64)__double_as_longlong(load_f64(c, r)); break;
                case OP_MIN_F:
                case OP_MAX_F: x = (u64)enc_f64(load_f64(c, r)); break;
                case OP_CNT_NN: x = 1ull; break;
                default: x = (u64)load_int(c, r); break;
                }
            }
            v[i] = x;
        }
    }
}

// ------------------------------------------------------------ distinct pairs
// COUNT(DISTINCT v) keeps, per distinct column, one open-addressing set of
// (group key, value) pairs in HBM.  A slot is claimed by one 128-bit
// compare-and-swap, so a pair is never half-written and no thread waits on
// another; the set is sized by the host to a load factor <= 1/2 before each
// ingest, so a probe always meets an empty slot.  The empty marker is the
// pair (EMPTY_KEY, EMPTY_KEY); the real pair equal to it (the INT64_MIN key
// with the INT64_MIN value) is tracked by a flag word instead.
#define DIST_NULL_KEY 0x4000000000000000ull  // NULL-key group of a key narrower than 64 bits

__device__ __forceinline__ void cas128(u64 *p, u64 cmp_lo, u64 cmp_hi, u64 new_lo, u64 new_hi, u64 &old_lo,
                                       u64 &old_hi) {
    asm volatile(
        "{\n\t.reg .b128 c, n, o;\n\t"
        "mov.b128 c, {%2, %3};\n\t"
        "mov.b128 n, {%4, %5};\n\t"
        "atom.global.cas.b128 o, [%6], c, n;\n\t"
        "mov.b128 {%0, %1}, o;\n\t}"
        : "=l"(old_lo), "=l"(old_hi)
        : "l"(cmp_lo), "l"(cmp_hi), "l"(new_lo), "l"(new_hi), "l"(p)
        : "memory");
}

__device__ __forceinline__ u64 pair_hash(u64 g, u64 v) { return mix64(mix64(g) ^ v); }

// Insert (g, v) into the set at `set` (mask + 1 slots).  Returns true when
// the pair is new.  meta: the plan's dmeta words; d: the set's index.
__device__ __forceinline__ bool dset_insert(u64 *set, u64 mask, u64 g, u64 v, unsigned long long *meta, int d) {
    if (g == EMPTY_KEY && v == EMPTY_KEY) return atomicExch(meta + 2 + d, 1ull) == 0ull;
    u64 s = pair_hash(g, v) & mask;
    for (u64 q = 0; q <= mask; q++) {
        u64 lo, hi;
        cas128(set + 2 * s, EMPTY_KEY, EMPTY_KEY, g, v, lo, hi);
        if (lo == EMPTY_KEY && hi == EMPTY_KEY) return true;
        if (lo == g && hi == v) return false;
        s = (s + 1) & mask;
    }
    atomicExch(meta + 1, 1ull);  // full: the host sized it wrongly
    return false;
}

// The narrow form: a 16/32-bit key and a 16/32-bit value packed into one
// 8-byte slot (key in the high half), claimed by one 64-bit compare-and-swap;
// the empty marker is all ones, and the real pair equal to it (key -1, value
// -1) is tracked by the same flag word as the wide form's marker pair.
__device__ __forceinline__ bool dset_insert_narrow(u64 *set, u64 mask, u64 e, unsigned long long *meta, int d) {
    if (e == ~0ull) return atomicExch(meta + 2 + d, 1ull) == 0ull;
    u64 s = mix64(e) & mask;
    for (u64 q = 0; q <= mask; q++) {
        const u64 old = atomicCAS((unsigned long long *)(set + s), ~0ull, e);
        if (old == ~0ull) return true;
        if (old == e) return false;
        s = (s + 1) & mask;
    }
    atomicExch(meta + 1, 1ull);  // full: the host sized it wrongly
    return false;
}

// Replace each OP_DIST contribution of row r (key pk of kind `kind`, as
// make_key returns) by 1 if its (group, value) pair is new, else 0.
__device__ __forceinline__ void dist_vals(const Plan &P, u64 r, int kind, u64 pk, u64 *v, u32 *new_pairs) {
#pragma unroll
    for (int i = 0; i < GB_MAX_OPS; i++) {
        if (i < P.n_ops && P.ops[i].kind == OP_DIST) {
            const Op o = P.ops[i];
            const DevCol &c = P.cols[o.col];
            u64 x = 0;
            if (row_valid(c.valid, r) && P.dnarrow) {
                const u64 e = ((u64)(uint32_t)pk << 32) | (uint32_t)load_int(c, r);
                if (dset_insert_narrow(P.dsets + (P.dmask + 1) * o.dset, P.dmask, e, P.dmeta, o.dset)) {
                    x = 1;
                    atomicAdd(new_pairs, 1u);
                }
            } else if (row_valid(c.valid, r)) {
                const u64 val = (u64)load_int(c, r);
                const u64 slots = P.dmask + 1;
                u64 *set = P.dsets + 2 * slots * o.dset;
                u64 g = pk;
                if (kind == 1) {
                    g = EMPTY_KEY;
                } else if (kind == 2) {
                    if (P.null_sets) {
                        set = P.null_sets + 2 * slots * o.dset;
                        g = 0;
                    } else {
                        g = DIST_NULL_KEY;
                    }
                }
                if (dset_insert(set, P.dmask, g, val, P.dmeta, o.dset)) {
                    x = 1;
                    atomicAdd(new_pairs, 1u);
                }
            }
            v[i] = x;
        }
    }
}

// ------------------------------------------------------------ HBM table
// Find or claim the slot of pk.  Returns the slot index or -1 if the probe
// bound was reached.  `new_groups` counts claimed slots (CTA-local).
__device__ __forceinline__ long long g_slot(const TableRef &T, u64 pk, u64 h, u32 *new_groups) {
    u64 s = h & (T.cap - 1);
    for (int p = 0; p < T.gmax_probe; p++) {
        u64 *kp = T.slots + s * (u64)T.stride;
        u64 k = *(volatile u64 *)kp;
        if (k == pk) return (long long)s;
        if (k == EMPTY_KEY) {
            u64 old = atomicCAS(kp, EMPTY_KEY, pk);
            if (old == EMPTY_KEY) {
                atomicAdd(new_groups, 1u);
                return (long long)s;
            }
            if (old == pk) return (long long)s;
        }
        s = (s + 1) & (T.cap - 1);
    }
    return -1;
}

__device__ __forceinline__ void apply_state(const Plan &P, u64 *w, u64 cnt, const u64 *v) {
    if (cnt) atomicAdd(w, cnt);
#pragma unroll
    for (int i = 0; i < GB_MAX_OPS; i++) {
        if (i < P.n_ops) {
            const Op o = P.ops[i];
            op_apply(o.kind, w + o.word, v[i], P.word_init[o.word]);
        }
    }
}

__device__ __forceinline__ void spill_record(const Plan &P, const TableRef &T, u64 pk, u64 cnt, const u64 *v) {
    u32 idx = atomicAdd(&T.ctl->spill_count, 1u);
    if (idx >= T.spill_cap) {
        atomicOr(&T.ctl->err, (u32)ERR_SPILL_OVERFLOW);
        return;
    }
    u64 *rec = T.spill + (u64)idx * (u64)(1 + P.words);
    rec[0] = pk;
    rec[1] = cnt;
    for (int i = 0; i < P.n_ops; i++) rec[1 + P.ops[i].word] = v[i];
}

// Fold a combined partial into the HBM table (or spill it).
__device__ __forceinline__ void global_fold(const Plan &P, const TableRef &T, u64 pk, u64 cnt, const u64 *v,
                                            u32 *new_groups) {
    long long s = g_slot(T, pk, mix64(pk), new_groups);
    if (s < 0) {
        spill_record(P, T, pk, cnt, v);
        return;
    }
    apply_state(P, T.slots + (u64)s * (u64)T.stride + 1, cnt, v);
}

// Out-of-band slots (EMPTY_KEY-valued key, NULL key) are folded directly.
__device__ __forceinline__ void special_fold(const Plan &P, const TableRef &T, int kind, u64 cnt, const u64 *v) {
    u64 *w = T.slots + (T.cap + (u64)(kind - 1)) * (u64)T.stride + 1;
    apply_state(P, w, cnt, v);
}

// ------------------------------------------------------ shared-memory table
struct SmemTable {
    u64 *keys;   // S keys
    u64 *st;     // S * words state words
    int S;       // power of two (0 = disabled)
    int probe;   // probe bound
};

__device__ __forceinline__ void smem_init(const Plan &P, SmemTable &t) {
    for (int i = threadIdx.x; i < t.S; i += blockDim.x) {
        t.keys[i] = EMPTY_KEY;
        for (int w = 0; w < P.words; w++) t.st[(u64)i * P.words + w] = P.word_init[w];
    }
}

// Returns true if folded into shared memory.
__device__ __forceinline__ bool smem_fold(const Plan &P, SmemTable &t, u64 pk, u64 h, u64 cnt, const u64 *v) {
    if (t.S == 0) return false;
    u32 s = (u32)(h >> 40) & (u32)(t.S - 1);
    volatile u64 *vk = t.keys;
    for (int p = 0; p < t.probe; p++) {
        u64 k = vk[s];
        bool hit = (k == pk);
        if (!hit && k == EMPTY_KEY) {
            u64 old = atomicCAS(&t.keys[s], EMPTY_KEY, pk);
            hit = (old == EMPTY_KEY || old == pk);
        }
        if (hit) {
            apply_state(P, t.st + (u64)s * P.words, cnt, v);
            return true;
        }
        s = (s + 1) & (u32)(t.S - 1);
    }
    return false;
}

__device__ __forceinline__ void smem_flush(const Plan &P, const TableRef &T, SmemTable &t, u32 *new_groups) {
    for (int i = threadIdx.x; i < t.S; i += blockDim.x) {
        u64 k = t.keys[i];
        if (k == EMPTY_KEY) continue;
        const u64 *st = t.st + (u64)i * P.words;
        u64 v[GB_MAX_OPS];
#pragma unroll
        for (int j = 0; j < GB_MAX_OPS; j++)
            if (j < P.n_ops) v[j] = st[P.ops[j].word];
        global_fold(P, T, k, st[0], v, new_groups);
    }
}

// ------------------------------------------------------- warp row step
// Processes rows [base, base+32) ∩ [.., end) of the current batch; rows
// index the column vectors (row_ids != nullptr: gather through ids).
template <bool PRECOMBINE>
__device__ __forceinline__ void warp_rows(const Plan &P, const TableRef &T, SmemTable &sm, u64 base, u64 end,
                                          u32 *new_groups, u32 *new_pairs) {
    const int lane = threadIdx.x & 31;
    const u64 r = base + lane;
    bool act = r < end;
    if (act && P.n_filters) act = pass_filters(P, r);
    u64 pk = 0;
    u64 v[GB_MAX_OPS];
#pragma unroll
    for (int i = 0; i < GB_MAX_OPS; i++) v[i] = 0;
    if (act) {
        int kind = make_key(P, r, pk);
        load_vals(P, r, v);
        if (P.n_dist && kind != 3) dist_vals(P, r, kind, pk, v, new_pairs);
        if (kind != 0) {
            if (kind == 3) atomicOr(&T.ctl->err, (u32)ERR_NULL_IN_WIDE_KEY);
            else special_fold(P, T, kind, 1, v);
            act = false;
        }
    }
    const unsigned am = __ballot_sync(FULL, act);
    if (am == 0) return;
    u64 cnt = 1;
    if (PRECOMBINE) {
        unsigned peers = __match_any_sync(FULL, pk) & am;
        const bool leader = act && ((__ffs(peers) - 1) == lane);
        unsigned rem = leader ? (peers & ~(1u << lane)) : 0u;
        cnt = __popc(peers);
        const int maxit = __reduce_max_sync(FULL, (unsigned)__popc(rem));
        for (int it = 0; it < maxit; it++) {
            const int src = rem ? (__ffs(rem) - 1) : lane;
            rem &= rem - 1u;
#pragma unroll
            for (int i = 0; i < GB_MAX_OPS; i++) {
                if (i < P.n_ops) {
                    u64 o = __shfl_sync(FULL, v[i], src);
                    if (src != lane) v[i] = op_combine(P.ops[i].kind, v[i], o);
                }
            }
        }
        act = leader;
    }
    if (!act) return;
    const u64 h = mix64(pk);
    if (!smem_fold(P, sm, pk, h, cnt, v)) global_fold(P, T, pk, cnt, v, new_groups);
}

// ------------------------------------------------------------ emit
struct EmitAgg {
    int32_t kind;      // gb_agg_kind
    int32_t in_type;   // gb_type of the input column (-1 for COUNT(*))
    int32_t out_type;  // gb_type of the output column
    int32_t val_word;  // state word of the value (-1 none)
    int32_t cnt_word;  // state word of the non-NULL count
    int32_t pad;
};

struct EmitArgs {
    EmitAgg aggs[GB_MAX_AGGS];
    void *out[2 + GB_MAX_AGGS];        // device column buffers
    uint64_t *valid[2 + GB_MAX_AGGS];  // validity words (pre-set to all ones)
    int32_t n_aggs;
    int32_t n_keys;
    u64 out_cap;
};

__device__ __forceinline__ void store_int(void *base, int type, u64 i, i64 v) {
    switch (type) {
    case GB_T_SMALLINT: ((int16_t *)base)[i] = (int16_t)v; break;
    case GB_T_INTEGER: ((int32_t *)base)[i] = (int32_t)v; break;
    default: ((long long *)base)[i] = v; break;
    }
}

__device__ __forceinline__ void clear_valid(uint64_t *vw, u64 i) {
    atomicAnd((unsigned long long *)(vw + (i >> 6)), ~(1ull << (i & 63)));
}

__device__ __forceinline__ i64 sext(u64 x, int bits) {
    if (bits >= 64) return (i64)x;
    u64 m = 1ull << (bits - 1);
    x &= (1ull << bits) - 1ull;
    return (i64)((x ^ m) - m);
}


// Write one group's result row `o` (key columns + finalised aggregates,
// agg_emit_helpers.cpp:26-98 rules).  `w` = the group's state words.
__device__ __forceinline__ void emit_group(const Plan &P, const EmitArgs &E, u64 o, u64 pk, bool null_key,
                                           const u64 *w) {
    if (P.key_mode == KEY_SINGLE || P.key_mode == KEY_STRING) {
        store_int(E.out[0], P.key_type[0], o, (i64)pk);
        if (null_key) clear_valid(E.valid[0], o);
    } else if (P.key_mode == KEY_PACKED) {
        const int bb = P.key_bits_b, ba = P.key_bits_a;
        i64 a = sext(pk >> bb, ba), b = sext(pk, bb);
        bool na = (pk >> (ba + bb)) & 1ull, nb = (pk >> (ba + bb + 1)) & 1ull;
        // a VARCHAR position holds its string id, emitted as BIGINT
        store_int(E.out[0], P.str_key == 0 ? GB_T_BIGINT : P.key_type[0], o, a);
        store_int(E.out[1], P.str_key == 1 ? GB_T_BIGINT : P.key_type[1], o, b);
        if (na) clear_valid(E.valid[0], o);
        if (nb) clear_valid(E.valid[1], o);
    } else {
        store_int(E.out[0], P.str_key == 0 ? GB_T_BIGINT : P.key_type[0], o, (i64)(int32_t)(uint32_t)(pk >> 32));
        store_int(E.out[1], P.str_key == 1 ? GB_T_BIGINT : P.key_type[1], o, (i64)(int32_t)(uint32_t)pk);
    }
    for (int a = 0; a < E.n_aggs; a++) {
        const EmitAgg &g = E.aggs[a];
        void *dst = E.out[E.n_keys + a];
        uint64_t *vw = E.valid[E.n_keys + a];
        const u64 cnt = w[g.cnt_word];
        switch (g.kind) {
        case GB_AGG_COUNT_STAR:
        case GB_AGG_COUNT: ((long long *)dst)[o] = (i64)cnt; break;
        case GB_AGG_COUNT_DISTINCT: ((long long *)dst)[o] = (i64)w[g.val_word]; break;
        case GB_AGG_SUM:
            if (cnt == 0) { ((long long *)dst)[o] = 0; clear_valid(vw, o); }
            else ((long long *)dst)[o] = (i64)w[g.val_word];  // int64 or double bits
            break;
        case GB_AGG_AVG:
            if (cnt == 0) { ((double *)dst)[o] = 0.0; clear_valid(vw, o); }
            else {
                double sum = (g.in_type == GB_T_DOUBLE) ? __longlong_as_double((i64)w[g.val_word])
                                                        : (double)(i64)w[g.val_word];
                ((double *)dst)[o] = sum / (double)cnt;
            }
            break;
        default:  // MIN / MAX
            if (cnt == 0) {
                store_int(dst, g.out_type == GB_T_DOUBLE ? GB_T_BIGINT : g.out_type, o, 0);
                clear_valid(vw, o);
            } else if (g.out_type == GB_T_DOUBLE) ((double *)dst)[o] = dec_f64((i64)w[g.val_word]);
            else store_int(dst, g.out_type, o, (i64)w[g.val_word]);
            break;
        }
    }
}

// Block-cooperative output reservation: every thread of the block passes the
// number of rows it will emit and gets the index of its first one; one global
// atomic per block (a per-warp atomic on the single counter serialises).
// Must be called by all threads of the block, blockDim.x a multiple of 32.
__device__ __forceinline__ u64 block_out_base(Ctl *ctl, u32 mine) {
    __shared__ u32 s_warp[32];
    __shared__ u32 s_total;
    __shared__ unsigned long long s_base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    u32 x = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const u32 y = __shfl_up_sync(FULL, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        u32 w = lane < nwarps ? s_warp[lane] : 0u;
        u32 incl = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const u32 y = __shfl_up_sync(FULL, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane < nwarps) s_warp[lane] = incl - w;
        if (lane == 31) s_total = incl;
    }
    __syncthreads();
    if (threadIdx.x == 0) s_base = s_total ? atomicAdd(&ctl->out_count, s_total) : 0u;
    __syncthreads();
    const u64 r = s_base + s_warp[warp] + (x - mine);
    __syncthreads();  // s_warp / s_base are reused by the next call
    return r;
}

// Reserve `n` output rows for a warp's occupied lanes (ballot + one atomic).
__device__ __forceinline__ u64 warp_out_slot(Ctl *ctl, bool occ, unsigned active) {
    const int lane = threadIdx.x & 31;
    const unsigned m = __ballot_sync(active, occ);
    u32 base = 0;
    const int leader = __ffs(active) - 1;
    if (lane == leader && m) base = atomicAdd(&ctl->out_count, (u32)__popc(m));
    base = __shfl_sync(active, base, leader);
    return (u64)base + __popc(m & ((1u << lane) - 1u));
}

}  // namespace gb
