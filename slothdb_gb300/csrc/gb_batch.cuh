// gb_batch.cuh — many independent GROUP BY queries in one pass (included at
// the end of gb_agg.cu, whose handle internals it reuses).
//
// The reference runs such queries one after another, each through its own
// PhysicalHashAggregate (src/execution/physical_planner.cpp:12291-12516 for
// composite / VARCHAR keys).  Here every query keeps its own gb_agg handle
// (plan, HBM table, outputs, string dictionary), and the batch executes:
//
//   k_batch_init     one launch: every query's table to its identity state;
//   k_batch_strdict  one launch: VARCHAR keys of every VARCHAR query → ids;
//   k_batch_fast /   one persistent launch per plan class over a device
//   k_batch_generic  work queue of (query, tile) items (query-major, so one
//                    table at a time is hot in L2; uneven sizes balance
//                    dynamically).  Integer plans run a specialised,
//                    register-resident pipeline with narrow shared-memory
//                    states; any other plan runs the single-query pipeline
//                    with its plan copied into shared memory per item;
//   k_batch_compact  one launch: every query's table → its dense result.
//
// The sequence is captured once in a CUDA graph and replayed.  The graph is
// the fast path: a query that needs a host decision (table spill, string
// dictionary growth) is re-run on its own handle afterwards.

#define BATCH_TILE 16384  // default rows per work item (option "tile_rows")
#define FAST_MAX_OPS 4        // ops a register-resident plan holds (single-query kernels)
#define BATCH_FAST_MAX_OPS 2  // ops of the batch's fast plan classes
#define FAST_MAX_FILTERS 2

// Integer-plan description kept in registers by the fast tile path (up to
// FAST_MAX_FILTERS predicates on integer or DOUBLE columns; keys SINGLE /
// PACKED / STRING; ops ADD_I, MIN_I, MAX_I, CNT_NN over integer columns).  kdesc = key_mode | kt0 << 4 | kt1 << 8 | bits_b << 16 |
// bits_a << 24; op[i] = kind | type << 4 | table word << 8 | shared word << 16
// | wide << 24, wide = a MIN/MAX over BIGINT (64-bit shared word).
struct FastPlan {
    const void *kp[2];
    const uint64_t *kv[2];
    const void *vp[FAST_MAX_OPS];
    const uint64_t *vv[FAST_MAX_OPS];
    u32 kdesc;
    u32 op[FAST_MAX_OPS];
    int32_t n_filters;
    int32_t n_ops;
    int32_t swords;    // 32-bit words per shared state: count, then the ops
    int32_t eligible;
    int32_t nulls;     // some key, op or filter column has a validity mask
};

// Predicates of the fast path (read from shared memory, once per row).
struct FastFilters {
    const void *fp[FAST_MAX_FILTERS];
    const uint64_t *fv[FAST_MAX_FILTERS];
    u64 fk[FAST_MAX_FILTERS];     // constant: int64, or the bits of a double
    u32 fdesc[FAST_MAX_FILTERS];  // column type | gb_cmp << 4
};

struct BQuery {
    FastPlan F;
    FastFilters FF;
    Plan P;
    TableRef T;
    EmitArgs E;
    StrDictRef D;
    const uint8_t *sbytes;
    const int64_t *soffs;
    const uint64_t *svalid;
    long long *ids;
    // VARCHAR results emitted inside the batch: per-row lengths, offsets
    // (n + 1), bytes, and per-chunk sums then bases
    int64_t *str_lens;
    int64_t *str_offs;
    uint8_t *str_out;
    int64_t *str_chunk;
    u32 *sretry;
    u64 n_rows;
    u64 table_words;
    u64 init_words;  // table words, output validity words, dictionary words
    int32_t smem_slots;
    int32_t is_str;
    int32_t pre;        // fast path: combine equal keys within a warp first
    u32 tile_rows;
};

struct BItem {
    u32 q;
    u32 idx;
};

__device__ __forceinline__ void copy_words(void *dst, const void *src, int bytes) {
    const u32 *s = (const u32 *)src;
    u32 *d = (u32 *)dst;
    for (int i = threadIdx.x; i < bytes / 4; i += blockDim.x) d[i] = s[i];
}

// Item (q, idx) covers words [idx * 65536, (idx+1) * 65536) of the query's
// init range: the table words, then the validity words of every output column
// (all ones; the emit clears the bits of NULL results), then (COUNT(DISTINCT))
// the pair sets, their NULL-key twins and the pair counters, after, for a VARCHAR
// key the dictionary's hash slots (free), ref slots (unpublished) and its
// eight counter words (zero).
__global__ void k_batch_init(const BQuery *qs, const BItem *items, u32 n_items) {
    for (u32 it = blockIdx.x; it < n_items; it += gridDim.x) {
        const BItem w = items[it];
        const BQuery &q = qs[w.q];
        const int stride = q.P.stride;
        const u64 vwords = (q.E.out_cap + 63) / 64;
        const u64 n0 = q.table_words, n1 = n0 + (u64)(q.E.n_keys + q.E.n_aggs) * vwords;
        const u64 dc = q.is_str ? q.D.cap : 0;
        const u64 n2 = n1 + (q.is_str ? 2 * dc + 8 : 0);
        const u64 sw = q.P.n_dist ? (q.P.dmask + 1) * (q.P.dnarrow ? 1 : 2) * (u64)q.P.n_dist : 0;
        const u64 nw = q.P.null_sets ? sw : 0;
        const u64 dempty = q.P.dnarrow ? ~0ull : EMPTY_KEY;
        const u64 lo = (u64)w.idx * 65536, hi = min(q.init_words, lo + 65536);
        for (u64 i = lo + threadIdx.x; i < hi; i += blockDim.x) {
            if (i < n0) {
                const int wd = (int)(i % (u64)stride);
                u64 v;
                if (wd == 0) v = EMPTY_KEY;
                else if (wd - 1 < q.P.words) v = q.P.word_init[wd - 1];
                else v = 0;
                q.T.slots[i] = v;
            } else if (i < n1) {
                const u64 j = i - n0;
                q.E.valid[j / vwords][j % vwords] = ~0ull;
            } else if (i < n1 + dc) {
                q.D.hash[i - n1] = EMPTY_KEY;
            } else if (i < n1 + 2 * dc) {
                q.D.ref[i - n1 - dc] = REF_PENDING;
            } else if (i < n2) {
                q.D.next_id[i - n1 - 2 * dc] = 0;  // next id, arena used, error word, spare
            } else if (i < n2 + sw) {
                q.P.dsets[i - n2] = dempty;  // COUNT(DISTINCT) pair sets: empty
            } else if (i < n2 + sw + nw) {
                q.P.null_sets[i - n2 - sw] = dempty;
            } else {
                q.P.dmeta[i - n2 - sw - nw] = 0;  // pairs, overflow flag, marker flags
            }
        }
    }
}

__global__ void __launch_bounds__(256, 4) k_batch_strdict(const BQuery *qs, const BItem *items, u32 n_items) {
    __shared__ StrDictRef D;
    __shared__ u32 s_new;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (u32 it = blockIdx.x; it < n_items; it += gridDim.x) {
        const BItem w = items[it];
        const BQuery &q = qs[w.q];
        if (threadIdx.x == 0) {
            D = q.D;
            s_new = 0;
        }
        __syncthreads();
        const u64 lo = (u64)w.idx * 8192, hi = min(q.n_rows, lo + 8192);
        for (u64 base = lo + (u64)warp * 32; base < hi; base += (u64)nwarps * 32) {
            const u64 r = base + lane;
            bool act = r < hi;
            if (act && q.svalid && !((q.svalid[r >> 6] >> (r & 63)) & 1ull)) {
                q.ids[r] = -1;
                act = false;
            }
            const int64_t a = act ? q.soffs[r] : 0;
            const u32 len = act ? (u32)(q.soffs[r + 1] - a) : 0u;
            const long long id = strdict_warp_encode(D, q.sbytes + a, len, act, &s_new);
            if (!act) continue;
            q.ids[r] = id;
            if (id < 0) atomicAdd(&q.T.ctl->aux1, 1u);  // needs the host: the query re-runs on its handle
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------- fast tiles
__device__ __forceinline__ i64 fast_load(const void *p, int t, u64 r) {
    switch (t) {
    case GB_T_SMALLINT: return (i64)__ldg((const int16_t *)p + r);
    case GB_T_INTEGER: return (i64)__ldg((const int32_t *)p + r);
    default: return (i64)__ldg((const long long *)p + r);
    }
}

__device__ __forceinline__ u64 fast_ident(int kind) {
    return kind == OP_MIN_I ? 0x7fffffffffffffffull : (kind == OP_MAX_I ? 0x8000000000000000ull : 0ull);
}

// Fold a partial into an HBM state (count at word 0, op i at its word).
template <int NOPS>
__device__ __forceinline__ void fast_apply_global(const FastPlan &F, u64 *w, u64 cnt, const u64 *v) {
    if (cnt) atomicAdd(w, cnt);
#pragma unroll
    for (int i = 0; i < NOPS; i++) {
        const u32 od = F.op[i];
        const int kind = od & 15;
        op_apply(kind, w + ((od >> 8) & 255), v[i], fast_ident(kind));
    }
}

template <int NOPS>
__device__ __forceinline__ void fast_global(const FastPlan &F, const TableRef &T, u64 pk, u64 cnt, const u64 *v,
                                            u32 *new_groups) {
    const long long s = g_slot(T, pk, mix64(pk), new_groups);
    if (s < 0) {
        atomicAdd(&T.ctl->spill_count, 1u);  // the query re-runs on its own handle
        return;
    }
    fast_apply_global<NOPS>(F, T.slots + (u64)s * (u64)T.stride + 1, cnt, v);
}

// As fast_global, for the single-query kernel: a key that finds no slot
// within the probe bound becomes a spill record (the host grows the table and
// merges the records) instead of a re-run.
template <int NOPS>
__device__ __forceinline__ void fast_global_spill(const FastPlan &F, const Plan &P, const TableRef &T, u64 pk, u64 cnt,
                                                  const u64 *v, u32 *new_groups) {
    const long long s = g_slot(T, pk, mix64(pk), new_groups);
    if (s < 0) {
        spill_record(P, T, pk, cnt, v);
        return;
    }
    fast_apply_global<NOPS>(F, T.slots + (u64)s * (u64)T.stride + 1, cnt, v);
}

// Narrow shared states: count u32; ADD as a (lo, hi) u32 pair with carry;
// CNT_NN u32; MIN/MAX s32 over SMALLINT/INTEGER, s64 over BIGINT.  Every
// update is a native 32-bit shared atomic except the 64-bit MIN/MAX.
template <int NOPS>
__device__ __forceinline__ void fast_apply_smem(const FastPlan &F, u32 *st, u64 cnt, const u64 *v) {
    atomicAdd(st, (u32)cnt);
#pragma unroll
    for (int i = 0; i < NOPS; i++) {
        const u32 od = F.op[i];
        const int kind = od & 15;
        if (v[i] == fast_ident(kind)) continue;
        u32 *w = st + ((od >> 16) & 255);
        const bool wide = (od >> 24) & 1;
        switch (kind) {
        case OP_ADD_I: {
            const u32 lo = (u32)v[i], hi = (u32)(v[i] >> 32);
            const u32 old = atomicAdd(w, lo);
            const u32 carry = (old + lo) < old ? 1u : 0u;
            if (hi + carry) atomicAdd(w + 1, hi + carry);
            break;
        }
        case OP_MIN_I:
            if (wide) atomicMin((long long *)w, (long long)v[i]);
            else atomicMin((int *)w, (int)(i64)v[i]);
            break;
        case OP_MAX_I:
            if (wide) atomicMax((long long *)w, (long long)v[i]);
            else atomicMax((int *)w, (int)(i64)v[i]);
            break;
        default:  // CNT_NN
            atomicAdd(w, (u32)v[i]);
            break;
        }
    }
}

template <int NOPS>
__device__ __forceinline__ void fast_smem_init(const FastPlan &F, u64 *keys, u32 *st, int S) {
    for (int i = threadIdx.x; i < S; i += blockDim.x) {
        keys[i] = EMPTY_KEY;
        u32 *w = st + (u64)i * F.swords;
        w[0] = 0;
#pragma unroll
        for (int j = 0; j < NOPS; j++) {
            const u32 od = F.op[j];
            const int kind = od & 15;
            u32 *x = w + ((od >> 16) & 255);
            const bool wide = (od >> 24) & 1;
            if (kind == OP_ADD_I) {
                x[0] = 0;
                x[1] = 0;
            } else if (kind == OP_MIN_I || kind == OP_MAX_I) {
                if (wide) *(u64 *)x = fast_ident(kind);
                else x[0] = kind == OP_MIN_I ? 0x7fffffffu : 0x80000000u;
            } else {
                x[0] = 0;
            }
        }
    }
}

template <int NOPS, bool SPILL = false>
__device__ __forceinline__ void fast_smem_flush(const FastPlan &F, const TableRef &T, const u64 *keys, const u32 *st,
                                                int S, u32 *new_groups, const Plan *SP = nullptr) {
    for (int i = threadIdx.x; i < S; i += blockDim.x) {
        const u64 k = keys[i];
        if (k == EMPTY_KEY) continue;
        const u32 *w = st + (u64)i * F.swords;
        u64 v[NOPS ? NOPS : 1];
#pragma unroll
        for (int j = 0; j < NOPS; j++) {
            const u32 od = F.op[j];
            const int kind = od & 15;
            const u32 *x = w + ((od >> 16) & 255);
            const bool wide = (od >> 24) & 1;
            if (kind == OP_ADD_I) v[j] = (u64)x[0] | ((u64)x[1] << 32);
            else if (kind == OP_MIN_I || kind == OP_MAX_I) v[j] = wide ? *(const u64 *)x : (u64)(i64)(int)x[0];
            else v[j] = x[0];
        }
        if (SPILL) fast_global_spill<NOPS>(F, *SP, T, k, w[0], v, new_groups);
        else fast_global<NOPS>(F, T, k, w[0], v, new_groups);
    }
}

// Raw column values of one row, loaded one warp step ahead of their use so
// that the next step's loads are in flight while this step folds.
template <int NOPS, bool FILT>
struct FastRaw {
    i64 a, b;
    i64 x[NOPS ? NOPS : 1];
    u64 f[FILT ? FAST_MAX_FILTERS : 1];  // filter column values (raw bits)
    u32 vbits;  // bit 0/1 key validity, bit 2+i op column validity, bit 8+j filter column validity
    bool act;
};

template <int NOPS, bool NULLS, bool FILT>
__device__ __forceinline__ void fast_fetch(const FastPlan &F, const FastFilters &FF, u64 r, u64 end,
                                           FastRaw<NOPS, FILT> &w) {
    w.act = r < end;
    w.a = w.b = 0;
    w.vbits = 0;
#pragma unroll
    for (int i = 0; i < NOPS; i++) w.x[i] = 0;
    if (!w.act) return;
    const u32 kd = F.kdesc;
    w.a = fast_load(F.kp[0], (kd >> 4) & 15, r);
    w.vbits = NULLS ? (row_valid(F.kv[0], r) ? 1u : 0u) : ~0u;
    if ((kd & 15) == KEY_PACKED) {
        w.b = fast_load(F.kp[1], (kd >> 8) & 15, r);
        if (NULLS) w.vbits |= row_valid(F.kv[1], r) ? 2u : 0u;
    }
#pragma unroll
    for (int i = 0; i < NOPS; i++) {
        const u32 od = F.op[i];
        if ((od & 15) != OP_CNT_NN) w.x[i] = fast_load(F.vp[i], (od >> 4) & 15, r);
        if (NULLS) w.vbits |= row_valid(F.vv[i], r) ? (4u << i) : 0u;
    }
#pragma unroll
    for (int j = 0; j < (FILT ? FAST_MAX_FILTERS : 0); j++) {
        w.f[j] = 0;
        if (j < F.n_filters) {
            const int t = FF.fdesc[j] & 15;
            w.f[j] = t == GB_T_DOUBLE ? (u64)__double_as_longlong(__ldg((const double *)FF.fp[j] + r))
                                      : (u64)fast_load(FF.fp[j], t, r);
            if (NULLS) w.vbits |= row_valid(FF.fv[j], r) ? (256u << j) : 0u;
        }
    }
}

// The row passes every predicate (a NULL input fails it, as pass_filters).
__device__ __forceinline__ bool fast_pass(const FastPlan &F, const FastFilters &FF, const u64 *f, u32 vbits) {
    bool ok = true;
#pragma unroll
    for (int j = 0; j < FAST_MAX_FILTERS; j++) {
        if (j < F.n_filters) {
            const u32 fd = FF.fdesc[j];
            const int op = (fd >> 4) & 15;
            bool p;
            if ((fd & 15) == GB_T_DOUBLE)
                p = cmp_f(op, __longlong_as_double((i64)f[j]), __longlong_as_double((i64)FF.fk[j]));
            else
                p = cmp_i(op, (i64)f[j], (i64)FF.fk[j]);
            ok = ok && p && (vbits & (256u << j));
        }
    }
    return ok;
}

// The packed key of a fetched row, exactly as make_key builds it.
__device__ __forceinline__ int fast_key_of(u32 kd, i64 a_, i64 b_, u32 vbits, u64 &pk) {
    const int mode = kd & 15;
    if (mode != KEY_PACKED) {
        if (!(vbits & 1u)) { pk = 0; return 2; }
        pk = (u64)a_;
        if (mode == KEY_STRING && a_ < 0) { pk = 0; return 2; }
        return pk == EMPTY_KEY ? 1 : 0;
    }
    const int bb = (kd >> 16) & 255, ba = (kd >> 24) & 255;
    const bool va = vbits & 1u, vb = vbits & 2u;
    const u64 a = va ? (u64)a_ : 0ull, b = vb ? (u64)b_ : 0ull;
    const u64 mb = (bb >= 64) ? ~0ull : ((1ull << bb) - 1ull);
    const u64 ma = (ba >= 64) ? ~0ull : ((1ull << ba) - 1ull);
    pk = ((a & ma) << bb) | (b & mb) | ((u64)(!va) << (ba + bb)) | ((u64)(!vb) << (ba + bb + 1));
    return 0;
}

// One warp step of the fast path on fetched rows.
template <bool PRECOMBINE, int NOPS, bool FILT, bool SPILL = false>
__device__ __forceinline__ void fast_rows(const FastPlan &F, const FastFilters &FF, const TableRef &T, u64 *keys,
                                          u32 *st, int S, const FastRaw<NOPS, FILT> &w, u32 *new_groups,
                                          const Plan *SP = nullptr) {
    const int lane = threadIdx.x & 31;
    bool act = w.act && (!FILT || fast_pass(F, FF, w.f, w.vbits));
    u64 pk = 0;
    u64 v[NOPS ? NOPS : 1];
#pragma unroll
    for (int i = 0; i < NOPS; i++) {
        const int kind = F.op[i] & 15;
        v[i] = fast_ident(kind);
        if (act && (w.vbits & (4u << i))) v[i] = kind == OP_CNT_NN ? 1ull : (u64)w.x[i];
    }
    if (act) {
        const int kind = fast_key_of(F.kdesc, w.a, w.b, w.vbits, pk);
        if (kind != 0) {
            fast_apply_global<NOPS>(F, T.slots + (T.cap + (u64)(kind - 1)) * (u64)T.stride + 1, 1, v);
            act = false;
        }
    }
    const unsigned am = __ballot_sync(FULL, act);
    if (am == 0) return;
    u64 cnt = 1;
    if (PRECOMBINE) {
        const unsigned peers = __match_any_sync(FULL, pk) & am;
        const bool leader = act && ((__ffs(peers) - 1) == lane);
        unsigned rem = leader ? (peers & ~(1u << lane)) : 0u;
        cnt = __popc(peers);
        const int maxit = __reduce_max_sync(FULL, (unsigned)__popc(rem));
        for (int it = 0; it < maxit; it++) {
            const int src = rem ? (__ffs(rem) - 1) : lane;
            rem &= rem - 1u;
#pragma unroll
            for (int i = 0; i < NOPS; i++) {
                const u64 o = __shfl_sync(FULL, v[i], src);
                if (src != lane) v[i] = op_combine(F.op[i] & 15, v[i], o);
            }
        }
        act = leader;
    }
    if (!act) return;
    if (S) {
        const u64 h = mix64(pk);
        u32 s = (u32)(h >> 40) & (u32)(S - 1);
        volatile u64 *vk = keys;
        for (int p = 0; p < 8; p++) {
            const u64 k = vk[s];
            bool hit = k == pk;
            if (!hit && k == EMPTY_KEY) {
                const u64 old = atomicCAS(&keys[s], EMPTY_KEY, pk);
                hit = old == EMPTY_KEY || old == pk;
            }
            if (hit) {
                fast_apply_smem<NOPS>(F, st + (u64)s * F.swords, cnt, v);
                return;
            }
            s = (s + 1) & (u32)(S - 1);
        }
    }
    if (SPILL) fast_global_spill<NOPS>(F, *SP, T, pk, cnt, v, new_groups);
    else fast_global<NOPS>(F, T, pk, cnt, v, new_groups);
}

// One tile of the fast path (inlined into its class's kernel: the plan's
// fields stay in registers).
template <bool PRECOMBINE, int NOPS, bool NULLS, bool FILT>
__device__ __forceinline__ void fast_tile(const FastPlan &F, const FastFilters &FF, const TableRef &T, u64 *bsm,
                                          int smem_bytes, int S, u64 t0, u64 t1, u32 *new_groups) {
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    while (S && (size_t)S * (8 + 4 * (size_t)F.swords) > (size_t)smem_bytes) S >>= 1;
    u64 *keys = bsm;
    u32 *st = (u32 *)(bsm + S);
    fast_smem_init<NOPS>(F, keys, st, S);
    __syncthreads();
    const u64 step = (u64)nwarps * 32;
    u64 base = t0 + (u64)warp * 32;
    FastRaw<NOPS, FILT> cur, nxt;
    fast_fetch<NOPS, NULLS, FILT>(F, FF, base + (threadIdx.x & 31), t1, cur);
    for (; base < t1; base += step) {
        fast_fetch<NOPS, NULLS, FILT>(F, FF, base + step + (threadIdx.x & 31), t1, nxt);
        fast_rows<PRECOMBINE, NOPS, FILT>(F, FF, T, keys, st, S, cur, new_groups);
        cur = nxt;
    }
    __syncthreads();
    fast_smem_flush<NOPS>(F, T, keys, st, S, new_groups);
}

// One tile of the generic path (any plan; the plan is in shared memory).
template <bool PRECOMBINE>
__device__ __noinline__ void generic_tile(const Plan &sP, const TableRef &sT, u64 *bsm, int S, int smem_bytes, u64 t0,
                                          u64 t1, u32 *new_groups) {
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    SmemTable sm;
    sm.S = S;
    while (sm.S && (size_t)sm.S * 8 * (1 + sP.words) > (size_t)smem_bytes) sm.S >>= 1;
    sm.probe = 8;
    sm.keys = bsm;
    sm.st = bsm + sm.S;
    __shared__ u32 s_pairs;  // COUNT(DISTINCT): new pairs of this tile
    if (threadIdx.x == 0) s_pairs = 0;
    smem_init(sP, sm);
    __syncthreads();
    for (u64 base = t0 + (u64)warp * 32; base < t1; base += (u64)nwarps * 32)
        warp_rows<PRECOMBINE>(sP, sT, sm, base, t1, new_groups, &s_pairs);
    __syncthreads();
    smem_flush(sP, sT, sm, new_groups);
    if (threadIdx.x == 0 && s_pairs) atomicAdd(sP.dmeta, (unsigned long long)s_pairs);
}

// The persistent loop shared by the ingest kernels: claim the next item of
// this kernel's class, skip queries stopped by their spill threshold (they
// re-run on their own handle), run `tile` on it, publish the group count.
template <class Tile>
__device__ __forceinline__ void batch_item_loop(const BQuery *qs, const BItem *items, u32 n_items, Ctl *cctl,
                                                Tile tile) {
    __shared__ u32 s_item, s_new, s_skip;
    for (;;) {
        if (threadIdx.x == 0) {
            u32 t = ~0u;
            const u32 c = atomicAdd(&cctl->tile_counter, 1u);
            if (c < n_items) t = c;
            s_item = t;
            s_new = 0;
            s_skip = t != ~0u && *(volatile u32 *)&qs[items[t].q].T.ctl->stop != 0;
        }
        __syncthreads();
        const u32 it = s_item;
        if (it == ~0u) break;
        if (s_skip) {
            __syncthreads();
            continue;
        }
        const BItem w = items[it];
        const BQuery &q = qs[w.q];
        const u64 t0 = (u64)w.idx * q.tile_rows, t1 = min(q.n_rows, t0 + q.tile_rows);
        Ctl *qctl = tile(q, t0, t1, &s_new);
        __syncthreads();
        if (threadIdx.x == 0) {
            if (s_new) atomicAdd(&qctl->n_groups, s_new);
            if (*(volatile u32 *)&qctl->spill_count > q.T.spill_threshold) atomicExch(&qctl->stop, 1u);
        }
        __syncthreads();
    }
}

// Fast-path ingest for one plan class (PRECOMBINE, NOPS, NULLS, FILT): a
// separate kernel per class, so each gets its own register allocation.
template <bool PRECOMBINE, int NOPS, bool NULLS, bool FILT>
__global__ void __launch_bounds__(512, 2) k_batch_fast(const BQuery *qs, const BItem *items, u32 n_items, Ctl *cctl,
                                                    int smem_bytes) {
    extern __shared__ u64 bsm[];
    __shared__ FastFilters sFF;
    batch_item_loop(qs, items, n_items, cctl, [&](const BQuery &q, u64 t0, u64 t1, u32 *s_new) -> Ctl * {
        if (FILT) {
            copy_words(&sFF, &q.FF, (int)sizeof(FastFilters));
            __syncthreads();
        }
        const FastPlan F = q.F;
        const TableRef T = q.T;
        fast_tile<PRECOMBINE, NOPS, NULLS, FILT>(F, sFF, T, bsm, smem_bytes, q.smem_slots, t0, t1, s_new);
        return T.ctl;
    });
}

// Generic-path ingest (any plan; the plan is copied to shared memory per item).
template <bool PRECOMBINE>
__global__ void __launch_bounds__(512, 2) k_batch_generic(const BQuery *qs, const BItem *items, u32 n_items,
                                                       Ctl *cctl, int smem_bytes) {
    extern __shared__ u64 bsm[];
    __shared__ Plan sP;
    __shared__ TableRef sT;
    batch_item_loop(qs, items, n_items, cctl, [&](const BQuery &q, u64 t0, u64 t1, u32 *s_new) -> Ctl * {
        copy_words(&sP, &q.P, (int)sizeof(Plan));
        copy_words(&sT, &q.T, (int)sizeof(TableRef));
        __syncthreads();
        generic_tile<PRECOMBINE>(sP, sT, bsm, q.smem_slots, smem_bytes, t0, t1, s_new);
        return q.T.ctl;
    });
}

// Plan classes: 0 = generic without / 1 = with the warp pre-combine;
// 2 + (pre * 12 + nops * 4 + nulls * 2 + filt) = a fast-path kernel.
constexpr int BATCH_CLASSES = 2 + 24;

typedef void (*BatchKernel)(const BQuery *, const BItem *, u32, Ctl *, int);

static BatchKernel batch_kernel(int cls) {
    static const BatchKernel tab[BATCH_CLASSES] = {
        k_batch_generic<false>, k_batch_generic<true>,
        k_batch_fast<false, 0, false, false>, k_batch_fast<false, 0, false, true>,
        k_batch_fast<false, 0, true, false>, k_batch_fast<false, 0, true, true>,
        k_batch_fast<false, 1, false, false>, k_batch_fast<false, 1, false, true>,
        k_batch_fast<false, 1, true, false>, k_batch_fast<false, 1, true, true>,
        k_batch_fast<false, 2, false, false>, k_batch_fast<false, 2, false, true>,
        k_batch_fast<false, 2, true, false>, k_batch_fast<false, 2, true, true>,
        k_batch_fast<true, 0, false, false>, k_batch_fast<true, 0, false, true>,
        k_batch_fast<true, 0, true, false>, k_batch_fast<true, 0, true, true>,
        k_batch_fast<true, 1, false, false>, k_batch_fast<true, 1, false, true>,
        k_batch_fast<true, 1, true, false>, k_batch_fast<true, 1, true, true>,
        k_batch_fast<true, 2, false, false>, k_batch_fast<true, 2, false, true>,
        k_batch_fast<true, 2, true, false>, k_batch_fast<true, 2, true, true>,
    };
    return tab[cls];
}

__global__ void k_batch_compact(const BQuery *qs, const BItem *items, u32 n_items) {
    __shared__ EmitArgs sE;
    __shared__ Plan sP;
    for (u32 it = blockIdx.x; it < n_items; it += gridDim.x) {
        const BItem w = items[it];
        const BQuery &q = qs[w.q];
        copy_words(&sE, &q.E, (int)sizeof(EmitArgs));
        copy_words(&sP, &q.P, (int)sizeof(Plan));
        __syncthreads();
        const u64 cap = q.T.cap, total = cap + 2;
        const int stride = q.T.stride;
        const u64 c0 = (u64)w.idx * (COMPACT_PER * 256);
        u32 mine = 0;
#pragma unroll
        for (int j = 0; j < COMPACT_PER; j++) {
            const u64 s = c0 + (u64)j * blockDim.x + threadIdx.x;
            if (s >= total) break;
            const u64 *sl = q.T.slots + s * (u64)stride;
            mine += (s < cap) ? (sl[0] != EMPTY_KEY) : (sl[1] != 0);
        }
        u64 o = block_out_base(q.T.ctl, mine);
#pragma unroll
        for (int j = 0; j < COMPACT_PER; j++) {
            const u64 s = c0 + (u64)j * blockDim.x + threadIdx.x;
            if (s >= total) break;
            const u64 *sl = q.T.slots + s * (u64)stride;
            const bool occ = (s < cap) ? (sl[0] != EMPTY_KEY) : (sl[1] != 0);
            if (!occ) continue;
            if (o >= sE.out_cap) {
                atomicOr(&q.T.ctl->err, (u32)ERR_OUT_OVERFLOW);
                continue;
            }
            const u64 pk = (s < cap) ? sl[0] : (s == cap ? EMPTY_KEY : 0ull);
            emit_group(sP, sE, o, pk, s == cap + 1, sl + 1);
            o++;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------- VARCHAR results
// The string ids a VARCHAR query emitted become offsets + bytes inside the
// batch (no per-query host round trip): lengths and per-chunk sums, one scan
// of the chunk sums per query, then offsets and a byte gather per chunk.
// The row count is the query's out_count, read on the device.
#define STR_EMIT_CHUNK 4096

__device__ __forceinline__ long long block_sum_ll(long long x, long long *s_part) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(FULL, x, o);
    if (lane == 0) s_part[warp] = x;
    __syncthreads();
    long long t = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < nwarps; w++) t += s_part[w];
    __syncthreads();
    return t;  // valid in thread 0
}

__global__ void k_batch_str_len(const BQuery *qs, const BItem *items, u32 n_items) {
    __shared__ long long s_part[32];
    for (u32 it = blockIdx.x; it < n_items; it += gridDim.x) {
        const BItem w = items[it];
        const BQuery &q = qs[w.q];
        const u64 n = min((u64)q.T.ctl->out_count, q.E.out_cap);  // an overflow re-runs on the handle
        const u64 lo = (u64)w.idx * STR_EMIT_CHUNK, hi = min(n, lo + STR_EMIT_CHUNK);
        const long long *ids = (const long long *)q.E.out[0];
        long long local = 0;
        for (u64 r = lo + threadIdx.x; r < hi; r += blockDim.x) {
            const long long id = ids[r];
            const int64_t len = id < 0 ? 0 : (int64_t)(q.D.ref_by_id[id] & 0xffffffu);
            if (id < 0) atomicAnd((unsigned long long *)&q.E.valid[0][r >> 6], ~(1ull << (r & 63)));
            q.str_lens[r] = len;
            local += len;
        }
        const long long t = block_sum_ll(local, s_part);
        if (threadIdx.x == 0) q.str_chunk[w.idx] = t;
    }
}

// One block per VARCHAR query: exclusive scan of its chunk sums (in place)
// and the final offset.
__global__ void k_batch_str_scan(const BQuery *qs, const u32 *str_queries, u32 n_q) {
    __shared__ long long s_part[32];
    __shared__ long long s_carry;
    for (u32 i = blockIdx.x; i < n_q; i += gridDim.x) {
        const BQuery &q = qs[str_queries[i]];
        const u64 n = min((u64)q.T.ctl->out_count, q.E.out_cap);  // an overflow re-runs on the handle
        const u64 nch = (n + STR_EMIT_CHUNK - 1) / STR_EMIT_CHUNK;
        if (threadIdx.x == 0) s_carry = 0;
        __syncthreads();
        for (u64 c0 = 0; c0 < nch; c0 += blockDim.x) {
            const u64 c = c0 + threadIdx.x;
            const long long x = c < nch ? q.str_chunk[c] : 0;
            // block inclusive scan
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
            long long incl = x;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const long long y = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += y;
            }
            if (lane == 31) s_part[warp] = incl;
            __syncthreads();
            if (warp == 0) {
                const long long wv = lane < nwarps ? s_part[lane] : 0;
                long long wi = wv;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const long long y = __shfl_up_sync(FULL, wi, o);
                    if (lane >= o) wi += y;
                }
                if (lane < nwarps) s_part[lane] = wi - wv;
            }
            __syncthreads();
            const long long base = s_carry + s_part[warp];
            if (c < nch) q.str_chunk[c] = base + incl - x;
            __syncthreads();
            if (threadIdx.x == blockDim.x - 1) s_carry = base + incl;
            __syncthreads();
        }
        if (threadIdx.x == 0) q.str_offs[n] = s_carry;
        __syncthreads();
    }
}

__global__ void k_batch_str_gather(const BQuery *qs, const BItem *items, u32 n_items) {
    __shared__ long long s_part[32];
    __shared__ long long s_run;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (u32 it = blockIdx.x; it < n_items; it += gridDim.x) {
        const BItem w = items[it];
        const BQuery &q = qs[w.q];
        const u64 n = min((u64)q.T.ctl->out_count, q.E.out_cap);  // an overflow re-runs on the handle
        const u64 lo = (u64)w.idx * STR_EMIT_CHUNK, hi = min(n, lo + STR_EMIT_CHUNK);
        if (lo >= hi) continue;  // uniform across the block
        if (threadIdx.x == 0) s_run = q.str_chunk[w.idx];
        __syncthreads();
        // offsets: block-wide exclusive scan of the lengths, blockDim rows at a time
        for (u64 r0 = lo; r0 < hi; r0 += blockDim.x) {
            const u64 r = r0 + threadIdx.x;
            const long long x = r < hi ? q.str_lens[r] : 0;
            long long incl = x;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const long long y = __shfl_up_sync(FULL, incl, o);
                if (lane >= o) incl += y;
            }
            if (lane == 31) s_part[warp] = incl;
            __syncthreads();
            if (warp == 0) {
                const long long wv = lane < nwarps ? s_part[lane] : 0;
                long long wi = wv;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const long long y = __shfl_up_sync(FULL, wi, o);
                    if (lane >= o) wi += y;
                }
                if (lane < nwarps) s_part[lane] = wi - wv;
            }
            __syncthreads();
            const long long off = s_run + s_part[warp] + incl - x;
            if (r < hi) q.str_offs[r] = off;
            __syncthreads();
            if (threadIdx.x == blockDim.x - 1) s_run = off + x;
            __syncthreads();
        }
        // bytes: one thread per string (the id → ref → bytes chains of a
        // block's rows overlap); arena entries are 8-byte aligned and padded,
        // so the source is read in whole words
        const long long *ids = (const long long *)q.E.out[0];
        for (u64 r = lo + threadIdx.x; r < hi; r += blockDim.x) {
            const long long id = ids[r];
            if (id < 0) continue;
            const u64 ref = q.D.ref_by_id[id];
            const u32 len = (u32)(ref & 0xffffffu);
            const u64 *src = (const u64 *)(q.D.arena + (ref >> 24));
            uint8_t *dst = q.str_out + q.str_offs[r];
            for (u32 b = 0; b < len; b += 8) {
                const u64 x = src[b >> 3];
                const u32 m = min(8u, len - b);
                for (u32 j = 0; j < m; j++) dst[b + j] = (uint8_t)(x >> (8 * j));
            }
        }
        __syncthreads();
    }
}

// ================================================================== host
struct gb_batch {
    std::vector<gb_agg *> handles;
    std::vector<std::vector<gb_col>> cols;
    std::vector<u64> rows;
    DevBuf qdesc, items_init, items_str, items_ingest, items_compact, items_semit, str_queries, bctl, qctl;
    HostBuf qctl_host;
    u32 n_init = 0, n_str = 0, n_ingest = 0, n_compact = 0, n_semit = 0, n_strq = 0;
    u32 cls_off[BATCH_CLASSES] = {}, cls_n[BATCH_CLASSES] = {};  // ingest items per plan class
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool prepared = false;
    bool use_graph = true;
    int ctas_per_sm = 2;
    int smem_slots_max = 4096;
    int precombine = 1;  // 0 never, 1 per query (auto), 2 always
    bool profiling = false;
    int order = 0;  // 0 query-major tiles, 1 interleaved
    bool fast = true;  // register-resident integer tiles where the plan allows
    u32 tile_rows = BATCH_TILE;
    struct BatchProf {
        const char *name;
        cudaEvent_t a = nullptr, b = nullptr;
        bool pending = false;
        double ms = 0;
        u64 n = 0;
    } prof[4] = {{"k_batch_init"}, {"k_batch_strdict"}, {"k_batch_ingest"}, {"k_batch_compact"}};
    u64 launches = 0;
    std::vector<int> slow;  // queries re-run on their handle in the last run
    std::unordered_multimap<std::string, gb_agg *> pool;  // idle handles kept by gb_batch_clear
};

// The fast-path description of a query's plan (eligible = 0 when the plan
// has more than FAST_MAX_FILTERS predicates or an IN / VARCHAR predicate, a
// full-width pair key, floating-point ops or more than max_ops ops: such
// queries take the generic tile path).
static FastPlan make_fast_plan(const Plan &P, FastFilters &FF, int max_ops = BATCH_FAST_MAX_OPS) {
    FastPlan F;
    memset(&F, 0, sizeof F);
    memset(&FF, 0, sizeof FF);
    if (P.n_filters > FAST_MAX_FILTERS || P.key_mode == KEY_WIDE || P.n_ops > max_ops ||
        P.n_ops > FAST_MAX_OPS)
        return F;
    auto is_int = [](int t) { return t == GB_T_SMALLINT || t == GB_T_INTEGER || t == GB_T_BIGINT; };
    for (int k = 0; k < P.n_keys; k++)
        if (!is_int(P.cols[P.key_col[k]].type)) return F;
    const int nk = P.key_mode == KEY_PACKED ? 2 : 1;
    for (int k = 0; k < nk; k++) {
        F.kp[k] = P.cols[P.key_col[k]].data;
        F.kv[k] = P.cols[P.key_col[k]].valid;
    }
    const int t1 = nk == 2 ? P.cols[P.key_col[1]].type : 0;
    F.kdesc = (u32)P.key_mode | ((u32)P.cols[P.key_col[0]].type << 4) | ((u32)t1 << 8);
    if (P.key_mode == KEY_PACKED) F.kdesc |= ((u32)P.key_bits_b << 16) | ((u32)P.key_bits_a << 24);
    int sw = 1;
    for (int i = 0; i < P.n_ops; i++) {
        const Op &o = P.ops[i];
        const int t = P.cols[o.col].type;
        if (o.kind != OP_ADD_I && o.kind != OP_MIN_I && o.kind != OP_MAX_I && o.kind != OP_CNT_NN) return F;
        if (o.kind != OP_CNT_NN && !is_int(t)) return F;
        const bool wide = (o.kind == OP_MIN_I || o.kind == OP_MAX_I) && t == GB_T_BIGINT;
        if (wide && (sw & 1)) sw++;
        F.op[i] = (u32)o.kind | ((u32)(t & 15) << 4) | ((u32)o.word << 8) | ((u32)sw << 16) | ((u32)wide << 24);
        sw += (wide || o.kind == OP_ADD_I) ? 2 : 1;
        F.vp[i] = P.cols[o.col].data;
        F.vv[i] = P.cols[o.col].valid;
    }
    for (int j = 0; j < P.n_filters; j++) {
        const Filter &f = P.filters[j];
        const int t = P.cols[f.col].type;
        if ((!is_int(t) && t != GB_T_DOUBLE) || f.op > GB_CMP_GE) return F;  // IN / VARCHAR forms: generic path
        FF.fp[j] = P.cols[f.col].data;
        FF.fv[j] = P.cols[f.col].valid;
        if (t == GB_T_DOUBLE) memcpy(&FF.fk[j], &f.dc, 8);
        else FF.fk[j] = (u64)f.ic;
        FF.fdesc[j] = (u32)t | ((u32)f.op << 4);
    }
    F.n_filters = P.n_filters;
    F.nulls = (F.kv[0] || F.kv[1]) ? 1 : 0;
    for (int i = 0; i < P.n_ops; i++) F.nulls |= F.vv[i] ? 1 : 0;
    for (int j = 0; j < P.n_filters; j++) F.nulls |= FF.fv[j] ? 1 : 0;
    if (sw & 1) sw++;  // 8-byte aligned states (64-bit MIN/MAX words)
    F.swords = sw;
    F.n_ops = P.n_ops;
    F.eligible = 1;
    return F;
}

// ----------------------------------------------------- single-query fast ingest
// The hash ingest of one query whose plan compiles into registers (integer
// keys and ops, up to FAST_MAX_OPS ops and FAST_MAX_FILTERS numeric
// predicates): the batch's fast tile path as a persistent kernel over the
// query's tiles, with one narrow shared table per CTA for the whole launch
// and spill records instead of re-runs.  Same tile-claim / spill-threshold
// protocol as k_ingest, so run_ingest drives both.
template <bool PRE, int NOPS, bool NULLS, bool FILT>
__global__ void __launch_bounds__(512, 2)
    k_ingest_fast(const __grid_constant__ Plan P, const __grid_constant__ FastPlan F,
                  const __grid_constant__ FastFilters FF, const TableRef T, const IngestArgs A) {
    extern __shared__ u64 bsm[];
    __shared__ u32 s_tile, s_new;
    const int S = A.smem_slots;
    u64 *keys = bsm;
    u32 *st = (u32 *)(bsm + S);
    if (threadIdx.x == 0) s_new = 0;
    fast_smem_init<NOPS>(F, keys, st, S);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const u64 step = (u64)(blockDim.x >> 5) * 32;
    for (;;) {
        if (threadIdx.x == 0) {
            u32 t = ~0u;
            if (*(volatile u32 *)&T.ctl->stop == 0) {
                const u32 c = atomicAdd(&T.ctl->tile_counter, 1u);
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
        u64 base = t0 + (u64)warp * 32;
        FastRaw<NOPS, FILT> cur, nxt;
        fast_fetch<NOPS, NULLS, FILT>(F, FF, base + lane, t1, cur);
        for (; base < t1; base += step) {
            fast_fetch<NOPS, NULLS, FILT>(F, FF, base + step + lane, t1, nxt);
            fast_rows<PRE, NOPS, FILT, true>(F, FF, T, keys, st, S, cur, &s_new, &P);
            cur = nxt;
        }
        if (threadIdx.x == 0 && *(volatile u32 *)&T.ctl->spill_count > T.spill_threshold)
            atomicExch(&T.ctl->stop, 1u);
    }
    __syncthreads();
    fast_smem_flush<NOPS, true>(F, T, keys, st, S, &s_new, &P);
    __syncthreads();
    if (threadIdx.x == 0 && s_new) atomicAdd(&T.ctl->n_groups, s_new);
}

typedef void (*FastIngestKernel)(Plan, FastPlan, FastFilters, TableRef, IngestArgs);

#define GB_FI4(PRE_, N_)                                                                        \
    {                                                                                           \
        {k_ingest_fast<PRE_, N_, false, false>, k_ingest_fast<PRE_, N_, false, true>},          \
        {                                                                                       \
            k_ingest_fast<PRE_, N_, true, false>, k_ingest_fast<PRE_, N_, true, true>           \
        }                                                                                       \
    }

static FastIngestKernel fast_ingest_kernel(int pre, int nops, int nulls, int filt) {
    static const FastIngestKernel tab[2][FAST_MAX_OPS + 1][2][2] = {
        {GB_FI4(false, 0), GB_FI4(false, 1), GB_FI4(false, 2), GB_FI4(false, 3), GB_FI4(false, 4)},
        {GB_FI4(true, 0), GB_FI4(true, 1), GB_FI4(true, 2), GB_FI4(true, 3), GB_FI4(true, 4)},
    };
    return tab[pre][nops][nulls][filt];
}
#undef GB_FI4

static gb_status launch_ingest_fast(gb_agg *h, const TableRef &T, IngestArgs A, int grid, cudaStream_t st,
                                    bool *launched) {
    *launched = false;
    if (!h->fast_ingest || h->plan.n_dist || h->plan.str_key >= 0) return GB_OK;
    FastFilters FF;
    const FastPlan F = make_fast_plan(h->plan, FF, FAST_MAX_OPS);
    if (!F.eligible) return GB_OK;
    // the shared table pays when the estimated groups fit it; otherwise rows
    // go straight to the HBM table (no probe of a full shared table)
    const int S = h->est_groups <= (u64)A.smem_slots ? A.smem_slots : 0;
    // narrow shared atomics beat the warp key match; without a shared table,
    // few groups mean hot HBM slots, which the match relieves
    const bool pre = h->precombine_set ? h->precombine : (S == 0 && h->est_groups <= 4096);
    A.smem_slots = S;
    const size_t smem = (size_t)S * (8 + 4 * (size_t)F.swords);
    static bool attr_set = false;
    if (!attr_set) {
        for (int a = 0; a < 2; a++)
            for (int n = 0; n <= FAST_MAX_OPS; n++)
                for (int u = 0; u < 2; u++)
                    for (int f = 0; f < 2; f++)
                        GB_CUDA(cudaFuncSetAttribute(fast_ingest_kernel(a, n, u, f),
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        attr_set = true;
    }
    {
        ProfScope ps(h, "k_ingest_fast", st);
        fast_ingest_kernel(pre, F.n_ops, F.nulls != 0, F.n_filters != 0)<<<grid, 512, smem, st>>>(h->plan, F, FF, T,
                                                                                                   A);
    }
    GB_CUDA(cudaGetLastError());
    *launched = true;
    return GB_OK;
}

// Dynamic shared memory of one k_batch_ingest CTA so that `ctas` CTAs fit on
// an SM (about 227 KB usable per SM, less each CTA's static shared memory).
static int batch_smem_bytes(int ctas) {
    int b = (227 * 1024) / std::max(1, ctas) - 4096;
    b = std::min(b, 96 * 1024);
    return b & ~4095;
}

static gb_status batch_prepare(gb_batch *b, cudaStream_t st) {
    const u32 nq = (u32)b->handles.size();
    std::vector<BQuery> qs(nq);
    std::vector<BItem> it_init, it_str, it_ing, it_cmp, it_semit;
    std::vector<u32> strq;
    gb_status s;
    if ((s = b->qctl.ensure((size_t)nq * sizeof(Ctl) + 64)) || (s = b->bctl.ensure(BATCH_CLASSES * sizeof(Ctl))) ||
        (s = b->qctl_host.ensure((size_t)nq * sizeof(Ctl) + 64)))
        return s;
    for (u32 q = 0; q < nq; q++) {
        gb_agg *h = b->handles[q];
        const u64 n = b->rows[q];
        const int nc = (int)h->col_types.size();
        for (int c = 0; c < nc; c++) {
            h->plan.cols[c].data = b->cols[q][c].data;
            h->plan.cols[c].valid = b->cols[q][c].validity;
            h->plan.cols[c].offsets = b->cols[q][c].offsets;
        }
        BQuery &d = qs[q];
        memset(&d, 0, sizeof d);
        d.n_rows = n;
        d.is_str = h->str_col >= 0;
        if (d.is_str) {
            // dictionary and arena sized for the whole query: no growth in the graph
            const gb_col &sc = b->cols[q][h->str_col];
            int64_t ends[2];
            GB_CUDA(cudaMemcpy(&ends[0], sc.offsets, 8, cudaMemcpyDeviceToHost));
            GB_CUDA(cudaMemcpy(&ends[1], sc.offsets + n, 8, cudaMemcpyDeviceToHost));
            u64 cap = 1024;
            while (cap < 2 * std::max<u64>(h->est_groups, 512)) cap <<= 1;
            cap = std::max(cap, h->sd_cap);  // a re-run on the handle may have grown it
            if ((s = strdict_init(h, cap, st))) return s;
            // arena entries are padded to 8 bytes: at most 7 more per non-empty string
            const u64 sbytes = (u64)(ends[1] - ends[0]);
            const u64 need = sbytes + 7 * std::min<u64>(n, sbytes) + 64;
            if (h->sd_arena_cap < need) {
                if ((s = h->sd_arena.ensure(need))) return s;
                h->sd_arena_cap = need;
            }
            if ((s = h->sd_ids.ensure(n * 8 + 8))) return s;
            h->plan.cols[nc].data = h->sd_ids.p;
            h->plan.cols[nc].valid = nullptr;
            d.D = strdict_ref(h);
            d.sbytes = (const uint8_t *)sc.data;
            d.soffs = sc.offsets;
            d.svalid = sc.validity;
            d.ids = (long long *)h->sd_ids.p;
            for (u64 c = 0; c * 8192 < n; c++) it_str.push_back({q, (u32)c});
        }
        // HBM table, spill buffer, outputs of the handle
        const int words = h->plan.words;
        const u64 need_spill = (1u << 16) + 4096;
        if (h->spill_cap < need_spill) {
            if ((s = h->spill.ensure((size_t)need_spill * (1 + words) * 8))) return s;
            h->spill_cap = (u32)need_spill;
        }
        if ((s = alloc_outputs(h, h->cap + 2))) return s;
        if (h->plan.n_dist) {
            // pair sets for this query's rows, emptied by the batch's init
            h->dpairs = 0;
            if ((s = dist_reserve(h, n, st))) return s;
        }
        d.P = h->plan;
        if (b->fast) d.F = make_fast_plan(h->plan, d.FF);
        d.T = table_ref(h);
        d.T.ctl = (Ctl *)b->qctl.p + q;
        d.T.spill_threshold = h->spill_cap / 2;
        fill_emit(h, d.E, h->out_cols, h->out_valid, h->out_cap);
        d.table_words = (h->cap + 2) * (u64)h->plan.stride;
        d.smem_slots = h->mode == 0 ? std::min(h->smem_slots, b->smem_slots_max) : 0;
        if (d.F.eligible) {
            // narrow shared states: as many slots as fit, used when the
            // estimated groups fit in them (else rows go straight to HBM)
            const int per = 8 + 4 * d.F.swords;
            int S = 1;
            while (S * 2 * per <= batch_smem_bytes(b->ctas_per_sm)) S *= 2;
            S = std::min(S, b->smem_slots_max);
            d.smem_slots = h->est_groups <= (u64)S ? S : 0;
            // narrow shared atomics beat the warp key match; without a shared
            // table, few groups mean hot HBM slots, which the match relieves
            d.pre = b->precombine == 2 || (b->precombine == 1 && d.smem_slots == 0 && h->est_groups <= 4096);
        } else if (h->est_groups > (u64)d.smem_slots) {
            d.smem_slots = 0;  // a shared table only pays when the estimated groups fit it
        }
        d.init_words = d.table_words + (u64)(d.E.n_keys + d.E.n_aggs) * ((d.E.out_cap + 63) / 64) +
                       (d.is_str ? 2 * d.D.cap + 8 : 0);
        if (h->plan.n_dist) {
            const u64 sw = (h->plan.dmask + 1) * (h->plan.dnarrow ? 1 : 2) * (u64)h->plan.n_dist;
            d.init_words += sw * (h->plan.null_sets ? 2 : 1) + 2 + GB_MAX_DISTINCT;
        }
        for (u64 c = 0; c * 65536 < d.init_words; c++) it_init.push_back({q, (u32)c});
        d.tile_rows = b->tile_rows;
        for (u64 c = 0; c * b->tile_rows < n; c++) it_ing.push_back({q, (u32)c});
        for (u64 c = 0; c * (COMPACT_PER * 256) < h->cap + 2; c++) it_cmp.push_back({q, (u32)c});
        if (d.is_str) {
            // string results for up to out_cap groups; their bytes are at most
            // the dictionary arena's (each distinct string is stored once)
            const u64 nch = (h->out_cap + STR_EMIT_CHUNK - 1) / STR_EMIT_CHUNK;
            if ((s = h->str_lens.ensure(h->out_cap * 8 + 8)) || (s = h->out_str_offs.ensure(h->out_cap * 8 + 16)) ||
                (s = h->out_str_bytes.ensure(h->sd_arena_cap + 16)) || (s = h->scan_tmp.ensure(nch * 8 + 16)))
                return s;
            d.str_lens = (int64_t *)h->str_lens.p;
            d.str_offs = (int64_t *)h->out_str_offs.p;
            d.str_out = (uint8_t *)h->out_str_bytes.p;
            d.str_chunk = (int64_t *)h->scan_tmp.p;
            for (u64 c = 0; c < nch; c++) it_semit.push_back({q, (u32)c});
            strq.push_back(q);
        }
    }
    // Tile order: query-major by default (the CTAs sweep one query's table
    // at a time, which keeps it in L2); "order" 1 interleaves the queries.
    std::vector<BItem> mixed;
    mixed.reserve(it_ing.size());
    if (b->order == 1) {
        std::vector<std::vector<BItem>> per(nq);
        for (auto &x : it_ing) per[x.q].push_back(x);
        size_t k = 0;
        bool any = true;
        while (any) {
            any = false;
            for (u32 q = 0; q < nq; q++)
                if (k < per[q].size()) {
                    mixed.push_back(per[q][k]);
                    any = true;
                }
            k++;
        }
    }
    if (b->order == 1) it_ing.swap(mixed);
    // group the items by plan class (one persistent kernel per class)
    {
        std::vector<int> qcls(nq);
        for (u32 q = 0; q < nq; q++) {
            const BQuery &d = qs[q];
            qcls[q] = d.F.eligible ? 2 + (d.pre ? 12 : 0) + d.F.n_ops * 4 + d.F.nulls * 2 + (d.F.n_filters ? 1 : 0)
                                   : (b->precombine ? 1 : 0);
        }
        std::vector<std::vector<BItem>> per(BATCH_CLASSES);
        for (auto &x : it_ing) per[qcls[x.q]].push_back(x);
        it_ing.clear();
        for (int c = 0; c < BATCH_CLASSES; c++) {
            b->cls_off[c] = (u32)it_ing.size();
            b->cls_n[c] = (u32)per[c].size();
            it_ing.insert(it_ing.end(), per[c].begin(), per[c].end());
        }
    }
    if ((s = b->qdesc.ensure(qs.size() * sizeof(BQuery) + 64)) ||
        (s = b->items_init.ensure(it_init.size() * sizeof(BItem) + 64)) ||
        (s = b->items_str.ensure(it_str.size() * sizeof(BItem) + 64)) ||
        (s = b->items_ingest.ensure(it_ing.size() * sizeof(BItem) + 64)) ||
        (s = b->items_compact.ensure(it_cmp.size() * sizeof(BItem) + 64)) ||
        (s = b->items_semit.ensure(it_semit.size() * sizeof(BItem) + 64)) ||
        (s = b->str_queries.ensure(strq.size() * sizeof(u32) + 64)))
        return s;
    GB_CUDA(cudaMemcpy(b->qdesc.p, qs.data(), qs.size() * sizeof(BQuery), cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemcpy(b->items_init.p, it_init.data(), it_init.size() * sizeof(BItem), cudaMemcpyHostToDevice));
    if (!it_str.empty())
        GB_CUDA(cudaMemcpy(b->items_str.p, it_str.data(), it_str.size() * sizeof(BItem), cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemcpy(b->items_ingest.p, it_ing.data(), it_ing.size() * sizeof(BItem), cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemcpy(b->items_compact.p, it_cmp.data(), it_cmp.size() * sizeof(BItem), cudaMemcpyHostToDevice));
    if (!strq.empty()) {
        GB_CUDA(cudaMemcpy(b->items_semit.p, it_semit.data(), it_semit.size() * sizeof(BItem), cudaMemcpyHostToDevice));
        GB_CUDA(cudaMemcpy(b->str_queries.p, strq.data(), strq.size() * sizeof(u32), cudaMemcpyHostToDevice));
    }
    b->n_semit = (u32)it_semit.size();
    b->n_strq = (u32)strq.size();
    b->n_init = (u32)it_init.size();
    b->n_str = (u32)it_str.size();
    b->n_ingest = (u32)it_ing.size();
    b->n_compact = (u32)it_cmp.size();
    static bool attr = false;
    if (!attr) {
        for (int c = 0; c < BATCH_CLASSES; c++)
            cudaFuncSetAttribute(batch_kernel(c), cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
        attr = true;
    }
    b->prepared = true;
    return GB_OK;
}


// Profiling (graph off): events around each of the four kernels.
using BatchProf = gb_batch::BatchProf;

static void batch_prof(gb_batch *b, int i, cudaStream_t st, bool begin) {
    if (!b->profiling) return;
    BatchProf &p = b->prof[i];
    if (!p.a) {
        cudaEventCreate(&p.a);
        cudaEventCreate(&p.b);
    }
    cudaEventRecord(begin ? p.a : p.b, st);
    if (!begin) p.pending = true;
}

static void batch_prof_collect(gb_batch *b) {
    for (auto &p : b->prof) {
        if (!p.pending) continue;
        float ms = 0;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            p.ms += ms;
            p.n++;
        } else {
            (void)cudaGetLastError();  // leave no sticky error behind
        }
        p.pending = false;
    }
}

// The graph body: every launch of one batch execution.
static gb_status batch_enqueue(gb_batch *b, cudaStream_t st) {
    const u32 nq = (u32)b->handles.size();
    const int sms = sm_count();
    GB_CUDA(cudaMemsetAsync(b->qctl.p, 0, (size_t)nq * sizeof(Ctl), st));
    GB_CUDA(cudaMemsetAsync(b->bctl.p, 0, BATCH_CLASSES * sizeof(Ctl), st));
    batch_prof(b, 0, st, true);
    k_batch_init<<<std::max(1, std::min((int)b->n_init, sms * 8)), 256, 0, st>>>((const BQuery *)b->qdesc.p,
                                                                               (const BItem *)b->items_init.p, b->n_init);
    GB_CUDA(cudaGetLastError());
    batch_prof(b, 0, st, false);
    if (b->n_str) {
        batch_prof(b, 1, st, true);
        k_batch_strdict<<<std::min((int)b->n_str, sms * 8), 256, 0, st>>>((const BQuery *)b->qdesc.p,
                                                                       (const BItem *)b->items_str.p, b->n_str);
        GB_CUDA(cudaGetLastError());
        batch_prof(b, 1, st, false);
    }
    const int smem_bytes = batch_smem_bytes(b->ctas_per_sm);
    batch_prof(b, 2, st, true);
    for (int c = 0; c < BATCH_CLASSES; c++) {
        if (!b->cls_n[c]) continue;
        const int grid = std::max(1, std::min((int)b->cls_n[c], sms * b->ctas_per_sm));
        batch_kernel(c)<<<grid, 512, smem_bytes, st>>>((const BQuery *)b->qdesc.p,
                                                      (const BItem *)b->items_ingest.p + b->cls_off[c], b->cls_n[c],
                                                      (Ctl *)b->bctl.p + c, smem_bytes);
        GB_CUDA(cudaGetLastError());
    }
    batch_prof(b, 2, st, false);
    batch_prof(b, 3, st, true);
    k_batch_compact<<<std::max(1, std::min((int)b->n_compact, sms * 8)), 256, 0, st>>>(
        (const BQuery *)b->qdesc.p, (const BItem *)b->items_compact.p, b->n_compact);
    GB_CUDA(cudaGetLastError());
    if (b->n_strq) {
        const BQuery *qd = (const BQuery *)b->qdesc.p;
        const BItem *si = (const BItem *)b->items_semit.p;
        const int g = std::max(1, std::min((int)b->n_semit, sms * 8));
        k_batch_str_len<<<g, 256, 0, st>>>(qd, si, b->n_semit);
        k_batch_str_scan<<<std::min((int)b->n_strq, sms * 4), 1024, 0, st>>>(qd, (const u32 *)b->str_queries.p,
                                                                            b->n_strq);
        k_batch_str_gather<<<g, 256, 0, st>>>(qd, si, b->n_semit);
        GB_CUDA(cudaGetLastError());
    }
    batch_prof(b, 3, st, false);
    GB_CUDA(cudaMemcpyAsync(b->qctl_host.p, b->qctl.p, (size_t)nq * sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    return GB_OK;
}

static gb_status cuda_sync_legacy() {
    GB_CUDA(cudaStreamSynchronize(0));
    return GB_OK;
}

// Pool key of a handle: its plan shape (without the filter constants) and
// the table capacity its estimate gives.
static std::string batch_pool_key(const gb_agg_spec &sp) {
    std::string k;
    auto put = [&](const void *p, size_t n) { k.append((const char *)p, n); };
    put(&sp.n_cols, 4);
    put(sp.col_types, 4 * sp.n_cols);
    put(&sp.n_groups, 4);
    put(sp.group_cols, 4 * sp.n_groups);
    put(&sp.n_aggs, 4);
    put(sp.aggs, sizeof(gb_agg_desc) * sp.n_aggs);
    put(&sp.n_filters, 4);
    for (uint32_t i = 0; i < sp.n_filters; i++) {
        put(&sp.filters[i].col, 4);
        put(&sp.filters[i].op, 4);
    }
    put(&sp.nullable_mask, 8);
    const u64 cap = std::max<u64>(1024, next_pow2(sp.est_groups * 2));
    put(&cap, 8);
    return k;
}

static std::string batch_pool_key(const gb_agg *h) {
    gb_agg_spec sp{};
    sp.n_cols = (uint32_t)h->col_types.size();
    sp.col_types = h->col_types.data();
    sp.n_groups = (uint32_t)h->group_cols.size();
    sp.group_cols = h->group_cols.data();
    sp.n_aggs = (uint32_t)h->aggs.size();
    sp.aggs = h->aggs.data();
    sp.n_filters = (uint32_t)h->filters.size();
    sp.filters = h->filters.data();
    sp.nullable_mask = h->nullable_mask;
    sp.est_groups = h->cap / 2;
    return batch_pool_key(sp);
}

constexpr size_t BATCH_POOL_MAX = 4096;

extern "C" {

gb_status gb_batch_clear(gb_batch *b) {
    if (!b) return GB_ERR_INVALID;
    cudaDeviceSynchronize();
    for (auto *h : b->handles) {
        if (b->pool.size() >= BATCH_POOL_MAX) {
            gb_agg_destroy(h);
            continue;
        }
        b->pool.emplace(batch_pool_key(h), h);
    }
    b->handles.clear();
    b->cols.clear();
    b->rows.clear();
    b->slow.clear();
    b->prepared = false;
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    return GB_OK;
}

gb_status gb_batch_create(gb_batch **out) {
    if (!out) return GB_ERR_INVALID;
    *out = new gb_batch();
    return GB_OK;
}

gb_status gb_batch_add(gb_batch *b, const gb_agg_spec *spec, const gb_col *cols, uint64_t nrows, uint32_t *qidx) {
    if (!b || !spec || (!cols && nrows)) return GB_ERR_INVALID;
    if (spec->n_groups == 2 && spec->group_cols && spec->col_types)
        for (uint32_t g = 0; g < 2; g++)
            if (spec->group_cols[g] >= 0 && (uint32_t)spec->group_cols[g] < spec->n_cols &&
                spec->col_types[spec->group_cols[g]] == GB_T_VARCHAR) {
                set_error("a VARCHAR in a pair key runs on its own handle (gb_agg_*), not in a batch");
                return GB_ERR_UNSUPPORTED;
            }
    // a table never has more groups than rows: size it for min(estimate, rows)
    gb_agg_spec sp = *spec;
    const u64 est = sp.est_groups ? sp.est_groups : (1u << 15);
    sp.est_groups = std::max<u64>(1, std::min<u64>(est, nrows));
    gb_agg *h = nullptr;
    gb_status s;
    const std::string key = batch_pool_key(sp);
    auto it = b->pool.find(key);
    if (it != b->pool.end()) {
        // an idle handle of the same plan shape and table size: rebind it
        h = it->second;
        b->pool.erase(it);
        h->filters.assign(sp.filters, sp.filters + sp.n_filters);
        if ((s = compile_filters(h))) {
            gb_agg_destroy(h);
            return s;
        }
        h->est_groups = sp.est_groups;
        h->finalized = h->has_result = h->topn_applied = false;
        h->rows_ingested = h->n_groups = h->n_rows_out = h->launches = 0;
        b->handles.push_back(h);
        b->cols.emplace_back(cols, cols + spec->n_cols);
        b->rows.push_back(nrows);
        b->prepared = false;
        if (b->exec) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
        if (qidx) *qidx = (uint32_t)(b->handles.size() - 1);
        return GB_OK;
    }
    if ((s = gb_agg_create(&sp, &h))) return s;
    if (h->mode == 1) {  // the batch runs the hash pipeline for every query
        h->mode = 0;
        u64 est = h->est_groups ? h->est_groups : (1u << 15);
        h->cap = std::max<u64>(1024, next_pow2(est * 2));
        if ((s = init_table(h, h->table, h->cap, 0)) || (s = cuda_sync_legacy())) {
            gb_agg_destroy(h);
            return s;
        }
    }
    b->handles.push_back(h);
    b->cols.emplace_back(cols, cols + spec->n_cols);
    b->rows.push_back(nrows);
    b->prepared = false;
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (qidx) *qidx = (uint32_t)(b->handles.size() - 1);
    return GB_OK;
}

gb_status gb_batch_set_option(gb_batch *b, const char *name, int64_t value) {
    if (!b || !name) return GB_ERR_INVALID;
    std::string n(name);
    if (n == "graph") b->use_graph = value != 0;
    else if (n == "ctas_per_sm" && value >= 1 && value <= 4) b->ctas_per_sm = (int)value;
    else if (n == "smem_slots" && value >= 0 && value <= 4096 && !(value & (value - 1))) b->smem_slots_max = (int)value;
    else if (n == "precombine" && value >= 0 && value <= 2) {
        b->precombine = (int)value;
        b->prepared = false;
    }
    else if (n == "profiling") b->profiling = value != 0;
    else if (n == "tile_rows" && value >= 1024 && value <= (1 << 20) && !(value & (value - 1))) {
        b->tile_rows = (u32)value;
        b->prepared = false;
    } else if (n == "fast") {
        b->fast = value != 0;
        b->prepared = false;
    }
    else if (n == "order" && (value == 0 || value == 1)) {
        b->order = (int)value;
        b->prepared = false;
    }
    else {
        set_error("unknown or invalid batch option '%s'", name);
        return GB_ERR_INVALID;
    }
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    return GB_OK;
}

gb_status gb_batch_run(gb_batch *b, void *stream) {
    if (!b) return GB_ERR_INVALID;
    cudaStream_t st = (cudaStream_t)stream;
    gb_status s;
    if (!b->prepared && (s = batch_prepare(b, st))) return s;
    const u32 nq = (u32)b->handles.size();
    if (b->use_graph && !b->profiling) {
        if (!b->exec) {
            cudaStream_t cs;
            GB_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
            GB_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
            gb_status es = batch_enqueue(b, cs);
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(cs, &g);
            cudaStreamDestroy(cs);
            if (es) return es;
            if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
            if (b->graph) cudaGraphDestroy(b->graph);
            b->graph = g;
            GB_CUDA(cudaGraphInstantiate(&b->exec, g, 0));
        }
        GB_CUDA(cudaGraphLaunch(b->exec, st));
    } else {
        if ((s = batch_enqueue(b, st))) return s;
    }
    u32 ncls = 0;
    for (int c = 0; c < BATCH_CLASSES; c++) ncls += b->cls_n[c] ? 1 : 0;
    b->launches += 2 + ncls + (b->n_str ? 1 : 0) + (b->n_strq ? 3 : 0);
    GB_CUDA(cudaStreamSynchronize(st));
    batch_prof_collect(b);
    const Ctl *qc = (const Ctl *)b->qctl_host.p;
    b->slow.clear();
    for (u32 q = 0; q < nq; q++) {
        gb_agg *h = b->handles[q];
        const Ctl &c = qc[q];
        bool bad = c.spill_count || c.err || c.aux1 || c.out_count > h->out_cap;
        if (!bad && h->plan.n_dist) {  // the pair sets' counters
            GB_CUDA(cudaMemcpy(h->dmeta_host, h->dmeta.p, sizeof(h->dmeta_host), cudaMemcpyDeviceToHost));
            bad = h->dmeta_host[1] != 0;
            h->dpairs = h->dmeta_host[0];
        }
        if (bad) {
            // host decisions needed (spill / dictionary growth): the whole query
            // re-runs on its own handle
            b->slow.push_back((int)q);
            if ((s = gb_agg_reset(h))) return s;
            if ((s = gb_agg_ingest(h, b->cols[q].data(), b->rows[q], GB_MEM_DEVICE, stream))) return s;
            if ((s = gb_agg_finalize(h, stream))) return s;
            continue;
        }
        h->n_groups = c.n_groups;
        h->n_rows_out = c.out_count;
        h->topn_applied = false;
        h->finalized = true;
        h->has_result = false;  // a VARCHAR key's strings were emitted inside the batch
    }
    if (b->handles.size() && b->slow.size() < nq) GB_CUDA(cudaStreamSynchronize(st));
    if (!b->slow.empty()) {
        // a re-run may have grown tables / dictionaries: the next run prepares
        // (and captures) again with the new sizes
        b->prepared = false;
        if (b->exec) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
    }
    return GB_OK;
}

uint32_t gb_batch_size(const gb_batch *b) { return b ? (uint32_t)b->handles.size() : 0; }

gb_status gb_batch_result(gb_batch *b, uint32_t q, gb_result *out) {
    if (!b || q >= b->handles.size()) return GB_ERR_INVALID;
    return gb_agg_result(b->handles[q], out);
}

gb_status gb_batch_result_device(gb_batch *b, uint32_t q, gb_result *out) {
    if (!b || q >= b->handles.size()) return GB_ERR_INVALID;
    return gb_agg_result_device(b->handles[q], out);
}

uint32_t gb_batch_slow_queries(const gb_batch *b) { return b ? (uint32_t)b->slow.size() : 0; }

uint64_t gb_batch_kernel_launches(const gb_batch *b) { return b ? b->launches : 0; }

uint32_t gb_batch_profile(const gb_batch *b, gb_kernel_stat *out, uint32_t max) {
    if (!b) return 0;
    uint32_t n = 0;
    for (const auto &p : b->prof) {
        if (!p.n) continue;
        if (out && n < max) {
            memset(&out[n], 0, sizeof out[n]);
            strncpy(out[n].name, p.name, sizeof(out[n].name) - 1);
            out[n].launches = p.n;
            out[n].ms = p.ms;
        }
        n++;
    }
    return n;
}

void gb_batch_destroy(gb_batch *b) {
    if (!b) return;
    cudaDeviceSynchronize();
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (auto &p : b->prof) {
        if (p.a) cudaEventDestroy(p.a);
        if (p.b) cudaEventDestroy(p.b);
    }
    for (auto *h : b->handles) gb_agg_destroy(h);
    for (auto &e : b->pool) gb_agg_destroy(e.second);
    for (DevBuf *d : {&b->qdesc, &b->items_init, &b->items_str, &b->items_ingest, &b->items_compact, &b->items_semit,
                      &b->str_queries, &b->bctl, &b->qctl})
        d->release();
    b->qctl_host.release();
    delete b;
}

}  // extern "C"
