// gb_noalloc.cu — an allocation-free GROUP BY entry point.
//
// Some callers cannot allocate device memory on their query path: an engine
// that reserved its whole device budget up front and hands out memory only
// from its own arena, a plugin host that forbids allocation inside operator
// calls, or a latency-sensitive path where cudaMalloc/cudaFree would
// implicitly synchronise the device and stall other streams.  For them,
// gb_hash_aggregate_noalloc() runs the same hash-aggregation kernel as
// gb_agg_* but keeps all of its scratch (hash table, control words, spill
// area) in file-scope __device__ arrays of fixed size, so a call allocates
// nothing: the caller passes device input and output buffers only.
//
// Limits: at most GB_NOALLOC_MAX_GROUPS distinct keys (the table has twice
// as many slots) and at most 2^31 rows per call.  The scratch lives in every
// GPU that loads the library until the process exits (about 8.1 MiB).
// All calls share the scratch: each call clears it first, so it keeps the
// previous call's contents only until the next call starts; calls whose
// work overlaps on the GPU (different streams, or host threads racing)
// corrupt each other's results and must be serialised by the caller.
#include <algorithm>
#include <mutex>

#include "gb_kernels.cuh"

namespace gb {
namespace noalloc {

constexpr u64 kCap = 1ull << 18;            // table slots
constexpr u64 kMaxGroups = kCap / 2;        // = GB_NOALLOC_MAX_GROUPS
constexpr int kStride = 4;                  // key, count, sum, pad
constexpr int kWords = 2;                   // count, sum
constexpr u32 kSpillCap = 4096;             // records of 1 + kWords words

static __device__ __align__(256) u64 g_table[(kCap + 2) * kStride];
static __device__ __align__(256) Ctl g_ctl;
static __device__ __align__(256) u64 g_spill[(u64)kSpillCap * (1 + kWords)];

struct DevScratch {
    u64 *table = nullptr;
    Ctl *ctl = nullptr;
    u64 *spill = nullptr;
};

// Device addresses of the scratch arrays, resolved once per device (the host
// names g_table etc. are host-side stand-ins, not device addresses).
static std::mutex g_mu;
static DevScratch g_addr[64];
static bool g_ready[64];

static gb_status scratch_for_current_device(DevScratch *out) {
    int dev = 0;
    GB_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("device ordinal %d out of range", dev);
        return GB_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_ready[dev]) {
        DevScratch s;
        GB_CUDA(cudaGetSymbolAddress((void **)&s.table, g_table));
        GB_CUDA(cudaGetSymbolAddress((void **)&s.ctl, g_ctl));
        GB_CUDA(cudaGetSymbolAddress((void **)&s.spill, g_spill));
        g_addr[dev] = s;
        g_ready[dev] = true;
    }
    *out = g_addr[dev];
    return GB_OK;
}

__global__ void k_clear(u64 *table, Ctl *ctl) {
    const u64 total = (kCap + 2) * kStride;
    for (u64 i = blockIdx.x * (u64)blockDim.x + threadIdx.x; i < total; i += (u64)gridDim.x * blockDim.x)
        table[i] = (i % kStride == 0) ? EMPTY_KEY : 0ull;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctl->n_groups = 0;
        ctl->spill_count = 0;
        ctl->tile_counter = 0;
        ctl->stop = 0;
        ctl->err = 0;
        ctl->out_count = 0;
    }
}

// Variant of the persistent ingest kernel: grid-stride over rows (no tile
// queue, no stop protocol) with the shared-memory pre-aggregation table and
// the fixed-size HBM table of this file.
__global__ void __launch_bounds__(512) k_ingest_noalloc(const __grid_constant__ Plan P, const TableRef T, u64 n,
                                                        int smem_slots) {
    extern __shared__ u64 smem[];
    __shared__ u32 s_new;
    SmemTable sm;
    sm.S = smem_slots;
    sm.probe = 8;
    sm.keys = smem;
    sm.st = smem + sm.S;
    if (threadIdx.x == 0) s_new = 0;
    smem_init(P, sm);
    __syncthreads();
    const int warp = threadIdx.x >> 5;
    const u64 warps_total = (u64)gridDim.x * (blockDim.x >> 5);
    for (u64 base = ((u64)blockIdx.x * (blockDim.x >> 5) + warp) * 32; base < n; base += warps_total * 32)
        warp_rows<true>(P, T, sm, base, n, &s_new, nullptr);  // COUNT and SUM only: no OP_DIST
    __syncthreads();
    smem_flush(P, T, sm, &s_new);
    __syncthreads();
    if (threadIdx.x == 0 && s_new) atomicAdd(&T.ctl->n_groups, s_new);
}

// Records the ingest spilled (a probe run longer than the bound: keys whose
// hashes cluster) fold into the table with an unbounded probe: at most
// kMaxGroups keys fill at most half of its kCap slots, so a free slot is
// always found.  Records beyond the spill area were lost and the call is
// refused (ERR_SPILL_OVERFLOW).
__global__ void k_merge_noalloc(const __grid_constant__ Plan P, const TableRef T) {
    __shared__ u32 s_new;  // new groups of this block (g_slot counts with a shared-memory atomic)
    if (threadIdx.x == 0) s_new = 0;
    __syncthreads();
    const u32 n = min(*(volatile u32 *)&T.ctl->spill_count, T.spill_cap);
    TableRef U = T;
    U.gmax_probe = (int32_t)kCap;
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const u64 *rec = T.spill + (u64)i * (1 + kWords);
        const long long s = g_slot(U, rec[0], mix64(rec[0]), &s_new);
        if (s < 0) {  // cannot happen below the limit (a free slot exists)
            atomicOr(&T.ctl->err, (u32)ERR_SPILL_OVERFLOW);
            continue;
        }
        u64 v[GB_MAX_OPS] = {rec[2]};
        apply_state(P, T.slots + (u64)s * (u64)T.stride + 1, rec[1], v);
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_new) atomicAdd(&T.ctl->n_groups, s_new);
}

__global__ void k_emit_noalloc(const u64 *table, Ctl *ctl, int64_t *out_keys, int64_t *out_sums,
                               int64_t *out_counts, u64 out_cap) {
    const int lane = threadIdx.x & 31;
    const u64 total = kCap + 2;
    for (u64 base = blockIdx.x * (u64)blockDim.x + threadIdx.x - lane; base < total;
         base += (u64)gridDim.x * blockDim.x) {
        const u64 s = base + lane;
        bool occ = false;
        const u64 *sl = table + s * kStride;
        if (s < kCap) occ = sl[0] != EMPTY_KEY;
        else if (s < total) occ = sl[1] != 0;
        const unsigned m = __ballot_sync(FULL, occ);
        if (m == 0) continue;
        u32 wbase = 0;
        if (lane == 0) wbase = atomicAdd(&ctl->out_count, (u32)__popc(m));
        wbase = __shfl_sync(FULL, wbase, 0);
        if (!occ) continue;
        const u64 o = wbase + __popc(m & ((1u << lane) - 1u));
        if (o >= out_cap) {
            atomicOr(&ctl->err, (u32)ERR_OUT_OVERFLOW);
            continue;
        }
        out_keys[o] = (s < kCap) ? (int64_t)sl[0] : (int64_t)EMPTY_KEY;
        out_counts[o] = (int64_t)sl[1];
        out_sums[o] = (int64_t)sl[2];
    }
}

}  // namespace noalloc
}  // namespace gb

using namespace gb;

extern "C" gb_status gb_hash_aggregate_noalloc(const int64_t *keys, const int64_t *values, uint64_t n,
                                               int64_t *out_keys, int64_t *out_sums, int64_t *out_counts,
                                               uint64_t out_cap, uint64_t *n_out, void *stream) {
    using namespace gb::noalloc;
    if (!n_out || (n && (!keys || !values)) || !out_keys || !out_sums || !out_counts) {
        set_error("null argument");
        return GB_ERR_INVALID;
    }
    if (n > (1ull << 31)) {
        set_error("%llu rows exceed the allocation-free entry point's limit of 2^31 rows per call",
                  (unsigned long long)n);
        return GB_ERR_INVALID;
    }
    if (out_cap > kMaxGroups) {
        set_error("output capacity %llu exceeds the allocation-free limit of %llu groups",
                  (unsigned long long)out_cap, (unsigned long long)kMaxGroups);
        return GB_ERR_INVALID;
    }
    DevScratch S;
    gb_status s = scratch_for_current_device(&S);
    if (s) return s;
    cudaStream_t st = (cudaStream_t)stream;

    Plan P;
    memset(&P, 0, sizeof P);
    P.n_cols = 2;
    P.cols[0].data = keys;
    P.cols[0].type = GB_T_BIGINT;
    P.cols[1].data = values;
    P.cols[1].type = GB_T_BIGINT;
    P.n_keys = 1;
    P.key_col[0] = 0;
    P.key_type[0] = GB_T_BIGINT;
    P.key_mode = KEY_SINGLE;
    P.n_ops = 1;
    P.ops[0].kind = OP_ADD_I;
    P.ops[0].col = 1;
    P.ops[0].word = 1;
    P.words = kWords;
    P.stride = kStride;

    TableRef T;
    T.slots = S.table;
    T.cap = kCap;
    T.stride = kStride;
    T.gmax_probe = 4096;  // at load <= 0.5 a longer probe run does not occur in practice
    T.ctl = S.ctl;
    T.spill = S.spill;
    T.spill_cap = kSpillCap;
    T.spill_threshold = kSpillCap;

    const int sms = sm_count();
    k_clear<<<sms * 4, 256, 0, st>>>(S.table, S.ctl);
    GB_CUDA(cudaGetLastError());
    if (n) {
        const int smem_slots = 1024;  // 24 KiB: within the default dynamic shared-memory limit
        const size_t smem = (size_t)smem_slots * 8 * (1 + kWords);
        u64 want = (n + 8191) / 8192;
        int grid = (int)std::min<u64>((u64)sms * 2, std::max<u64>(1, want));
        k_ingest_noalloc<<<grid, 512, smem, st>>>(P, T, n, smem_slots);
        GB_CUDA(cudaGetLastError());
        k_merge_noalloc<<<(kSpillCap + 255) / 256, 256, 0, st>>>(P, T);
        GB_CUDA(cudaGetLastError());
    }
    k_emit_noalloc<<<sms * 4, 256, 0, st>>>(S.table, S.ctl, out_keys, out_sums, out_counts, out_cap);
    GB_CUDA(cudaGetLastError());
    Ctl c;
    GB_CUDA(cudaMemcpyAsync(&c, S.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if (c.err & ERR_SPILL_OVERFLOW) {
        set_error("more than %llu distinct keys: beyond the allocation-free table",
                  (unsigned long long)kMaxGroups);
        return GB_ERR_UNSUPPORTED;
    }
    if (c.n_groups > kMaxGroups) {
        set_error("%u distinct keys exceed the allocation-free limit of %llu groups", c.n_groups,
                  (unsigned long long)kMaxGroups);
        return GB_ERR_UNSUPPORTED;
    }
    // (the key INT64_MIN, the table's empty marker, has its own slot and is
    // emitted like any other group)
    if (c.err & ERR_OUT_OVERFLOW) {
        set_error("%u groups do not fit the output capacity %llu", c.out_count, (unsigned long long)out_cap);
        return GB_ERR_INVALID;
    }
    *n_out = c.out_count;
    return GB_OK;
}
