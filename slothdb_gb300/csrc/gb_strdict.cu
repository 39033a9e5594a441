// gb_strdict.cu — VARCHAR group keys on GB300: a device string dictionary.
//
// The reference groups VARCHAR keys by their bytes (the string-key branch of
// the chunk loop, src/execution/physical_planner.cpp:7951-7973, and
// AppendGroupKey, 6185-6206).  Here every distinct string gets an id — the
// index of its slot in an open-addressing table of {hash, ref} pairs, where
// ref = (arena byte offset << 24) | length of a copy of the string in an
// append-only device arena — and the integer aggregation runs on the ids.
// Equality is exact: a hash match is confirmed by comparing the bytes with
// the slot's representative.  A slot's ref is published right after its hash
// is claimed; a reader that sees the hash before the ref waits a bounded
// number of iterations and then reports a timeout instead of hanging.
#include <algorithm>
#include <cstring>
#include <vector>

#include "gb_kernels.cuh"
#include "gb_strdict.h"

namespace gb {

// Encode rows [0, n) (or the rows listed in `rows`) of a VARCHAR column into
// ids, one row per lane of warp-uniform groups of 32; rows that found no slot
// are appended to `retry` for the host to re-run after growing the table /
// arena.
__global__ void __launch_bounds__(256, 4) k_strdict_encode(const StrDictRef D, const uint8_t *bytes, const int64_t *offsets, int64_t off_base,
                                 const uint64_t *valid, u64 n, const u32 *rows, long long *ids, u32 *retry,
                                 u32 *retry_n, u32 *new_strs_total) {
    __shared__ u32 s_new;
    if (threadIdx.x == 0) s_new = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const u64 warp = (blockIdx.x * (u64)blockDim.x + threadIdx.x) >> 5;
    const u64 nwarps = ((u64)gridDim.x * blockDim.x) >> 5;
    for (u64 base = warp * 32; base < n; base += nwarps * 32) {
        const u64 i = base + lane;
        bool act = i < n;
        u64 r = 0;
        if (act) {
            r = rows ? rows[i] : i;
            if (valid && !((valid[r >> 6] >> (r & 63)) & 1ull)) {
                ids[r] = -1;  // NULL key: the aggregation treats it as the NULL group
                act = false;
            }
        }
        const int64_t a = act ? offsets[r] - off_base : 0;
        const u32 len = act ? (u32)(offsets[r + 1] - off_base - a) : 0u;
        const long long id = strdict_warp_encode(D, bytes + a, len, act, &s_new);
        if (!act) continue;
        if (id >= 0) {
            ids[r] = id;
        } else {
            ids[r] = -1;
            if (id == -1) {
                const u32 q = atomicAdd(retry_n, 1u);
                retry[q] = (u32)r;  // the retry list holds every row of the call at most once
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_new) atomicAdd(new_strs_total, s_new);
}

// Move every used slot of `old` into the (larger) table `D`.
__global__ void k_strdict_rehash(const u64 *old_hash, const u64 *old_ref, const u64 *old_id, u64 old_cap,
                                 const StrDictRef D) {
    for (u64 s = blockIdx.x * (u64)blockDim.x + threadIdx.x; s < old_cap; s += (u64)gridDim.x * blockDim.x) {
        const u64 h = old_hash[s];
        if (h == EMPTY_KEY || (old_ref[s] >> 24) == DEAD_OFF || old_ref[s] == REF_PENDING) continue;
        u64 slot = h & (D.cap - 1);
        for (u64 p = 0; p < D.cap; p++) {
            const u64 old = atomicCAS(D.hash + slot, EMPTY_KEY, h);
            if (old == EMPTY_KEY) {
                D.ref[slot] = old_ref[s];
                D.id[slot] = old_id[s];
                break;
            }
            slot = (slot + 1) & (D.cap - 1);
        }
    }
}

// Output strings of ids[0, n): lengths first (for the offsets scan), then bytes.
__global__ void k_strdict_lengths(const StrDictRef D, const long long *ids, u64 n, int64_t *lens, uint64_t *valid) {
    for (u64 i = blockIdx.x * (u64)blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
        const long long id = ids[i];
        lens[i] = id < 0 ? 0 : (int64_t)(D.ref_by_id[id] & 0xffffffu);
        if (id < 0 && valid) atomicAnd((unsigned long long *)&valid[i >> 6], ~(1ull << (i & 63)));  // NULL string
    }
}

__global__ void k_strdict_gather(const StrDictRef D, const long long *ids, u64 n, const int64_t *offs, uint8_t *out) {
    // one warp per string
    const int lane = threadIdx.x & 31;
    const u64 w = (blockIdx.x * (u64)blockDim.x + threadIdx.x) >> 5;
    const u64 nw = ((u64)gridDim.x * blockDim.x) >> 5;
    for (u64 i = w; i < n; i += nw) {
        const long long id = ids[i];
        if (id < 0) continue;
        const u64 r = D.ref_by_id[id];
        const u32 len = (u32)(r & 0xffffffu);
        const uint8_t *src = D.arena + (r >> 24);
        for (u32 b = lane; b < len; b += 32) out[offs[i] + b] = src[b];
    }
}

// Exclusive scan of n int64 (single pass per block + carry kernels).
__global__ void k_scan_blocks(const int64_t *in, int64_t *out, u64 n, int64_t *block_sums) {
    __shared__ int64_t sm[1024];
    const u64 i = blockIdx.x * (u64)blockDim.x + threadIdx.x;
    int64_t x = i < n ? in[i] : 0;
    sm[threadIdx.x] = x;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
        int64_t y = threadIdx.x >= (unsigned)o ? sm[threadIdx.x - o] : 0;
        __syncthreads();
        sm[threadIdx.x] += y;
        __syncthreads();
    }
    if (i < n) out[i] = sm[threadIdx.x] - x;
    if (threadIdx.x == blockDim.x - 1) block_sums[blockIdx.x] = sm[threadIdx.x];
}

__global__ void k_scan_carry(int64_t *out, u64 n, const int64_t *block_prefix) {
    const u64 i = blockIdx.x * (u64)blockDim.x + threadIdx.x;
    if (i < n) out[i] += block_prefix[blockIdx.x];
}

// ================================================================== host
static int grid_n(u64 work, int block, int cap) {
    u64 g = (work + block - 1) / block;
    return (int)std::max<u64>(1, std::min<u64>(g, (u64)cap));
}

gb_status strdict_launch_encode(const StrDictRef &D, const uint8_t *bytes, const int64_t *offsets, int64_t off_base,
                                const uint64_t *valid, u64 n, const u32 *rows, long long *ids, u32 *retry, u32 *retry_n,
                                u32 *new_strs, cudaStream_t st) {
    if (n == 0) return GB_OK;
    k_strdict_encode<<<grid_n(n, 256, sm_count() * 8), 256, 0, st>>>(D, bytes, offsets, off_base, valid, n, rows, ids,
                                                                   retry, retry_n, new_strs);
    GB_CUDA(cudaGetLastError());
    return GB_OK;
}

gb_status strdict_launch_rehash(const u64 *old_hash, const u64 *old_ref, const u64 *old_id, u64 old_cap,
                                const StrDictRef &D, cudaStream_t st) {
    k_strdict_rehash<<<grid_n(old_cap, 256, sm_count() * 8), 256, 0, st>>>(old_hash, old_ref, old_id, old_cap, D);
    GB_CUDA(cudaGetLastError());
    return GB_OK;
}

__global__ void k_fill64(u64 *p, u64 n, u64 v) {
    for (u64 i = blockIdx.x * (u64)blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) p[i] = v;
}

gb_status strdict_fill(u64 *p, u64 n, u64 v, cudaStream_t st) {
    if (!n) return GB_OK;
    k_fill64<<<grid_n(n, 256, sm_count() * 8), 256, 0, st>>>(p, n, v);
    GB_CUDA(cudaGetLastError());
    return GB_OK;
}

// Scan lens[0, n) into offs[0, n] (offs[n] = total); returns total in *total.
gb_status device_exclusive_scan(const int64_t *lens, int64_t *offs, u64 n, int64_t *tmp, cudaStream_t st,
                                int64_t *total) {
    const int B = 1024;
    u64 nb = (n + B - 1) / B;
    if (nb == 0) {
        *total = 0;
        GB_CUDA(cudaMemsetAsync(offs, 0, 8, st));
        return GB_OK;
    }
    k_scan_blocks<<<(unsigned)nb, B, 0, st>>>(lens, offs, n, tmp);
    GB_CUDA(cudaGetLastError());
    std::vector<int64_t> bs(nb);
    GB_CUDA(cudaMemcpyAsync(bs.data(), tmp, nb * 8, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    int64_t acc = 0;
    for (u64 b = 0; b < nb; b++) {
        int64_t s = bs[b];
        bs[b] = acc;
        acc += s;
    }
    GB_CUDA(cudaMemcpyAsync(tmp, bs.data(), nb * 8, cudaMemcpyHostToDevice, st));
    k_scan_carry<<<(unsigned)nb, B, 0, st>>>(offs, n, tmp);
    GB_CUDA(cudaGetLastError());
    GB_CUDA(cudaMemcpyAsync(offs + n, &acc, 8, cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaStreamSynchronize(st));
    *total = acc;
    return GB_OK;
}

gb_status strdict_launch_lengths(const StrDictRef &D, const long long *ids, u64 n, int64_t *lens, cudaStream_t st,
                                 uint64_t *valid) {
    if (!n) return GB_OK;
    k_strdict_lengths<<<grid_n(n, 256, sm_count() * 8), 256, 0, st>>>(D, ids, n, lens, valid);
    GB_CUDA(cudaGetLastError());
    return GB_OK;
}

gb_status strdict_launch_gather(const StrDictRef &D, const long long *ids, u64 n, const int64_t *offs, uint8_t *out,
                                cudaStream_t st) {
    if (!n) return GB_OK;
    k_strdict_gather<<<grid_n(n * 32, 256, sm_count() * 8), 256, 0, st>>>(D, ids, n, offs, out);
    GB_CUDA(cudaGetLastError());
    return GB_OK;
}

}  // namespace gb
