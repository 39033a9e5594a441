// gb_radix.h — host interface of the radix-partitioned GROUP BY kernels.
#pragma once
#include "gb_kernels.cuh"

#define RADIX_MAX_V 3
#define RADIX_ROWS 4
#define RADIX_BLOCK 1024
#define CURSOR_PAD 8  // partition cursors 32 bytes apart (one sector each)

namespace gb {

struct RadixPlan {
    int32_t V;                          // value words per tuple
    int32_t vcol[RADIX_MAX_V];          // column of each tuple value
    int32_t op_v[GB_MAX_OPS];           // tuple value index of each op
    uint8_t word_kind[GB_MAX_WORDS];    // op kind owning each state word (0: count)
    int32_t pbits;                      // partitions = 1 << pbits
    int32_t HS;                         // hot-table slots (power of two)
    int32_t hot_probe;
    int32_t agg_probe;
};

struct RadixRef {
    u64 *part;           // partitions: (1 << pbits) regions of cap_p tuples of (1 + V) words
    u64 cap_p;
    u32 *cursor;         // per-partition fill, CURSOR_PAD apart
    u64 *ovf;            // overflow tuples (partition, key, values...)
    u32 ovf_cap;
    u32 ovf_threshold;
    const u64 *hot_keys; // HS keys (EMPTY_KEY = unused)
    u64 *hot_part;       // [grid][HS][words] per-CTA hot partials
};

struct RadixTile {
    u64 n_rows;
    u32 n_tiles;
    u32 first_tile;
};

gb_status radix_prepare(const Plan &P, RadixPlan &R, u64 est_groups, u64 nullable_mask);
size_t radix_p1_smem(const Plan &P, const RadixPlan &R);
u32 radix_tile_rows(const RadixPlan &R);
int radix_sp(const Plan &P);
gb_status radix_launch_sample(const Plan &P, const RadixPlan &R, u64 n, u64 *skeys, u32 *scnt, u64 scap, u32 *hist,
                              u64 *hot_keys, cudaStream_t st, u64 *launches);
gb_status radix_launch_p1(const Plan &P, const RadixPlan &R, const RadixRef &X, const TableRef &T,
                          const RadixTile &A, int grid, cudaStream_t st);
gb_status radix_launch_drain(const RadixRef &X, int V, u32 n, cudaStream_t st);
gb_status radix_launch_p2(const Plan &P, const RadixPlan &R, const RadixRef &X, const TableRef &T, const EmitArgs &E,
                          cudaStream_t st);
gb_status radix_launch_p3(const Plan &P, const RadixPlan &R, const RadixRef &X, int G, Ctl *ctl, const EmitArgs &E,
                          cudaStream_t st);
gb_status radix_fill_identity(u64 *dst, u64 n, int W, const Plan &P, cudaStream_t st);

}  // namespace gb
