// gb_radix.h — host interface of the radix-partitioned GROUP BY kernels.
#pragma once
#include <stdint.h>

#include "gb_kernels.cuh"

#define RADIX_MAX_V 3
#define RADIX_MAX_OPS 4
#define RADIX_ROWS 4
#define P1_WARPS 32   // P1 block = 1024 threads (64 registers each: 32 warps per SM)
#define REG_HOT 4     // hottest keys accumulated in per-lane registers
#define RADIX_BLOCK 1024
#define CURSOR_PAD 32    // partition cursors 128 bytes apart (spread over L2 slices)
#define HIST_BINS 1024   // sample-count histogram bins

namespace gb {

struct RadixPlan {
    int32_t V;                          // value words per tuple
    int32_t vcol[RADIX_MAX_V];          // column of each tuple value
    int32_t op_v[GB_MAX_OPS];           // tuple value index of each op
    uint8_t word_kind[GB_MAX_WORDS];    // op kind owning each state word (0: count)
    int32_t pbits;                      // partitions = 1 << pbits
    int32_t HS;                         // hot hash-table slots (power of two)
    int32_t nh;                         // hot keys (dense indices [0, nh))
    int32_t nsup;                       // super-hot keys: indices [0, nsup)
    int32_t sub;                        // P2 shared-table slots (power of two)
    int32_t wcb;                        // P1 write-combining tuples per partition
    int32_t hot_probe;
    int32_t agg_probe;
    int32_t p2_pre;                     // P2: warps pre-combine equal keys (1) or fold each tuple (0)
    int32_t spec;                       // specialised P1 (OP_ADD_F / OP_ADD_I) or 0
};

struct RadixRef {
    u64 *part;                // partition regions of (1 + V)-word tuples
    const u64 *part_off;      // first tuple of each region
    const u32 *part_cap;      // tuples each region holds
    u32 *cursor;              // per-partition fill, CURSOR_PAD apart
    u64 *ovf;                 // overflow tuples (partition, key, values...)
    u32 ovf_cap;
    u32 ovf_threshold;
    const u64 *hot_keys;      // HS/2 buckets of 2 keys (EMPTY_KEY = unused)
    const uint16_t *hot_idx;  // hot rank of each bucket slot
    const u64 *hot_list;      // nh keys by hot index
    u64 *hot_part;            // [grid][nh][words] per-CTA hot partials
    u64 *p2_words;            // [np][sub][words - 1] P2 state words when they fold in L2 (or null)
};

struct RadixTile {
    u64 n_rows;
    u32 n_tiles;
    u32 first_tile;
};

gb_status radix_prepare(const Plan &P, RadixPlan &R, u64 est_groups, u64 nullable_mask);
size_t radix_p1_smem(const Plan &P, const RadixPlan &R);
gb_status radix_set_bits(const Plan &P, RadixPlan &R, int bits);
// The specialised-P1 kind radix_prepare would pick for P now (0: none); a
// plan whose predicates changed re-prepares when it differs from R.spec.
int radix_spec_of(const Plan &P, const RadixPlan &R, u64 nullable_mask);
size_t radix_p2_smem(const Plan &P, const RadixPlan &R);
bool radix_p2_global_words(const Plan &P, const RadixPlan &R);
u32 radix_tile_rows(const RadixPlan &R);
u64 radix_inflight_rows(const RadixPlan &R, int grid);
size_t radix_p1d_smem(const RadixPlan &R);
gb_status radix_launch_sample(const Plan &P, const RadixPlan &R, u64 n, u64 *skeys, u32 *scnt, u64 scap, u32 *hist,
                              u32 *hstate, u64 *cand_key, u32 *cand_cnt, u64 *hot_keys, uint16_t *hot_idx,
                              u64 *hot_list, cudaStream_t st, u64 *launches);
gb_status radix_launch_p1(const Plan &P, const RadixPlan &R, const RadixRef &X, const TableRef &T,
                          const RadixTile &A, int grid, cudaStream_t st);
gb_status radix_launch_drain(const RadixRef &X, int V, u32 n, cudaStream_t st);
gb_status radix_launch_move(const RadixRef &from, const RadixRef &to, int V, int np, cudaStream_t st);
gb_status radix_launch_p2(const Plan &P, const RadixPlan &R, const RadixRef &X, const TableRef &T, const EmitArgs &E,
                          cudaStream_t st);
gb_status radix_launch_p3(const Plan &P, const RadixPlan &R, const RadixRef &X, int G, const u32 *hstate, Ctl *ctl,
                          const EmitArgs &E, cudaStream_t st);
gb_status radix_fill_u64(u64 *dst, u64 n, u64 value, cudaStream_t st);
gb_status radix_fill_identity(u64 *dst, u64 n, int W, const Plan &P, cudaStream_t st);

}  // namespace gb
