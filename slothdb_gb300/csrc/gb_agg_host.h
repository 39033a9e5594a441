// gb_agg_host.h — host-side hooks shared between translation units.
#pragma once
#include "../../include/slothdb_gb300.h"

// Applies default (or autotuned) launch parameters to a freshly compiled
// handle: shared-table slots, CTAs per SM, block size.
void gb_apply_tuning(gb_agg *h);

#include "gb_internal.cuh"

// A read-only view of the handle's spec for the Parquet ingest.
struct AggView {
    int n_cols;           // spec columns
    int str_col;          // the VARCHAR group key's column (-1: none)
    const int32_t *col_types;
    int n_filters;
    gb::Filter filters[GB_MAX_FILTERS];
    uint64_t nullable_mask;  // spec columns declared nullable (bit c)
};
gb_status gb_agg_view(gb_agg *h, AggView *v);
void gb_agg_count_launch(gb_agg *h, int n);
void gb_agg_count_pruned(gb_agg *h, uint64_t n);
// Device-resident columns whose rows already passed the spec's filters.
gb_status gb_agg_ingest_prefiltered(gb_agg *h, const gb_col *cols, uint64_t nrows, void *stream);
// As above for a VARCHAR group key whose rows arrive as this handle's string
// ids (`ids`, one per row) instead of strings: no per-row encode.
gb_status gb_agg_ingest_prefiltered_ids(gb_agg *h, const gb_col *cols, uint64_t nrows, const int64_t *ids,
                                        void *stream);
// Encode `n` strings (offsets[n + 1] into `bytes`, device) into the handle's
// string dictionary; on success *ids points at their ids (device, valid
// until the handle's next encode).
gb_status gb_agg_encode_strings(gb_agg *h, const uint8_t *bytes, const int64_t *offsets, uint64_t n,
                                uint64_t total_bytes, void *stream, const int64_t **ids);
// Profiling events around a kernel launched outside gb_agg.cu (no-ops
// unless the handle's profiling is on).
struct gb_prof_mark;
gb_prof_mark *gb_agg_prof_begin(gb_agg *h, const char *name, cudaStream_t st);
void gb_agg_prof_end(gb_agg *h, gb_prof_mark *m, cudaStream_t st);
// Frees the per-handle Parquet scratch (called by gb_agg_destroy).
void gb_pq_release_scratch(gb_agg *h);
