/*
 * slothdb_gb300.h — C ABI of the GB300 GROUP BY execution path.
 *
 * One handle (gb_agg) executes one GROUP BY: it is created from a plan
 * description (group columns, aggregates, simple scan predicates), is fed
 * row batches (typed column vectors or raw Parquet row groups), and is
 * finalised into a typed result table.  Every entry point returns a
 * gb_status; gb_last_error() gives the message of the calling thread's most
 * recent failure.  There is no CPU fallback: a shape the GPU path does not
 * implement is rejected with GB_ERR_UNSUPPORTED.
 *
 * Handles are thread-compatible (one thread at a time per handle).  Host
 * pointers passed in are borrowed for the duration of the call; result
 * buffers are owned by the handle until the next reset/destroy.
 *
 * Every function names the reference (SlothDB) interface it replaces; paths
 * are relative to the reference project root.
 */
#ifndef SLOTHDB_GB300_H
#define SLOTHDB_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GB_ABI_VERSION 1

typedef enum gb_status {
    GB_OK = 0,
    GB_ERR_INVALID = 1,      /* bad argument or malformed plan                */
    GB_ERR_OOM = 2,          /* device or pinned-host allocation failed       */
    GB_ERR_UNSUPPORTED = 3,  /* shape not implemented on the GPU path         */
    GB_ERR_TIMEOUT = 4,      /* a bounded device wait gave up                 */
    GB_ERR_CUDA = 5,         /* CUDA runtime error                            */
    GB_ERR_CORRUPT = 6,      /* malformed Parquet page / footer               */
    GB_ERR_STATE = 7,        /* call out of order (e.g. result before finalize) */
    GB_ERR_BUDGET = 8        /* admission refused: over the memory budget     */
} gb_status;

/* Column types, named after the reference's LogicalTypeId values that the
 * GROUP BY path accepts (include/slothdb/common/types/logical_type.hpp). */
typedef enum gb_type {
    GB_T_SMALLINT = 1,  /* int16  */
    GB_T_INTEGER = 2,   /* int32  */
    GB_T_BIGINT = 3,    /* int64  */
    GB_T_DOUBLE = 4,    /* double */
    GB_T_VARCHAR = 5    /* bytes + int64 offsets[n+1] */
} gb_type;

/* Aggregates the binder resolves for GROUP BY
 * (src/binder/binder.cpp:1345-1391): COUNT → BIGINT; SUM(int) → BIGINT;
 * SUM(double) → DOUBLE; AVG → DOUBLE; MIN/MAX → input type.
 * COUNT(DISTINCT col) → BIGINT: the number of distinct non-NULL values of an
 * integer column in the group (the per-group value sets of
 * src/execution/int_group_agg.cpp:89-92, union sizes at 154-270); 0 for a
 * group whose values are all NULL.  It runs in hash mode and in batches
 * (not in radix mode); at most GB_MAX_DISTINCT distinct columns per query. */
typedef enum gb_agg_kind {
    GB_AGG_COUNT_STAR = 0,
    GB_AGG_COUNT = 1,
    GB_AGG_SUM = 2,
    GB_AGG_AVG = 3,
    GB_AGG_MIN = 4,
    GB_AGG_MAX = 5,
    GB_AGG_COUNT_DISTINCT = 6
} gb_agg_kind;

#define GB_MAX_DISTINCT 2

/* Comparison of a SimplePredicate (src/execution/physical_planner.cpp:110-135):
 * the six numeric compares; INTEGER/BIGINT/SMALLINT `col IN (set)`
 * (int_in_form); VARCHAR `col = 'lit'` / `col <> 'lit'` (str_form); VARCHAR
 * `col LIKE '%needle%'` / `NOT LIKE` (like_contains / like_negated:
 * case-sensitive byte substring, an empty needle matches every non-NULL
 * value).  A NULL row never passes. */
typedef enum gb_cmp {
    GB_CMP_EQ = 0, GB_CMP_NE = 1, GB_CMP_LT = 2,
    GB_CMP_LE = 3, GB_CMP_GT = 4, GB_CMP_GE = 5,
    GB_CMP_IN = 6,         /* data: int64_t[n] set members (any order, duplicates allowed) */
    GB_CMP_STR_EQ = 7,     /* data: n literal bytes */
    GB_CMP_STR_NE = 8,
    GB_CMP_LIKE = 9,       /* data: n needle bytes of LIKE '%needle%' */
    GB_CMP_NOT_LIKE = 10
} gb_cmp;
#define GB_MAX_IN_SET 65536       /* members of one IN set */
#define GB_MAX_STR_LITERAL 4096   /* bytes of one string literal */

typedef struct gb_agg_desc {
    int32_t kind;   /* gb_agg_kind */
    int32_t col;    /* input column index; -1 for COUNT(*) */
} gb_agg_desc;

/* col OP constant.  Integer columns compare in int64 (the reference widens
 * to int64 before comparing, physical_planner.cpp:466-479, 693-716); DOUBLE
 * columns compare against d_const.  IN and the VARCHAR forms read their
 * literal from `data` (host memory, n elements / bytes): the library keeps
 * its own copy, so the caller's buffer is needed only during the call that
 * takes the filter. */
typedef struct gb_filter {
    int32_t col;
    int32_t op;      /* gb_cmp */
    int64_t i_const;
    double d_const;
    const void *data;  /* GB_CMP_IN / STR / LIKE literal, else NULL */
    uint64_t n;
} gb_filter;

#define GB_SPEC_COL_NULLABLE_BITS 0  /* see gb_agg_spec.nullable_mask */

typedef struct gb_agg_spec {
    uint32_t n_cols;            /* input schema width                        */
    const int32_t *col_types;   /* gb_type per input column                  */
    uint32_t n_groups;          /* 1 or 2 group columns                      */
    const int32_t *group_cols;
    uint32_t n_aggs;
    const gb_agg_desc *aggs;
    uint32_t n_filters;         /* conjunction of predicates (WHERE)         */
    const gb_filter *filters;
    uint64_t nullable_mask;     /* bit c set: column c may carry NULLs       */
    uint64_t est_groups;        /* planner estimate; 0 = unknown             */
} gb_agg_spec;

/* One input column vector.  Validity uses the reference's ValidityMask
 * layout (include/slothdb/common/types/validity_mask.hpp:9-69): 64-bit
 * words, bit (i % 64) of word (i / 64) set = row i valid; NULL = all valid. */
typedef struct gb_col {
    const void *data;
    const uint64_t *validity;
    const int64_t *offsets;     /* VARCHAR only: n+1 byte offsets into data  */
} gb_col;

typedef enum gb_mem { GB_MEM_HOST = 0, GB_MEM_DEVICE = 1 } gb_mem;

/* Result table: [group columns..., aggregate columns...], the output slot
 * order of PhysicalHashAggregate (physical_planner.cpp:6017-6021). */
typedef struct gb_result {
    uint64_t n_rows;
    uint32_t n_cols;
    const int32_t *types;             /* gb_type per output column          */
    const void *const *data;          /* per column                         */
    const int64_t *const *offsets;    /* VARCHAR columns, else NULL         */
    const uint64_t *const *validity;  /* NULL entry = all valid             */
} gb_result;

typedef struct gb_agg gb_agg;

/* Thread-local message of the last failed call ("" if none). */
const char *gb_last_error(void);
int gb_abi_version(void);

/* Replaces PhysicalHashAggregate(groups, aggregates, result_types)
 * (src/execution/physical_planner.cpp:6011-6015) as constructed by
 * PhysicalPlanner::PlanAggregate (physical_planner.cpp:14356-14362). */
gb_status gb_agg_create(const gb_agg_spec *spec, gb_agg **out);

/* Device bytes a GROUP BY of `nrows` rows with this spec is expected to hold
 * (hash table sized from min(est_groups, nrows), result columns, spill
 * records, string dictionary).  Compiles the plan only; allocates nothing.
 * Used for admission control; no reference counterpart. */
gb_status gb_agg_estimate_bytes(const gb_agg_spec *spec, uint64_t nrows, uint64_t *bytes);

/* Replaces the handle's WHERE predicates (same plan otherwise), after create
 * or reset and before the first ingest — so a pooled handle can serve the
 * next query of the same shape without reallocating.  No reference
 * counterpart (the reference builds a new operator per query). */
gb_status gb_agg_set_filters(gb_agg *h, const gb_filter *filters, uint32_t n_filters);

/* Replaces PhysicalHashAggregate::SetTopNHint (physical_planner.cpp:6022-6027):
 * keep only the best `limit` rows by output column `col_idx` (output slot
 * space; ties broken by group key ascending). */
gb_status gb_agg_set_topn(gb_agg *h, uint32_t col_idx, int32_t ascending, uint64_t limit);

/* Replaces PhysicalHashAggregate::SetRowLimit (physical_planner.cpp:6032). */
gb_status gb_agg_set_row_limit(gb_agg *h, uint64_t limit);

/* Replaces the child GetData(DataChunk&) consumption of the chunk loops
 * (physical_planner.cpp:7933-8021, 12291-12516): aggregates `nrows` rows of
 * the spec's input columns.  May be called repeatedly; states accumulate.
 * mem = GB_MEM_HOST copies the vectors to HBM inside the call (pinned
 * host memory is copied directly, overlapped with the aggregation);
 * GB_MEM_DEVICE reads device-resident vectors.  `stream` is a cudaStream_t
 * (NULL = legacy default stream). */
gb_status gb_agg_ingest(gb_agg *h, const gb_col *cols, uint64_t nrows, int32_t mem, void *stream);

/* Replaces the merge + emit of ComputeAggregates (physical_planner.cpp:
 * 7871-7908 merge, 8027-8173 direct emit / TopN, agg_emit_helpers.cpp:26-165). */
gb_status gb_agg_finalize(gb_agg *h, void *stream);

/* Replaces PhysicalHashAggregate::GetData emission (physical_planner.cpp:
 * 6040-6060): host copies of the result columns, owned by the handle. */
gb_status gb_agg_result(gb_agg *h, gb_result *out);

/* Device-resident view of the same result (no copy). */
gb_status gb_agg_result_device(gb_agg *h, gb_result *out);

/* Rewinds the handle to the empty state, keeping its device allocations
 * (re-execution of the same plan: PhysicalHashAggregate::Init,
 * physical_planner.cpp:6034-6038). */
gb_status gb_agg_reset(gb_agg *h);

void gb_agg_destroy(gb_agg *h);

/* Number of kernels this handle launched since create/reset (for launch
 * accounting). */
uint64_t gb_agg_kernel_launches(const gb_agg *h);

/* Parquet row groups that this handle's gb_agg_ingest_parquet calls skipped
 * since create/reset because their statistics rule out a predicate (the
 * reference marks the same row groups RGWork::pruned,
 * physical_planner.cpp:1020, 1142-1182). */
uint64_t gb_agg_row_groups_pruned(const gb_agg *h);

/* Execution options of a handle, set before its first ingest (the
 * autotuner's knobs; no reference counterpart beyond the hard-coded thread
 * counts of physical_planner.cpp:7320-7641):
 *   "mode"        0 auto, 1 hash (shared + HBM tables), 2 radix partitions
 *   "smem_slots"  shared pre-aggregation table slots (power of two, hash)
 *   "precombine"  warp pre-combine of duplicate keys (0/1, hash)
 *   "ctas_per_sm" persistent CTAs per SM (hash)
 *   "tile_rows"   rows per claimed tile (hash)
 *   "hot_slots"   heavy-hitter table slots (power of two, radix)
 *   "radix_bits"  log2 of the partition count, 6..12 (radix)
 *   "radix_precombine"  1 = the partition pass combines a warp's equal keys
 *                 before folding, 0 = folds tuple by tuple (radix; default 0
 *                 when every op is a DOUBLE SUM, else 1) */
gb_status gb_agg_set_option(gb_agg *h, const char *name, int64_t value);
/* 1 = radix mode, 0 = hash mode. */
int32_t gb_agg_get_mode(const gb_agg *h);

/* Per-kernel device time of this handle, measured with CUDA events on the
 * stream each kernel is launched on (enabled by gb_agg_set_profiling; no
 * reference counterpart: the reference's SLOTH_PROFILE counters,
 * include/slothdb/storage/parquet.hpp:22-44, are host timers). */
typedef struct gb_kernel_stat {
    char name[32];
    uint64_t launches;
    double ms;
} gb_kernel_stat;

gb_status gb_agg_set_profiling(gb_agg *h, int32_t on);
uint32_t gb_agg_profile(const gb_agg *h, gb_kernel_stat *out, uint32_t max);

/* Replaces GPUEngine::HashAggregate (include/slothdb/execution/gpu/
 * gpu_engine.hpp:78-84): group int32 keys, SUM and COUNT int32 values.
 * Host in, host out.  Output arrays hold `*n_out` groups (capacity
 * `cap`, GB_ERR_INVALID if more groups than cap). */
gb_status gb_engine_hash_aggregate(const int32_t *keys, const int32_t *values, uint64_t n,
                                   int32_t *out_keys, int64_t *out_sums, int64_t *out_counts,
                                   uint64_t cap, uint64_t *n_out);

/* ---------------------------------------------------------------- Parquet
 * A Parquet file held in host memory (read or mmap'd by the caller).
 * gb_pq_open parses the footer and every page header into a page index —
 * replaces ParquetReader's metadata/page walk (src/storage/parquet.cpp:
 * 92-470 thrift + page headers, 1107-1366 metadata, 2475-2706 ReadColumnInto).
 * Supported: uncompressed column chunks, REQUIRED flat columns of INT32
 * (INT(16) annotation → SMALLINT), INT64 and DOUBLE, PLAIN or dictionary
 * (RLE / bit-packed hybrid) encoded, data page v1 and v2, and a
 * dictionary-encoded BYTE_ARRAY column as the VARCHAR group key. */
typedef struct gb_pq_file gb_pq_file;
gb_status gb_pq_open(const uint8_t *bytes, uint64_t size, gb_pq_file **out);
uint32_t gb_pq_num_row_groups(const gb_pq_file *f);
uint64_t gb_pq_num_rows(const gb_pq_file *f);
uint32_t gb_pq_num_columns(const gb_pq_file *f);
gb_status gb_pq_column_info(const gb_pq_file *f, uint32_t col, char *name, uint32_t name_cap, int32_t *type);
/* Zone map: *might = 0 when row group `rg`'s column statistics (Statistics
 * min_value / max_value, or the deprecated min / max) prove that no row passes
 * every filter (filter columns are spec columns, mapped to file columns by
 * col_map[0, n_cols)), else 1 — IsRowGroupPruned / RowGroupMightMatch
 * (physical_planner.cpp:1142-1150, src/storage/parquet.cpp:3200-3240).
 * INTEGER, BIGINT and DOUBLE statistics are read (the reference reads none
 * for SMALLINT).  gb_agg_ingest_parquet skips the row groups this rules out. */
/* Ungrouped SUM and COUNT of one INT64 dictionary-encoded column over row
 * groups [rg_begin, rg_end) without decoding it: a histogram of each row
 * group's dictionary indices, then sum_idx count[idx] * dict[idx]
 * (TryDictHistogramAgg, include/slothdb/execution/dict_histogram.hpp:34, per
 * row group ParquetReader::DecodeBigintColumnHistogram,
 * src/storage/parquet.cpp:2726-2897, the fast path of
 * SELECT SUM(c) / AVG(c) / COUNT(c) FROM file, physical_planner.cpp:
 * 8745-8790).  PLAIN pages of the column (dictionary fallback) are summed as
 * they are; indices past the dictionary are not counted, as there.  *count =
 * the values counted, *sum = their exact sum rounded once to double.
 * GB_ERR_UNSUPPORTED — the reference's `false`, after which the engine takes
 * the fused path — when the column is not INT64, a row group has no
 * dictionary page, a page holds NULLs, or a chunk is compressed.  mem:
 * GB_MEM_DEVICE reads the uploaded file (gb_pq_upload), GB_MEM_HOST copies
 * the column's byte range. */
gb_status gb_pq_dict_sum(gb_pq_file *f, uint32_t col, uint32_t rg_begin, uint32_t rg_end, int32_t mem, void *stream,
                         int64_t *count, double *sum);
gb_status gb_pq_row_group_might_match(const gb_pq_file *f, uint32_t rg, const int32_t *col_map, uint32_t n_cols,
                                      const gb_filter *filters, uint32_t n_filters, int32_t *might);
/* Copies the whole file into HBM once (a resident table). */
gb_status gb_pq_upload(gb_pq_file *f, void *stream);
void gb_pq_close(gb_pq_file *f);

/* Replaces the RG-consumer path of the fused Parquet aggregate
 * (PhysicalParquetScan::SetRGConsumer / RunParallelRGs / DecodeRowGroupInto,
 * physical_planner.cpp:1060-1062, 1070-1135, 1175-1203, consumed by the
 * TLSingle loop 7613-7931): row groups [rg_begin, rg_end) are decoded on the
 * GPU (dictionary RLE/bit-unpack + gather, PLAIN loads), filtered by the
 * spec's predicates and aggregated.  Spec column c reads file column
 * col_map[c].  mem = GB_MEM_DEVICE reads the gb_pq_upload'ed copy;
 * GB_MEM_HOST copies the row groups' bytes to HBM inside the call. */
gb_status gb_agg_ingest_parquet(gb_agg *h, gb_pq_file *f, uint32_t rg_begin, uint32_t rg_end, const int32_t *col_map,
                                int32_t mem, void *stream);

/* ----------------------------------------------------------------- batches
 * Many independent GROUP BY queries over device-resident tables, executed
 * together.  The reference runs each such query on its own, through the
 * generic chunk loop of its hash aggregate (composite / VARCHAR keys,
 * src/execution/physical_planner.cpp:12291-12516, AppendGroupKey
 * 6185-6206); gb_batch_add takes the same gb_agg_spec a single query takes,
 * and gb_batch_result returns what gb_agg_result would for that query.
 * gb_batch_run executes every query with a few launches in total — table
 * init, VARCHAR key encoding, one persistent aggregation kernel over a
 * device work queue of (query, tile) items, compaction — captured as a CUDA
 * graph on the first run and replayed on later runs.  A query that needs a
 * host decision (hash-table growth, string-dictionary growth) is re-run on
 * its own afterwards; gb_batch_slow_queries counts them for the last run.
 * Column pointers (gb_col) must be device memory and stay valid, with the
 * same row counts, for every run of the batch.  Options ("graph" 0/1,
 * "ctas_per_sm" 1..4, "smem_slots" 0 or a power of two <= 4096,
 * "precombine" 0 never / 1 per query / 2 always, "profiling" 0/1, "order" 0
 * query-major tiles / 1
 * interleaved, "tile_rows" a power of two in [1024, 2^20], "fast" 0/1 for
 * the register-resident integer tile path) take effect at the next run; with
 * profiling on, runs skip the graph and gb_batch_profile reports CUDA-event
 * times of the four kernels. */
typedef struct gb_batch gb_batch;
gb_status gb_batch_create(gb_batch **out);
gb_status gb_batch_add(gb_batch *b, const gb_agg_spec *spec, const gb_col *cols, uint64_t nrows, uint32_t *query_index);
gb_status gb_batch_set_option(gb_batch *b, const char *name, int64_t value);
gb_status gb_batch_run(gb_batch *b, void *stream);
/* Removes every query from the batch but keeps its device buffers; the
 * queries' handles stay in an idle pool and a later gb_batch_add of the same
 * plan shape and table size reuses one (new filter constants allowed), so a
 * long-lived batch object allocates nothing in steady state. */
gb_status gb_batch_clear(gb_batch *b);
uint32_t gb_batch_size(const gb_batch *b);
gb_status gb_batch_result(gb_batch *b, uint32_t query_index, gb_result *out);
/* Device-resident view of query i's result (valid until the next run/clear). */
gb_status gb_batch_result_device(gb_batch *b, uint32_t query_index, gb_result *out);
uint32_t gb_batch_slow_queries(const gb_batch *b);
uint64_t gb_batch_kernel_launches(const gb_batch *b);
uint32_t gb_batch_profile(const gb_batch *b, gb_kernel_stat *out, uint32_t max);
void gb_batch_destroy(gb_batch *b);

/* ----------------------------------------------------------------- serving
 * A served stream of GROUP BY queries over tables resident in HBM (no
 * reference counterpart: the reference plans and runs each query on the
 * caller's thread, Connection::Query → PhysicalPlanner::PlanAggregate,
 * physical_planner.cpp:14356-14362).  One dispatcher thread owns the GPU:
 * queued queries are admitted in arrival order while the sum of their
 * estimated device bytes (gb_agg_estimate_bytes) stays within
 * `budget_bytes` (a query whose estimate alone exceeds it fails with
 * GB_ERR_BUDGET), at most `max_batch` per batch, and run together as one
 * gb_batch; queries estimated at >= 2^20 groups run alone on their own
 * handle.  mode 1 runs every query alone, one at a time (the baseline).
 * Queries that arrive while a batch executes form the next batch.
 * Tables are registered (device columns, borrowed; validity-masked tables
 * are sliced at multiples of 64 rows) before the first submit.  A query is
 * a gb_agg_spec over the table's columns plus a row range.  Results are
 * host copies owned by the ticket until gb_server_release.  gb_server_wait
 * returns the query's status (GB_ERR_TIMEOUT if not done within timeout_us;
 * timeout_us < 0 waits without limit).  gb_server_destroy drains the queue. */
typedef struct gb_server gb_server;
typedef struct gb_server_stat {
    uint64_t batches, completed, rejected, failed, queued;
    uint64_t peak_admitted_bytes;
    double busy_ms;
    uint64_t kernel_launches;
    uint64_t result_bytes; /* device→host bytes of the results copied so far */
} gb_server_stat;
gb_status gb_server_create(uint64_t budget_bytes, uint32_t max_batch, int32_t mode, gb_server **out);
/* Execution lanes (1..8, before the first submit; continuous batching
 * defaults to 2, one-at-a-time mode runs 1): each lane is a thread with its
 * own stream that admits work from the shared queue, so the lanes' kernels,
 * result copies and host round trips overlap on the device.  The budget
 * bounds the estimated bytes of every lane's work together. */
gb_status gb_server_set_lanes(gb_server *s, uint32_t lanes);
gb_status gb_server_add_table(gb_server *s, const int32_t *col_types, uint32_t n_cols, const gb_col *cols,
                              uint64_t nrows, uint32_t *table_id);
gb_status gb_server_submit(gb_server *s, uint32_t table_id, uint64_t row_begin, uint64_t row_end,
                           const gb_agg_spec *spec, uint64_t *ticket);
gb_status gb_server_wait(gb_server *s, uint64_t ticket, int64_t timeout_us);
gb_status gb_server_result(gb_server *s, uint64_t ticket, gb_result *out);
gb_status gb_server_query_times(gb_server *s, uint64_t ticket, double *queue_ms, double *exec_ms,
                                uint32_t *batch_size);
gb_status gb_server_release(gb_server *s, uint64_t ticket);
gb_status gb_server_stats(gb_server *s, gb_server_stat *out);
void gb_server_destroy(gb_server *s);

/* Allocation-free GROUP BY for callers that cannot allocate device memory
 * on their query path (an engine that hands out device memory only from
 * its own pre-reserved arena, a plugin host that forbids allocation inside
 * operator calls, or a latency-critical path where cudaMalloc/cudaFree
 * would synchronise the device).  No counterpart in the reference: it is
 * the GPU engine's HashAggregate shape (int64 keys; SUM and COUNT of int64
 * values) on DEVICE buffers, with all scratch in fixed-size device arrays
 * inside the library (about 8.1 MiB, held by every GPU that loads the
 * library until the process exits).  Limits: out_cap <= GB_NOALLOC_MAX_GROUPS
 * and at most that many distinct keys (the key INT64_MIN included), n <=
 * 2^31 rows; beyond them the call fails with a message and writes no result
 * count.  Keys whose hashes cluster are still exact: records of probe runs
 * past the table's bound fold back in a second pass.  The first call on a
 * device resolves the scratch addresses (cudaGetSymbolAddress), so make it
 * before any stream capture.  All calls share the scratch, which each call
 * clears first: calls that overlap on the GPU race and must be serialised.
 * Outputs: *n_out groups in out_keys/out_sums/out_counts (device). */
#define GB_NOALLOC_MAX_GROUPS 131072
gb_status gb_hash_aggregate_noalloc(const int64_t *keys, const int64_t *values, uint64_t n,
                                    int64_t *out_keys, int64_t *out_sums, int64_t *out_counts,
                                    uint64_t out_cap, uint64_t *n_out, void *stream);

/* Pinned host memory helpers (so a caller can stage inputs for the
 * overlapped host→HBM path without linking CUDA itself). */
gb_status gb_host_alloc(void **ptr, size_t bytes);
gb_status gb_host_free(void *ptr);
gb_status gb_device_alloc(void **ptr, size_t bytes);
gb_status gb_device_free(void *ptr);
gb_status gb_memcpy(void *dst, const void *src, size_t bytes, int32_t kind /* 0 h2d,1 d2h,2 d2d */);
gb_status gb_device_sync(void);

#ifdef __cplusplus
}
#endif

#endif /* SLOTHDB_GB300_H */
