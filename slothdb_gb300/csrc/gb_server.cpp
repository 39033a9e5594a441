// gb_server.cpp — a served stream of GROUP BY queries over tables resident
// in HBM.
//
// The reference has no server: each query is one Connection::Query call
// that plans and runs its own PhysicalHashAggregate (physical_planner.cpp:
// 14356-14362) on the caller's thread.  Here one dispatcher thread owns the
// GPU and executes the queued queries with continuous batching:
//
//   submit   (any thread) appends a query (table, row range, plan) to a FIFO
//            queue and returns a ticket;
//   dispatch the dispatcher takes queued queries in arrival order while the
//            sum of their estimated device bytes (gb_agg_estimate_bytes)
//            stays within the admission budget and the batch holds at most
//            max_batch queries; a query whose estimate alone exceeds the
//            budget is rejected with GB_ERR_BUDGET;
//   execute  the admitted queries run as one gb_batch (one pass of a few
//            persistent kernels), except high-cardinality queries (estimated
//            groups >= 2^20), which run one by one on their own handle (the
//            radix path), and queries with a VARCHAR in a pair key, which run
//            alone on a hash handle; in mode 1 every query runs alone on its
//            own handle (the one-at-a-time baseline);
//   complete results are copied to host memory owned by the ticket, the
//            ticket records queue / execution times, and waiters wake up.
//
// Queries that arrive while a batch executes form the next batch.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/slothdb_gb300.h"

namespace gb {
void set_error(const char *fmt, ...);  // the library's thread-local error message
}

namespace {

using gb::set_error;
typedef unsigned long long u64;

constexpr u64 RADIX_GROUPS = 1ull << 20;

u64 now_ns() {
    return (u64)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

int type_bytes(int t) {
    switch (t) {
    case GB_T_SMALLINT: return 2;
    case GB_T_INTEGER: return 4;
    default: return 8;
    }
}

struct Table {
    std::vector<int32_t> types;
    std::vector<gb_col> cols;
    u64 nrows = 0;
};

// Page-locked host blocks recycled between results (size classes of powers
// of two), so a result is copied once, device → pinned host, at full link
// bandwidth, with no allocation in steady state.
class PinnedPool {
public:
    struct Block {
        void *p;
        size_t cls;
    };
    Block get(size_t bytes) {
        size_t cls = 4096;
        while (cls < bytes) cls <<= 1;
        {
            std::lock_guard<std::mutex> lk(mu_);
            auto it = free_.find(cls);
            if (it != free_.end()) {
                Block b{it->second, cls};
                free_.erase(it);
                free_bytes_ -= cls;
                return b;
            }
        }
        void *p = nullptr;
        if (cudaMallocHost(&p, cls) != cudaSuccess) {
            (void)cudaGetLastError();
            return {nullptr, 0};
        }
        return {p, cls};
    }
    void put(const Block &b) {
        if (!b.p) return;
        std::lock_guard<std::mutex> lk(mu_);
        if (free_bytes_ + b.cls > kKeepBytes) {
            cudaFreeHost(b.p);
            return;
        }
        free_.emplace(b.cls, b.p);
        free_bytes_ += b.cls;
    }
    ~PinnedPool() {
        for (auto &e : free_) cudaFreeHost(e.second);
    }

private:
    static constexpr size_t kKeepBytes = (size_t)8 << 30;  // idle pinned memory kept for reuse
    std::mutex mu_;
    std::multimap<size_t, void *> free_;
    size_t free_bytes_ = 0;
};

// A host copy of one result, in pinned blocks of the pool.
struct HostResult {
    u64 n_rows = 0;
    u64 bytes = 0;  // device→host bytes copied
    std::vector<int32_t> types;
    std::vector<PinnedPool::Block> blocks;
    std::vector<const void *> data_p;
    std::vector<const int64_t *> offs_p;
    std::vector<const uint64_t *> valid_p;
};

struct Query {
    u64 ticket = 0;
    uint32_t table = 0;
    u64 r0 = 0, r1 = 0;
    std::vector<int32_t> col_types, group_cols;
    std::vector<gb_agg_desc> aggs;
    std::vector<gb_filter> filters;
    std::vector<std::vector<uint8_t>> literals;  // the filters' IN sets / strings (the caller's may be gone)
    u64 nullable_mask = 0, est_groups = 0;
    u64 est_bytes = 0;
    bool done = false;
    gb_status status = GB_OK;
    std::string error;
    HostResult res;
    u64 t_submit = 0, t_start = 0, t_done = 0;
    uint32_t batch_size = 0;

    // queries the batch kernels do not take (a VARCHAR in a pair key) run
    // alone on their own handle
    bool batch_refused() const {
        if (group_cols.size() == 2)
            for (int32_t g : group_cols)
                if (col_types[g] == GB_T_VARCHAR) return true;
        return false;
    }

    gb_agg_spec spec() const {
        gb_agg_spec s{};
        s.n_cols = (uint32_t)col_types.size();
        s.col_types = col_types.data();
        s.n_groups = (uint32_t)group_cols.size();
        s.group_cols = group_cols.data();
        s.n_aggs = (uint32_t)aggs.size();
        s.aggs = aggs.data();
        s.n_filters = (uint32_t)filters.size();
        s.filters = filters.empty() ? nullptr : filters.data();
        s.nullable_mask = nullable_mask;
        s.est_groups = est_groups;
        return s;
    }
};


// One execution lane: its own stream, batch object and pool of lone
// handles; lanes run on their own threads, so a lane's host work (result
// copies, reservations, syncs) overlaps another lane's kernels.
struct Lane {
    cudaStream_t stream = nullptr;
    gb_batch *batch = nullptr;                              // reused: gb_batch_clear keeps its handles pooled
    std::unordered_multimap<std::string, gb_agg *> alone;   // idle handles of queries run alone, by plan shape
    std::deque<std::string> alone_order;
};

}  // namespace

struct gb_server {
    u64 budget = 0;
    uint32_t max_batch = 256;
    int mode = 0;  // 0 continuous batching, 1 one at a time
    std::vector<Table> tables;
    std::deque<Query *> queue;
    std::unordered_map<u64, std::unique_ptr<Query>> all;
    u64 next_ticket = 1;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::vector<std::thread> workers;
    bool stopping = false;
    bool started = false;
    int device = 0;
    uint32_t n_lanes = 1;
    std::vector<Lane> lanes;
    PinnedPool pinned;  // host result blocks
    u64 inflight_bytes = 0;  // estimated bytes of the queries the lanes are running
    int active = 0;          // lanes running work (busy time is the union)
    u64 busy_since = 0;
    // statistics
    u64 n_batches = 0, n_done = 0, n_rejected = 0, n_failed = 0, peak_admitted = 0, busy_ns = 0;
    // written by the dispatcher outside the lock, read by gb_server_stats
    std::atomic<u64> launches{0}, result_bytes{0};
};

namespace {

// Copy a device-resident result into pinned blocks: fixed-width columns,
// validity words and VARCHAR offsets first, then the string bytes.
gb_status copy_result_device(const gb_result &r, HostResult &out, PinnedPool &pool, cudaStream_t st) {
    const u64 n = r.n_rows;
    out.n_rows = n;
    out.types.assign(r.types, r.types + r.n_cols);
    out.data_p.assign(r.n_cols, nullptr);
    out.offs_p.assign(r.n_cols, nullptr);
    out.valid_p.assign(r.n_cols, nullptr);
    const u64 vw = (n + 63) / 64;
    out.bytes = 0;
    auto take = [&](size_t bytes) -> void * {
        PinnedPool::Block b = pool.get(std::max<size_t>(bytes, 8));
        if (b.p) out.blocks.push_back(b);
        return b.p;
    };
    for (uint32_t c = 0; c < r.n_cols; c++) {
        uint64_t *v = (uint64_t *)take(vw * 8);
        if (!v) return GB_ERR_OOM;
        if (r.validity && r.validity[c]) {
            if (vw && cudaMemcpyAsync(v, r.validity[c], vw * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess)
                return GB_ERR_CUDA;
            out.bytes += vw * 8;
        } else {
            for (u64 i = 0; i < vw; i++) v[i] = ~0ull;
        }
        out.valid_p[c] = v;
        if (r.types[c] == GB_T_VARCHAR) {
            int64_t *o = (int64_t *)take((n + 1) * 8);
            if (!o) return GB_ERR_OOM;
            if (cudaMemcpyAsync(o, r.offsets[c], (n + 1) * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess)
                return GB_ERR_CUDA;
            out.bytes += (n + 1) * 8;
            out.offs_p[c] = o;
        } else if (n) {
            void *d = take(n * (u64)type_bytes(r.types[c]));
            if (!d) return GB_ERR_OOM;
            if (cudaMemcpyAsync(d, r.data[c], n * (u64)type_bytes(r.types[c]), cudaMemcpyDeviceToHost, st) !=
                cudaSuccess)
                return GB_ERR_CUDA;
            out.bytes += n * (u64)type_bytes(r.types[c]);
            out.data_p[c] = d;
        }
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) return GB_ERR_CUDA;
    for (uint32_t c = 0; c < r.n_cols; c++) {
        if (r.types[c] != GB_T_VARCHAR) continue;
        const int64_t *o = out.offs_p[c];
        const u64 nb = (u64)(o[n] - o[0]);
        void *d = take(nb + 8);
        if (!d) return GB_ERR_OOM;
        if (nb && cudaMemcpyAsync(d, (const uint8_t *)r.data[c] + o[0], nb, cudaMemcpyDeviceToHost, st) != cudaSuccess)
            return GB_ERR_CUDA;
        out.bytes += nb;
        out.data_p[c] = d;
        if (o[0]) {  // offsets relative to the copied bytes
            int64_t *w = const_cast<int64_t *>(o);
            const int64_t b0 = o[0];
            for (u64 i = 0; i <= n; i++) w[i] -= b0;
        }
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) return GB_ERR_CUDA;
    return GB_OK;
}

void release_result(HostResult &r, PinnedPool &pool) {
    for (const auto &b : r.blocks) pool.put(b);
    r.blocks.clear();
}

// The columns of rows [r0, r1) of a table (validity slices start at a
// multiple of 64 rows; checked at submit).
std::vector<gb_col> slice_cols(const Table &t, u64 r0) {
    std::vector<gb_col> c(t.cols.size());
    for (size_t i = 0; i < t.cols.size(); i++) {
        const gb_col &s = t.cols[i];
        c[i] = s;
        if (t.types[i] == GB_T_VARCHAR) {
            c[i].offsets = s.offsets + r0;  // offsets index the column's whole byte buffer
        } else {
            c[i].data = (const uint8_t *)s.data + r0 * (u64)type_bytes(t.types[i]);
        }
        if (s.validity) c[i].validity = s.validity + r0 / 64;
    }
    return c;
}

void finish(Query *q, gb_status st, const char *msg) {
    q->status = st;
    if (st != GB_OK) q->error = msg ? msg : "";
}

// Pool key of a query run alone: plan shape without filter constants, and
// the estimate's power-of-two bucket.
std::string alone_key(const Query *q) {
    std::string k;
    auto put = [&](const void *p, size_t n) { k.append((const char *)p, n); };
    put(q->col_types.data(), 4 * q->col_types.size());
    k.push_back('|');
    put(q->group_cols.data(), 4 * q->group_cols.size());
    k.push_back('|');
    put(q->aggs.data(), sizeof(gb_agg_desc) * q->aggs.size());
    k.push_back('|');
    for (const gb_filter &f : q->filters) {
        put(&f.col, 4);
        put(&f.op, 4);
    }
    put(&q->nullable_mask, 8);
    u64 b = 1;
    while (b < q->est_groups) b <<= 1;
    put(&b, 8);
    return k;
}

constexpr size_t ALONE_POOL_MAX = 8;  // idle lone handles kept (a radix handle holds GBs)

// One query on its own handle (the radix path for high-cardinality keys,
// and every query in one-at-a-time mode).  Handles are pooled by plan shape
// and reused with new predicates (gb_agg_reset + gb_agg_set_filters).
void run_alone(gb_server *s, Lane &L, Query *q) {
    const gb_agg_spec sp = q->spec();
    gb_agg *h = nullptr;
    gb_status st = GB_OK;
    const std::string key = alone_key(q);
    auto it = L.alone.find(key);
    if (it != L.alone.end()) {
        h = it->second;
        L.alone.erase(it);
        st = gb_agg_reset(h);
        if (st == GB_OK) st = gb_agg_set_filters(h, sp.filters, sp.n_filters);
    } else {
        st = gb_agg_create(&sp, &h);
    }
    if (st == GB_OK) {
        std::vector<gb_col> cols = slice_cols(s->tables[q->table], q->r0);
        st = gb_agg_ingest(h, cols.data(), q->r1 - q->r0, GB_MEM_DEVICE, L.stream);
        if (st == GB_OK) st = gb_agg_finalize(h, L.stream);
        gb_result r{};
        if (st == GB_OK) st = gb_agg_result_device(h, &r);
        if (st == GB_OK) st = copy_result_device(r, q->res, s->pinned, L.stream);
        if (st == GB_OK) s->result_bytes += q->res.bytes;
        s->launches += gb_agg_kernel_launches(h);
    }
    finish(q, st, st ? gb_last_error() : nullptr);
    if (!h) return;
    if (st != GB_OK) {
        gb_agg_destroy(h);
        return;
    }
    L.alone.emplace(key, h);
    L.alone_order.push_back(key);
    while (L.alone.size() > ALONE_POOL_MAX && !L.alone_order.empty()) {
        auto e = L.alone.find(L.alone_order.front());
        L.alone_order.pop_front();
        if (e != L.alone.end()) {
            gb_agg_destroy(e->second);
            L.alone.erase(e);
        }
    }
}

void run_batch(gb_server *s, Lane &L, std::vector<Query *> &qs) {
    gb_status st = GB_OK;
    if (!L.batch) {
        st = gb_batch_create(&L.batch);
        if (st == GB_OK) gb_batch_set_option(L.batch, "graph", 0);  // one-off batches: capture costs more
    } else {
        st = gb_batch_clear(L.batch);
    }
    if (st) {
        for (Query *q : qs) finish(q, st, gb_last_error());
        return;
    }
    gb_batch *b = L.batch;
    std::vector<Query *> in;
    for (Query *q : qs) {
        const gb_agg_spec sp = q->spec();
        std::vector<gb_col> cols = slice_cols(s->tables[q->table], q->r0);
        uint32_t idx = 0;
        gb_status a = gb_batch_add(b, &sp, cols.data(), q->r1 - q->r0, &idx);
        if (a) finish(q, a, gb_last_error());
        else in.push_back(q);
    }
    if (!in.empty()) {
        const u64 l0 = gb_batch_kernel_launches(b);
        st = gb_batch_run(b, L.stream);
        for (size_t i = 0; i < in.size(); i++) {
            gb_result r{};
            gb_status rs = st ? st : gb_batch_result_device(b, (uint32_t)i, &r);
            if (rs == GB_OK) rs = copy_result_device(r, in[i]->res, s->pinned, L.stream);
            if (rs == GB_OK) s->result_bytes += in[i]->res.bytes;
            finish(in[i], rs, rs ? gb_last_error() : nullptr);
        }
        s->launches += gb_batch_kernel_launches(b) - l0;
    }
}

// A query that takes the lone-handle path (radix-sized estimate, a VARCHAR
// in a pair key, or one-at-a-time mode).
bool runs_alone(const gb_server *s, const Query *q) {
    return s->mode == 1 || q->est_groups >= RADIX_GROUPS || q->batch_refused();
}

// One lane's loop: admit queries from the front of the queue (FIFO) while
// their estimated bytes fit the budget beside what the other lanes run — at
// most max_batch small queries (one batch) and at most one lone query per
// turn, so lanes share the large queries — then run them.
void dispatcher(gb_server *s, int lane) {
    cudaSetDevice(s->device);
    Lane &L = s->lanes[lane];
    for (;;) {
        std::vector<Query *> big, small;
        u64 sum = 0;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            for (;;) {
                // reject what can never fit, then admit what fits now
                while (!s->queue.empty() && s->queue.front()->est_bytes > s->budget) {
                    Query *q = s->queue.front();
                    s->queue.pop_front();
                    finish(q, GB_ERR_BUDGET, "estimated device bytes exceed the admission budget");
                    q->t_start = q->t_done = now_ns();
                    q->done = true;
                    s->n_rejected++;
                }
                while (!s->queue.empty() && small.size() < s->max_batch) {
                    Query *q = s->queue.front();
                    if (q->est_bytes > s->budget) break;  // rejected on the next pass
                    if (s->inflight_bytes + sum + q->est_bytes > s->budget) break;
                    const bool alone = runs_alone(s, q);
                    if (alone && !big.empty()) break;
                    s->queue.pop_front();
                    (alone ? big : small).push_back(q);
                    sum += q->est_bytes;
                }
                s->cv_done.notify_all();
                if (!big.empty() || !small.empty()) break;
                if (s->stopping && s->queue.empty()) return;  // stopping and drained
                s->cv_work.wait(lk);
            }
            s->inflight_bytes += sum;
            s->peak_admitted = std::max(s->peak_admitted, s->inflight_bytes);
            if (s->active++ == 0) s->busy_since = now_ns();
        }
        const u64 t0 = now_ns();
        // a query's start / done times: its batch's, or its own when it runs alone
        auto complete = [&](std::vector<Query *> &qs, u64 ts, u64 td) {
            std::lock_guard<std::mutex> lk(s->mu);
            for (Query *q : qs) {
                q->t_start = ts;
                q->t_done = td;
                q->done = true;
                if (q->status) s->n_failed++;
                s->n_done++;
            }
        };
        if (!small.empty()) {
            for (Query *q : small) q->batch_size = (uint32_t)small.size();
            run_batch(s, L, small);
            complete(small, t0, now_ns());
            s->cv_done.notify_all();
        }
        for (Query *q : big) {
            std::vector<Query *> one{q};
            q->batch_size = 1;
            const u64 ts = now_ns();
            run_alone(s, L, q);
            complete(one, ts, now_ns());
            s->cv_done.notify_all();
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->n_batches++;
            s->inflight_bytes -= sum;
            if (--s->active == 0) s->busy_ns += now_ns() - s->busy_since;
        }
        s->cv_work.notify_all();  // budget freed: another lane may admit
    }
}

}  // namespace

extern "C" {

gb_status gb_server_create(uint64_t budget_bytes, uint32_t max_batch, int32_t mode, gb_server **out) {
    if (!out || budget_bytes == 0 || max_batch == 0 || (mode != 0 && mode != 1)) {
        set_error("invalid server arguments");
        return GB_ERR_INVALID;
    }
    gb_server *s = new gb_server();
    s->budget = budget_bytes;
    s->max_batch = max_batch;
    s->mode = mode;
    s->n_lanes = mode == 0 ? 2 : 1;
    cudaGetDevice(&s->device);
    *out = s;
    return GB_OK;
}

gb_status gb_server_set_lanes(gb_server *s, uint32_t lanes) {
    if (!s || lanes == 0 || lanes > 8) {
        set_error("lanes must be 1..8");
        return GB_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->started) {
        set_error("lanes are set before the first query");
        return GB_ERR_STATE;
    }
    if (s->mode == 1 && lanes != 1) {
        set_error("one-at-a-time mode runs one lane");
        return GB_ERR_INVALID;
    }
    s->n_lanes = lanes;
    return GB_OK;
}

gb_status gb_server_add_table(gb_server *s, const int32_t *col_types, uint32_t n_cols, const gb_col *cols,
                              uint64_t nrows, uint32_t *table_id) {
    if (!s || !col_types || !cols || n_cols == 0 || !table_id) return GB_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->started) {
        set_error("tables are registered before the first query");
        return GB_ERR_STATE;
    }
    Table t;
    t.types.assign(col_types, col_types + n_cols);
    t.cols.assign(cols, cols + n_cols);
    t.nrows = nrows;
    s->tables.push_back(t);
    *table_id = (uint32_t)(s->tables.size() - 1);
    return GB_OK;
}

gb_status gb_server_submit(gb_server *s, uint32_t table_id, uint64_t row_begin, uint64_t row_end,
                           const gb_agg_spec *spec, uint64_t *ticket) {
    if (!s || !spec || !ticket) return GB_ERR_INVALID;
    if (table_id >= s->tables.size()) {
        set_error("unknown table %u", table_id);
        return GB_ERR_INVALID;
    }
    const Table &t = s->tables[table_id];
    if (row_begin > row_end || row_end > t.nrows) {
        set_error("row range [%llu, %llu) outside the table", (u64)row_begin, (u64)row_end);
        return GB_ERR_INVALID;
    }
    if (spec->n_cols != t.types.size() || memcmp(spec->col_types, t.types.data(), 4 * t.types.size()) != 0) {
        set_error("spec columns do not match the table's");
        return GB_ERR_INVALID;
    }
    bool has_valid = false;
    for (const gb_col &c : t.cols) has_valid |= c.validity != nullptr;
    if (has_valid && (row_begin % 64) != 0) {
        set_error("a table with validity masks is sliced at multiples of 64 rows");
        return GB_ERR_INVALID;
    }
    auto q = std::make_unique<Query>();
    q->table = table_id;
    q->r0 = row_begin;
    q->r1 = row_end;
    q->col_types.assign(spec->col_types, spec->col_types + spec->n_cols);
    q->group_cols.assign(spec->group_cols, spec->group_cols + spec->n_groups);
    q->aggs.assign(spec->aggs, spec->aggs + spec->n_aggs);
    if (spec->n_filters) q->filters.assign(spec->filters, spec->filters + spec->n_filters);
    q->literals.resize(q->filters.size());
    for (size_t i = 0; i < q->filters.size(); i++) {
        gb_filter &f = q->filters[i];
        if (f.op < GB_CMP_IN || !f.data) continue;
        const size_t bytes = f.op == GB_CMP_IN ? f.n * sizeof(int64_t) : f.n;
        q->literals[i].assign((const uint8_t *)f.data, (const uint8_t *)f.data + bytes);
        f.data = q->literals[i].data();
    }
    q->nullable_mask = spec->nullable_mask;
    q->est_groups = spec->est_groups;
    const gb_agg_spec sp = q->spec();
    uint64_t bytes = 0;
    gb_status st = gb_agg_estimate_bytes(&sp, row_end - row_begin, &bytes);
    if (st) return st;  // an invalid plan is reported at submit
    q->est_bytes = bytes;
    q->t_submit = now_ns();
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stopping) return GB_ERR_STATE;
    q->ticket = s->next_ticket++;
    *ticket = q->ticket;
    s->queue.push_back(q.get());
    s->all[q->ticket] = std::move(q);
    if (!s->started) {
        s->lanes.resize(s->n_lanes);
        for (Lane &L : s->lanes)
            if (cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking) != cudaSuccess) {
                s->all.erase(*ticket);
                s->queue.pop_back();
                set_error("cudaStreamCreate failed");
                return GB_ERR_CUDA;
            }
        s->started = true;
        for (uint32_t i = 0; i < s->n_lanes; i++) s->workers.emplace_back(dispatcher, s, (int)i);
    }
    s->cv_work.notify_one();
    return GB_OK;
}

gb_status gb_server_wait(gb_server *s, uint64_t ticket, int64_t timeout_us) {
    if (!s) return GB_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return GB_ERR_INVALID;
    Query *q = it->second.get();
    auto pred = [&] { return q->done; };
    if (timeout_us < 0) s->cv_done.wait(lk, pred);
    else if (!s->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), pred)) return GB_ERR_TIMEOUT;
    if (q->status) set_error("%s", q->error.c_str());
    return q->status;
}

gb_status gb_server_result(gb_server *s, uint64_t ticket, gb_result *out) {
    if (!s || !out) return GB_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return GB_ERR_INVALID;
    Query *q = it->second.get();
    if (!q->done) return GB_ERR_STATE;
    if (q->status) {
        set_error("%s", q->error.c_str());
        return q->status;
    }
    HostResult &r = q->res;
    out->n_rows = r.n_rows;
    out->n_cols = (uint32_t)r.types.size();
    out->types = r.types.data();
    out->data = r.data_p.data();
    out->offsets = r.offs_p.data();
    out->validity = r.valid_p.data();  // pinned blocks owned by the ticket
    return GB_OK;
}

gb_status gb_server_query_times(gb_server *s, uint64_t ticket, double *queue_ms, double *exec_ms,
                                uint32_t *batch_size) {
    if (!s) return GB_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return GB_ERR_INVALID;
    Query *q = it->second.get();
    if (!q->done) return GB_ERR_STATE;
    if (queue_ms) *queue_ms = (double)(q->t_start - q->t_submit) / 1e6;
    if (exec_ms) *exec_ms = (double)(q->t_done - q->t_start) / 1e6;
    if (batch_size) *batch_size = q->batch_size;
    return GB_OK;
}

gb_status gb_server_release(gb_server *s, uint64_t ticket) {
    if (!s) return GB_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return GB_ERR_INVALID;
    if (!it->second->done) return GB_ERR_STATE;
    release_result(it->second->res, s->pinned);
    s->all.erase(it);
    return GB_OK;
}

gb_status gb_server_stats(gb_server *s, gb_server_stat *out) {
    if (!s || !out) return GB_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    out->batches = s->n_batches;
    out->completed = s->n_done;
    out->rejected = s->n_rejected;
    out->failed = s->n_failed;
    out->queued = s->queue.size();
    out->peak_admitted_bytes = s->peak_admitted;
    out->busy_ms = (double)s->busy_ns / 1e6;
    out->kernel_launches = s->launches.load();
    out->result_bytes = s->result_bytes.load();
    return GB_OK;
}

void gb_server_destroy(gb_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cv_work.notify_all();
    for (std::thread &t : s->workers)
        if (t.joinable()) t.join();
    for (Lane &L : s->lanes) {
        if (L.batch) gb_batch_destroy(L.batch);
        for (auto &e : L.alone) gb_agg_destroy(e.second);
        if (L.stream) cudaStreamDestroy(L.stream);
    }
    for (auto &e : s->all) release_result(e.second->res, s->pinned);
    delete s;
}

}  // extern "C"
