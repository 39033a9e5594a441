// gpu_operator.cpp — PhysicalGpuHashAggregate over the C ABI.
//
// Init() resets; the first GetData() pulls every child chunk (the reference's
// ComputeAggregates pulls its child the same way, physical_planner.cpp:
// 7933-8021), stages the vectors in pinned host memory and hands them to
// gb_agg_ingest in batches of STAGE_ROWS rows (the library overlaps the
// host→HBM copies with the aggregation), finalises, and then emits the
// result in VECTOR_SIZE-row chunks like PhysicalHashAggregate::GetData
// (6039-6060).
#include "gpu_operator.hpp"

#include <algorithm>
#include <cstring>

namespace slothdb_gb300 {
namespace engine {

static int type_width(LogicalTypeId t) {
    switch (t) {
    case LogicalTypeId::SMALLINT: return 2;
    case LogicalTypeId::INTEGER: return 4;
    case LogicalTypeId::VARCHAR: return 0;
    default: return 8;
    }
}

#ifndef SLOTHDB_GB300_ENGINE_HEADERS
void ValidityMask::SetInvalid(idx_t i, idx_t capacity) {
    if (words_.empty()) words_.assign((capacity + 63) / 64, ~0ull);
    words_[i >> 6] &= ~(1ull << (i & 63));
}

Vector::Vector(LogicalType type, idx_t capacity) : type_(type), capacity_(capacity) {
    if (type.id == LogicalTypeId::VARCHAR) strings_.resize(capacity);
    else data_.resize(capacity * type_width(type.id));
}

void DataChunk::Initialize(const std::vector<LogicalType> &types, idx_t capacity) {
    data.clear();
    for (const auto &t : types) data.emplace_back(t, capacity);
    count_ = 0;
}

void DataChunk::Reset() {
    for (auto &v : data) v.GetValidity().Reset();
    count_ = 0;
}
#endif

}  // namespace engine

using namespace engine;

static int32_t to_gb(LogicalTypeId t) {
    switch (t) {
    case LogicalTypeId::SMALLINT: return GB_T_SMALLINT;
    case LogicalTypeId::INTEGER: return GB_T_INTEGER;
    case LogicalTypeId::BIGINT: return GB_T_BIGINT;
    case LogicalTypeId::DOUBLE: return GB_T_DOUBLE;
    default: return GB_T_VARCHAR;
    }
}

static void check(gb_status s, const char *what) {
    if (s != GB_OK) throw GpuAggregateError(s, std::string(what) + ": " + gb_last_error());
}

constexpr idx_t STAGE_ROWS = 1 << 20;

// Pinned host buffers for up to STAGE_ROWS rows of every input column.
struct PhysicalGpuHashAggregate::Stage {
    std::vector<void *> cols;       // fixed width: STAGE_ROWS * width; VARCHAR: bytes (grown)
    std::vector<size_t> col_cap;    // bytes allocated per column
    std::vector<int64_t *> offs;    // VARCHAR offsets (STAGE_ROWS + 1)
    std::vector<uint64_t *> valid;  // validity words
    std::vector<bool> has_null;
    std::vector<int64_t> str_used;
    idx_t rows = 0;
    ~Stage() {
        for (void *p : cols) gb_host_free(p);
        for (int64_t *p : offs) gb_host_free(p);
        for (uint64_t *p : valid) gb_host_free(p);
    }
};

PhysicalGpuHashAggregate::PhysicalGpuHashAggregate(std::vector<idx_t> groups, std::vector<GpuAggregate> aggregates,
                                                   std::vector<LogicalType> result_types,
                                                   std::vector<LogicalType> input_types,
                                                   std::vector<GpuPredicate> filters, uint64_t est_groups)
    : GB300_OPERATOR_BASE(std::move(result_types)), groups_(std::move(groups)), aggregates_(std::move(aggregates)),
      input_types_(std::move(input_types)), filters_(std::move(filters)) {
    std::vector<int32_t> ct, gc;
    for (const auto &t : input_types_) ct.push_back(to_gb(type_id(t)));
    for (idx_t g : groups_) gc.push_back((int32_t)g);
    std::vector<gb_agg_desc> ad;
    for (const auto &a : aggregates_) ad.push_back({a.kind, a.column});
    std::vector<gb_filter> fl;
    for (const auto &f : filters_) fl.push_back({f.column, f.op, f.i, f.d});
    gb_agg_spec spec{};
    spec.n_cols = (uint32_t)ct.size();
    spec.col_types = ct.data();
    spec.n_groups = (uint32_t)gc.size();
    spec.group_cols = gc.data();
    spec.n_aggs = (uint32_t)ad.size();
    spec.aggs = ad.data();
    spec.n_filters = (uint32_t)fl.size();
    spec.filters = fl.empty() ? nullptr : fl.data();
    spec.nullable_mask = ~0ull >> (64 - std::min<size_t>(64, std::max<size_t>(1, ct.size())));
    spec.est_groups = est_groups;
    check(gb_agg_create(&spec, &h_), "gb_agg_create");
}

PhysicalGpuHashAggregate::~PhysicalGpuHashAggregate() { gb_agg_destroy(h_); }

void PhysicalGpuHashAggregate::SetTopNHint(idx_t col_idx, bool ascending, idx_t limit) {
    check(gb_agg_set_topn(h_, (uint32_t)col_idx, ascending ? 1 : 0, limit), "SetTopNHint");
}

void PhysicalGpuHashAggregate::SetRowLimit(idx_t n) { check(gb_agg_set_row_limit(h_, n), "SetRowLimit"); }

void PhysicalGpuHashAggregate::Init() {
    for (auto &c : children) c->Init();
    if (computed_) check(gb_agg_reset(h_), "gb_agg_reset");
    computed_ = false;
    emit_pos_ = 0;
}

uint64_t PhysicalGpuHashAggregate::KernelLaunches() const { return gb_agg_kernel_launches(h_); }

void PhysicalGpuHashAggregate::Flush() {
    Stage &S = *stage_;
    if (S.rows == 0) return;
    const size_t nc = input_types_.size();
    std::vector<gb_col> cols(nc);
    for (size_t c = 0; c < nc; c++) {
        cols[c].data = S.cols[c];
        cols[c].validity = S.has_null[c] ? S.valid[c] : nullptr;
        cols[c].offsets = type_id(input_types_[c]) == LogicalTypeId::VARCHAR ? S.offs[c] : nullptr;
    }
    check(gb_agg_ingest(h_, cols.data(), S.rows, GB_MEM_HOST, nullptr), "gb_agg_ingest");
    S.rows = 0;
    for (size_t c = 0; c < nc; c++) {
        S.has_null[c] = false;
        S.str_used[c] = 0;
        if (S.offs[c]) S.offs[c][0] = 0;
        memset(S.valid[c], 0xff, (STAGE_ROWS + 63) / 64 * 8);
    }
}

void PhysicalGpuHashAggregate::ComputeAggregates() {
    const size_t nc = input_types_.size();
    if (!stage_) {
        stage_.reset(new Stage());
        Stage &S = *stage_;
        S.cols.resize(nc, nullptr);
        S.col_cap.resize(nc, 0);
        S.offs.resize(nc, nullptr);
        S.valid.resize(nc, nullptr);
        S.has_null.assign(nc, false);
        S.str_used.assign(nc, 0);
        for (size_t c = 0; c < nc; c++) {
            const bool str = type_id(input_types_[c]) == LogicalTypeId::VARCHAR;
            size_t bytes = str ? (size_t)STAGE_ROWS * 16 : (size_t)STAGE_ROWS * type_width(type_id(input_types_[c]));
            check(gb_host_alloc(&S.cols[c], bytes), "gb_host_alloc");
            S.col_cap[c] = bytes;
            if (str) {
                void *p = nullptr;
                check(gb_host_alloc(&p, (STAGE_ROWS + 1) * 8), "gb_host_alloc");
                S.offs[c] = (int64_t *)p;
                S.offs[c][0] = 0;
            }
            void *v = nullptr;
            check(gb_host_alloc(&v, (STAGE_ROWS + 63) / 64 * 8), "gb_host_alloc");
            S.valid[c] = (uint64_t *)v;
            memset(S.valid[c], 0xff, (STAGE_ROWS + 63) / 64 * 8);
        }
    }
    Stage &S = *stage_;
    DataChunk chunk;
    for (auto &child : children) {
        for (;;) {
            chunk.Reset();
            if (!child->GetData(chunk)) break;
            const idx_t n = chunk.size();
            if (chunk.ColumnCount() != nc) throw GpuAggregateError(GB_ERR_INVALID, "child chunk width mismatch");
            for (idx_t r0 = 0; r0 < n;) {
                const idx_t take = std::min<idx_t>(n - r0, STAGE_ROWS - S.rows);
                for (size_t c = 0; c < nc; c++) {
                    const Vector &v = chunk.GetVector(c);
                    if (type_id(input_types_[c]) == LogicalTypeId::VARCHAR) {
                        for (idx_t i = 0; i < take; i++) {
                            const char *sp = nullptr;
                            size_t sn = 0;
                            string_at(v, r0 + i, &sp, &sn);
                            size_t need = (size_t)S.str_used[c] + sn;
                            if (need > S.col_cap[c]) {  // grow the pinned byte buffer
                                void *p = nullptr;
                                check(gb_host_alloc(&p, need * 2), "gb_host_alloc");
                                memcpy(p, S.cols[c], (size_t)S.str_used[c]);
                                gb_host_free(S.cols[c]);
                                S.cols[c] = p;
                                S.col_cap[c] = need * 2;
                            }
                            if (sn) memcpy((char *)S.cols[c] + S.str_used[c], sp, sn);
                            S.str_used[c] += (int64_t)sn;
                            S.offs[c][S.rows + i + 1] = S.str_used[c];
                        }
                    } else {
                        const int w = type_width(type_id(input_types_[c]));
                        memcpy((char *)S.cols[c] + S.rows * w, v.GetData<char>() + r0 * w, take * w);
                    }
                    if (!v.GetValidity().AllValid()) {
                        for (idx_t i = 0; i < take; i++)
                            if (!v.GetValidity().RowIsValid(r0 + i)) {
                                const idx_t d = S.rows + i;
                                S.valid[c][d >> 6] &= ~(1ull << (d & 63));
                                S.has_null[c] = true;
                            }
                    }
                }
                S.rows += take;
                r0 += take;
                if (S.rows == STAGE_ROWS) Flush();
            }
        }
    }
    Flush();
    check(gb_agg_finalize(h_, nullptr), "gb_agg_finalize");
    check(gb_agg_result(h_, &res_), "gb_agg_result");
    // the operator returns exactly the declared result types (binder.cpp:1345-1391)
    const auto &rt = GetTypes();
    if (rt.size() != res_.n_cols) throw GpuAggregateError(GB_ERR_INVALID, "result_types width differs from the plan's");
    for (uint32_t c = 0; c < res_.n_cols; c++)
        if (to_gb(type_id(rt[c])) != res_.types[c])
            throw GpuAggregateError(GB_ERR_INVALID, "result type of output slot " + std::to_string(c) +
                                                        " differs from the plan's");
}

bool PhysicalGpuHashAggregate::GetData(DataChunk &result) {
    if (!computed_) {
        ComputeAggregates();
        computed_ = true;
    }
    if (emit_pos_ >= res_.n_rows) return false;
    result.Initialize(GetTypes());
    const idx_t count = std::min<idx_t>(VECTOR_SIZE, res_.n_rows - emit_pos_);
    for (uint32_t c = 0; c < res_.n_cols; c++) {
        if (!needed_.empty() && c < needed_.size() && !needed_[c]) continue;
        Vector &v = result.GetVector(c);
        const int32_t t = res_.types[c];
        if (t == GB_T_VARCHAR) {
            const int64_t *o = res_.offsets[c];
            const char *b = (const char *)res_.data[c];
            for (idx_t i = 0; i < count; i++)
                set_string(v, i, b + o[emit_pos_ + i], (size_t)(o[emit_pos_ + i + 1] - o[emit_pos_ + i]));
        } else {
            const int w = t == GB_T_SMALLINT ? 2 : (t == GB_T_INTEGER ? 4 : 8);
            memcpy(v.GetData<char>(), (const char *)res_.data[c] + emit_pos_ * w, count * w);
        }
        const uint64_t *vw = res_.validity ? res_.validity[c] : nullptr;
        if (vw)
            for (idx_t i = 0; i < count; i++) {
                const idx_t r = emit_pos_ + i;
                if (!((vw[r >> 6] >> (r & 63)) & 1ull)) set_invalid(v.GetValidity(), i, VECTOR_SIZE);
            }
    }
    emit_pos_ += count;
    result.SetCardinality(count);
    return count > 0;
}

}  // namespace slothdb_gb300
