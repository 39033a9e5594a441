// gpu_operator.hpp — the GROUP BY operator in the shape of SlothDB's
// physical-operator interface, running on the GB300 path through the C ABI.
//
// Mirrors, with the same names and argument meaning:
//   PhysicalOperator        include/slothdb/execution/physical_operator.hpp:22-65
//                           (Init, pull-based GetData(DataChunk&) → false when
//                           done, SetTopNHint(col_idx, ascending, limit) in
//                           output-slot space, SetRowLimit, SetNeededOutputs,
//                           children)
//   PhysicalHashAggregate   src/execution/physical_planner.cpp:6009-6060
//                           (ctor (groups, aggregates, result_types); output
//                           slots [group cols…, agg cols…]; Init resets;
//                           GetData computes on first call, then emits
//                           VECTOR_SIZE-row chunks)
//   DataChunk / Vector /    include/slothdb/common/types/data_chunk.hpp:10-55,
//   ValidityMask            vector.hpp:65-120, validity_mask.hpp:9-69
//
// The engine types below are minimal stand-ins with the reference's names so
// that this operator and its tests compile on their own.  Built with
// SLOTHDB_GB300_ENGINE_HEADERS defined and the engine's include directory on
// the path, the operator uses the engine's own types instead
// (include/slothdb/common/types/data_chunk.hpp, vector.hpp, validity_mask.hpp,
// string_type.hpp, include/slothdb/execution/physical_operator.hpp); the few
// places where the two differ go through the adapters below.
// Group keys and aggregate arguments are input column indices — the planner
// places a projection below the operator for expressions.  Failures throw
// GpuAggregateError (SlothDB converts it to InternalException); there is no
// CPU fallback.
#pragma once

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/slothdb_gb300.h"

#ifdef SLOTHDB_GB300_ENGINE_HEADERS
#include "slothdb/common/types/data_chunk.hpp"
#include "slothdb/execution/physical_operator.hpp"

namespace slothdb_gb300 {
namespace engine {

using slothdb::DataChunk;
using slothdb::idx_t;
using slothdb::LogicalType;
using slothdb::LogicalTypeId;
using slothdb::PhysicalOperator;
using slothdb::ValidityMask;
using slothdb::Vector;
using slothdb::VECTOR_SIZE;

inline LogicalTypeId type_id(const LogicalType &t) { return t.id(); }
// VARCHAR values are string_t views; written strings live in the vector's
// string buffer
inline void string_at(const Vector &v, idx_t i, const char **p, size_t *n) {
    const slothdb::string_t &s = v.GetData<slothdb::string_t>()[i];
    *p = s.GetData();
    *n = s.GetSize();
}
inline void set_string(Vector &v, idx_t i, const char *p, size_t n) {
    const char *q = v.GetStringBuffer().AddString(p, (idx_t)n);
    v.GetData<slothdb::string_t>()[i] = slothdb::string_t(q, (uint32_t)n);
}
inline void set_invalid(ValidityMask &m, idx_t i, idx_t) { m.SetInvalid(i); }

}  // namespace engine
// PhysicalHashAggregate passes TABLE_SCAN (physical_planner.cpp:6014): the
// engine's PhysicalOperatorType has no aggregate member
#define GB300_OPERATOR_BASE(types) engine::PhysicalOperator(slothdb::PhysicalOperatorType::TABLE_SCAN, types)
#else
namespace slothdb_gb300 {
namespace engine {

typedef uint64_t idx_t;
constexpr idx_t VECTOR_SIZE = 2048;  // constants.hpp:16

enum class LogicalTypeId : uint8_t { SMALLINT, INTEGER, BIGINT, DOUBLE, VARCHAR };

struct LogicalType {
    LogicalTypeId id;
    LogicalType(LogicalTypeId i = LogicalTypeId::INTEGER) : id(i) {}
    bool operator==(const LogicalType &o) const { return id == o.id; }
};

// 64-bit words, bit (i % 64) of word (i / 64) set = row i valid; empty = all valid.
class ValidityMask {
public:
    bool AllValid() const { return words_.empty(); }
    bool RowIsValid(idx_t i) const { return words_.empty() || ((words_[i >> 6] >> (i & 63)) & 1ull); }
    void SetInvalid(idx_t i, idx_t capacity);
    void Reset() { words_.clear(); }
    const uint64_t *Data() const { return words_.empty() ? nullptr : words_.data(); }

private:
    std::vector<uint64_t> words_;
};

// A flat vector: fixed-width values in `data`, VARCHAR as std::string values.
class Vector {
public:
    explicit Vector(LogicalType type, idx_t capacity = VECTOR_SIZE);
    const LogicalType &GetType() const { return type_; }
    template <class T> T *GetData() { return reinterpret_cast<T *>(data_.data()); }
    template <class T> const T *GetData() const { return reinterpret_cast<const T *>(data_.data()); }
    std::vector<std::string> &Strings() { return strings_; }
    const std::vector<std::string> &Strings() const { return strings_; }
    ValidityMask &GetValidity() { return validity_; }
    const ValidityMask &GetValidity() const { return validity_; }
    idx_t Capacity() const { return capacity_; }

private:
    LogicalType type_;
    idx_t capacity_;
    std::vector<uint8_t> data_;
    std::vector<std::string> strings_;
    ValidityMask validity_;
};

class DataChunk {
public:
    void Initialize(const std::vector<LogicalType> &types, idx_t capacity = VECTOR_SIZE);
    idx_t ColumnCount() const { return (idx_t)data.size(); }
    idx_t size() const { return count_; }
    void SetCardinality(idx_t count) { count_ = count; }
    void Reset();
    Vector &GetVector(idx_t c) { return data[c]; }
    const Vector &GetVector(idx_t c) const { return data[c]; }
    std::vector<Vector> data;

private:
    idx_t count_ = 0;
};

class PhysicalOperator {
public:
    explicit PhysicalOperator(std::vector<LogicalType> types) : types_(std::move(types)) {}
    virtual ~PhysicalOperator() = default;
    const std::vector<LogicalType> &GetTypes() const { return types_; }
    virtual void Init() {}
    virtual bool GetData(DataChunk &result) = 0;
    virtual void SetNeededOutputs(const std::vector<bool> &) {}
    virtual void SetRowLimit(idx_t) {}
    virtual void SetTopNHint(idx_t, bool, idx_t) {}
    std::vector<std::unique_ptr<PhysicalOperator>> children;

private:
    std::vector<LogicalType> types_;
};

}  // namespace engine

namespace engine {
inline LogicalTypeId type_id(const LogicalType &t) { return t.id; }
inline void string_at(const Vector &v, idx_t i, const char **p, size_t *n) {
    const std::string &s = v.Strings()[i];
    *p = s.data();
    *n = s.size();
}
inline void set_string(Vector &v, idx_t i, const char *p, size_t n) { v.Strings()[i].assign(p, n); }
inline void set_invalid(ValidityMask &m, idx_t i, idx_t capacity) { m.SetInvalid(i, capacity); }
}  // namespace engine
#define GB300_OPERATOR_BASE(types) engine::PhysicalOperator(types)
#endif

class GpuAggregateError : public std::runtime_error {
public:
    GpuAggregateError(gb_status s, const std::string &what) : std::runtime_error(what), status(s) {}
    gb_status status;
};

// One aggregate: kind + input column (-1 for COUNT(*)).
struct GpuAggregate {
    gb_agg_kind kind;
    int32_t column;
};

// col OP constant (integer columns compare in int64, DOUBLE against d).
struct GpuPredicate {
    int32_t column;
    gb_cmp op;
    int64_t i = 0;
    double d = 0.0;
};

class PhysicalGpuHashAggregate : public engine::PhysicalOperator {
public:
    // groups / aggregates over the child's columns; result_types are the
    // output slots [group cols…, agg cols…] with the binder's types.
    PhysicalGpuHashAggregate(std::vector<engine::idx_t> groups, std::vector<GpuAggregate> aggregates,
                             std::vector<engine::LogicalType> result_types,
                             std::vector<engine::LogicalType> input_types, std::vector<GpuPredicate> filters = {},
                             uint64_t est_groups = 0);
    ~PhysicalGpuHashAggregate() override;

    void SetTopNHint(engine::idx_t col_idx, bool ascending, engine::idx_t limit) override;
    void SetRowLimit(engine::idx_t n) override;
    void SetNeededOutputs(const std::vector<bool> &needed) override { needed_ = needed; }
    void Init() override;
    bool GetData(engine::DataChunk &result) override;

    uint64_t KernelLaunches() const;

private:
    void ComputeAggregates();
    void Flush();

    std::vector<engine::idx_t> groups_;
    std::vector<GpuAggregate> aggregates_;
    std::vector<engine::LogicalType> input_types_;
    std::vector<GpuPredicate> filters_;
    std::vector<bool> needed_;
    gb_agg *h_ = nullptr;
    bool computed_ = false;
    engine::idx_t emit_pos_ = 0;
    gb_result res_{};
    // pinned staging of child chunks, handed to gb_agg_ingest in large batches
    struct Stage;
    std::unique_ptr<Stage> stage_;
};

}  // namespace slothdb_gb300
