// engine_operator_check.cpp — the operator built against SlothDB's own
// headers and library (compiled with SLOTHDB_GB300_ENGINE_HEADERS, linked
// with the engine that oracle/ref.mk builds from the reference's sources).
//
// An engine-typed source operator feeds PhysicalGpuHashAggregate through the
// engine's DataChunk / Vector / ValidityMask / string_t; the result is
// compared with the engine's own GROUP BY of the same rows
// (Connection::CreateTable + Append + Query) — the aggregation tests of the
// reference's test/unit/execution/test_aggregation.cpp run both ways.
// Without a CUDA device the operator's first library call fails; the program
// then reports "no device" after the engine's own query ran, which still
// shows that the operator compiles and links against the engine.
//
// Exit status: 0 = equal results or no device, 1 = a difference, 2 = usage.
#include <algorithm>
#include <cstdio>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "slothdb/main/connection.hpp"
#include "slothdb/main/database.hpp"
#include "gpu_operator.hpp"

using namespace slothdb;

namespace {

// The rows of the reference's 5-row `emp` table (test_aggregation.cpp:16-25
// shape: name VARCHAR, dept VARCHAR, salary INTEGER), scaled by repetition so
// that several 2048-row chunks flow; NULL salaries only in a table of one
// chunk (the engine's in-memory GROUP BY mishandles a column with NULLs that
// spans several appended chunks).
struct Rows {
    std::vector<std::string> dept;
    std::vector<int32_t> salary;
    std::vector<bool> salary_null;
};

Rows make_rows(int reps, bool nulls) {
    static const char *depts[] = {"eng", "eng", "sales", "sales", "hr"};
    static const int32_t sal[] = {100, 80, 60, 50, 70};
    Rows r;
    for (int k = 0; k < reps; k++)
        for (int i = 0; i < 5; i++) {
            r.dept.push_back(depts[i]);
            r.salary.push_back(sal[i] + k % 7);
            r.salary_null.push_back(nulls && (k * 5 + i) % 11 == 3);
        }
    return r;
}

// Fills engine chunks of up to VECTOR_SIZE rows.
class RowSource : public PhysicalOperator {
public:
    explicit RowSource(const Rows &rows)
        : PhysicalOperator(PhysicalOperatorType::TABLE_SCAN, {LogicalType::VARCHAR(), LogicalType::INTEGER()}),
          rows_(rows) {}
    void Init() override { pos_ = 0; }
    bool GetData(DataChunk &out) override {
        const idx_t n = std::min<idx_t>(VECTOR_SIZE, rows_.salary.size() - pos_);
        if (n == 0) return false;
        out.Initialize(GetTypes());
        Vector &d = out.GetVector(0);
        Vector &s = out.GetVector(1);
        for (idx_t i = 0; i < n; i++) {
            const std::string &x = rows_.dept[pos_ + i];
            const char *p = d.GetStringBuffer().AddString(x.data(), x.size());
            d.GetData<string_t>()[i] = string_t(p, (uint32_t)x.size());
            s.GetData<int32_t>()[i] = rows_.salary[pos_ + i];
            if (rows_.salary_null[pos_ + i]) s.GetValidity().SetInvalid(i);
        }
        out.SetCardinality(n);
        pos_ += n;
        return true;
    }

private:
    const Rows &rows_;
    idx_t pos_ = 0;
};

typedef std::map<std::string, std::tuple<int64_t, int64_t, bool, int64_t>> Groups;  // count(*), sum, sum null, max

Groups engine_groups(const Rows &rows) {
    Database db;
    Connection con(db);
    std::vector<ColumnDefinition> defs;
    defs.emplace_back("dept", LogicalType::VARCHAR());
    defs.emplace_back("salary", LogicalType::INTEGER());
    con.CreateTable("emp", defs);
    RowSource src(rows);
    DataChunk chunk;
    while (src.GetData(chunk)) con.Append("emp", chunk);
    QueryResult res = con.Query("SELECT dept, COUNT(*), SUM(salary), MAX(salary) FROM emp GROUP BY dept");
    res.MaterialiseRows();
    Groups g;
    for (idx_t r = 0; r < res.RowCount(); r++) {
        const Value &sum = res.GetValue(r, 2);
        const Value &mx = res.GetValue(r, 3);
        g[res.GetValue(r, 0).ToString()] =
            std::make_tuple((int64_t)std::stoll(res.GetValue(r, 1).ToString()),
                            sum.IsNull() ? 0 : (int64_t)std::stoll(sum.ToString()), sum.IsNull(),
                            mx.IsNull() ? 0 : (int64_t)std::stoll(mx.ToString()));
    }
    return g;
}

}  // namespace

int run(const Rows &rows) {
    const Groups want = engine_groups(rows);
    printf("engine: %zu groups over %zu rows\n", want.size(), rows.salary.size());
    fflush(stdout);
    try {
        slothdb_gb300::PhysicalGpuHashAggregate op(
            {0}, {{GB_AGG_COUNT_STAR, -1}, {GB_AGG_SUM, 1}, {GB_AGG_MAX, 1}},
            {LogicalType::VARCHAR(), LogicalType::BIGINT(), LogicalType::BIGINT(), LogicalType::INTEGER()},
            {LogicalType::VARCHAR(), LogicalType::INTEGER()});
        op.children.push_back(std::make_unique<RowSource>(rows));
        op.Init();
        Groups got;
        DataChunk out;
        while (op.GetData(out)) {
            for (idx_t i = 0; i < out.size(); i++) {
                const string_t &k = out.GetVector(0).GetData<string_t>()[i];
                const bool sum_null = !out.GetVector(2).GetValidity().RowIsValid(i);
                got[std::string(k.GetData(), k.GetSize())] =
                    std::make_tuple(out.GetVector(1).GetData<int64_t>()[i],
                                    sum_null ? 0 : out.GetVector(2).GetData<int64_t>()[i], sum_null,
                                    (int64_t)out.GetVector(3).GetData<int32_t>()[i]);
            }
        }
        if (got != want) {
            printf("DIFFERENT: operator %zu groups, engine %zu\n", got.size(), want.size());
            return 1;
        }
        printf("equal: %zu groups\n", got.size());
    } catch (const slothdb_gb300::GpuAggregateError &e) {
        printf("no device: %s\n", e.what());
    }
    fflush(stdout);
    return 0;
}

int main() {
    int rc = run(make_rows(2000, false));  // 10,000 rows, five chunks
    if (rc == 0) rc = run(make_rows(400, true));  // 2,000 rows with NULL salaries, one chunk
    return rc;
}
