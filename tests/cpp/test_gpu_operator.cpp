// test_gpu_operator.cpp — PhysicalGpuHashAggregate driven like SlothDB's
// own operator tests: a child operator hands out DataChunks, the aggregate
// is pulled with GetData until it returns false, and the result rows are
// checked against known answers.
//
// Known answers follow the reference's tests for this path:
//   test/test_performance.cpp:149-173  HashAggregate {1: 90/3, 2: 60/2}
//   test/test_aggregation.cpp:16-212   5-row emp table GROUP BY dept
//   test/test_parallel.cpp:105-160     SUM(1..10000) = 50005000; 5 x 10,000 COUNT
// plus a 1M-row GROUP BY checked against a direct host computation, NULL
// handling, the TopN hint and re-execution after Init().
//
// Exit status 0 = all passed.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <random>
#include <set>
#include <string>
#include <tuple>
#include <vector>

#include "gpu_operator.hpp"

using namespace slothdb_gb300;
using namespace slothdb_gb300::engine;

static int g_fail = 0;
#define REQUIRE(c)                                                         \
    do {                                                                   \
        if (!(c)) {                                                        \
            std::fprintf(stderr, "%s:%d: REQUIRE(%s) failed\n", __FILE__, __LINE__, #c); \
            g_fail++;                                                      \
        }                                                                  \
    } while (0)

// A child operator that hands out pre-built columns in VECTOR_SIZE chunks.
class ColumnSource : public PhysicalOperator {
public:
    ColumnSource(std::vector<LogicalType> types, idx_t rows) : PhysicalOperator(types), rows_(rows) {}
    std::vector<std::vector<int64_t>> ints;        // per column (fixed width, widened)
    std::vector<std::vector<std::string>> strs;    // per column (VARCHAR)
    std::vector<std::vector<bool>> nulls;          // per column (empty = none)
    void Init() override { pos_ = 0; }
    bool GetData(DataChunk &out) override {
        if (pos_ >= rows_) return false;
        out.Initialize(GetTypes());
        const idx_t n = std::min<idx_t>(VECTOR_SIZE, rows_ - pos_);
        for (size_t c = 0; c < GetTypes().size(); c++) {
            Vector &v = out.GetVector(c);
            for (idx_t i = 0; i < n; i++) {
                const idx_t r = pos_ + i;
                switch (GetTypes()[c].id) {
                case LogicalTypeId::SMALLINT: v.GetData<int16_t>()[i] = (int16_t)ints[c][r]; break;
                case LogicalTypeId::INTEGER: v.GetData<int32_t>()[i] = (int32_t)ints[c][r]; break;
                case LogicalTypeId::BIGINT: v.GetData<int64_t>()[i] = ints[c][r]; break;
                case LogicalTypeId::DOUBLE: v.GetData<double>()[i] = (double)ints[c][r]; break;
                case LogicalTypeId::VARCHAR: v.Strings()[i] = strs[c][r]; break;
                }
                if (!nulls.empty() && !nulls[c].empty() && nulls[c][r]) v.GetValidity().SetInvalid(i, VECTOR_SIZE);
            }
        }
        out.SetCardinality(n);
        pos_ += n;
        return true;
    }

private:
    idx_t rows_, pos_ = 0;
};

struct Row {
    std::vector<std::string> cells;  // rendered values, "NULL" for NULL
    bool operator<(const Row &o) const { return cells < o.cells; }
};

static std::vector<Row> pull(PhysicalOperator &op) {
    std::vector<Row> rows;
    DataChunk chunk;
    while (op.GetData(chunk)) {
        for (idx_t i = 0; i < chunk.size(); i++) {
            Row r;
            for (idx_t c = 0; c < chunk.ColumnCount(); c++) {
                const Vector &v = chunk.GetVector(c);
                if (!v.GetValidity().RowIsValid(i)) {
                    r.cells.push_back("NULL");
                    continue;
                }
                char buf[64];
                switch (v.GetType().id) {
                case LogicalTypeId::SMALLINT: std::snprintf(buf, sizeof buf, "%d", v.GetData<int16_t>()[i]); break;
                case LogicalTypeId::INTEGER: std::snprintf(buf, sizeof buf, "%d", v.GetData<int32_t>()[i]); break;
                case LogicalTypeId::BIGINT:
                    std::snprintf(buf, sizeof buf, "%lld", (long long)v.GetData<int64_t>()[i]);
                    break;
                case LogicalTypeId::DOUBLE: std::snprintf(buf, sizeof buf, "%.6f", v.GetData<double>()[i]); break;
                case LogicalTypeId::VARCHAR: r.cells.push_back(v.Strings()[i]); continue;
                }
                r.cells.push_back(buf);
            }
            rows.push_back(r);
        }
    }
    return rows;
}

static const LogicalType SMALLINT_T(LogicalTypeId::SMALLINT), INTEGER_T(LogicalTypeId::INTEGER),
    BIGINT_T(LogicalTypeId::BIGINT), DOUBLE_T(LogicalTypeId::DOUBLE), VARCHAR_T(LogicalTypeId::VARCHAR);

static void test_hash_aggregate_known_answer() {
    auto src = std::make_unique<ColumnSource>(std::vector<LogicalType>{INTEGER_T, INTEGER_T}, 5);
    src->ints = {{1, 2, 1, 2, 1}, {10, 20, 30, 40, 50}};
    PhysicalGpuHashAggregate agg({0}, {{GB_AGG_SUM, 1}, {GB_AGG_COUNT_STAR, -1}}, {INTEGER_T, BIGINT_T, BIGINT_T},
                                 {INTEGER_T, INTEGER_T});
    agg.children.push_back(std::move(src));
    agg.Init();
    auto rows = pull(agg);
    std::sort(rows.begin(), rows.end());
    REQUIRE(rows.size() == 2);
    REQUIRE(rows.size() == 2 && rows[0].cells == std::vector<std::string>({"1", "90", "3"}));
    REQUIRE(rows.size() == 2 && rows[1].cells == std::vector<std::string>({"2", "60", "2"}));
    REQUIRE(agg.KernelLaunches() > 0);
}

static void test_emp_group_by_dept() {
    auto src = std::make_unique<ColumnSource>(std::vector<LogicalType>{VARCHAR_T, VARCHAR_T, INTEGER_T}, 5);
    src->ints = {{}, {}, {100, 120, 80, 90, 95}};
    src->strs = {{"Alice", "Bob", "Charlie", "Diana", "Eve"},
                 {"Engineering", "Engineering", "Sales", "Sales", "Marketing"},
                 {}};
    // SELECT dept, COUNT(*), SUM(salary), AVG(salary) FROM emp GROUP BY dept
    PhysicalGpuHashAggregate agg({1}, {{GB_AGG_COUNT_STAR, -1}, {GB_AGG_SUM, 2}, {GB_AGG_AVG, 2}},
                                 {VARCHAR_T, BIGINT_T, BIGINT_T, DOUBLE_T}, {VARCHAR_T, VARCHAR_T, INTEGER_T});
    agg.children.push_back(std::move(src));
    agg.Init();
    auto rows = pull(agg);
    std::sort(rows.begin(), rows.end());
    REQUIRE(rows.size() == 3);
    if (rows.size() == 3) {
        REQUIRE(rows[0].cells == std::vector<std::string>({"Engineering", "2", "220", "110.000000"}));
        REQUIRE(rows[1].cells == std::vector<std::string>({"Marketing", "1", "95", "95.000000"}));
        REQUIRE(rows[2].cells == std::vector<std::string>({"Sales", "2", "170", "85.000000"}));
    }
}

static void test_parallel_sum_and_counts() {
    const idx_t n = 10000;
    auto src = std::make_unique<ColumnSource>(std::vector<LogicalType>{INTEGER_T, INTEGER_T}, n);
    src->ints.assign(2, std::vector<int64_t>(n));
    for (idx_t i = 0; i < n; i++) src->ints[1][i] = (int64_t)i + 1;
    PhysicalGpuHashAggregate agg({0}, {{GB_AGG_SUM, 1}}, {INTEGER_T, BIGINT_T}, {INTEGER_T, INTEGER_T});
    agg.children.push_back(std::move(src));
    agg.Init();
    auto rows = pull(agg);
    REQUIRE(rows.size() == 1 && rows[0].cells[1] == "50005000");

    const idx_t m = 50000;
    auto src2 = std::make_unique<ColumnSource>(std::vector<LogicalType>{INTEGER_T}, m);
    src2->ints.assign(1, std::vector<int64_t>(m));
    for (idx_t i = 0; i < m; i++) src2->ints[0][i] = (int64_t)(i % 5);
    PhysicalGpuHashAggregate agg2({0}, {{GB_AGG_COUNT_STAR, -1}}, {INTEGER_T, BIGINT_T}, {INTEGER_T});
    agg2.children.push_back(std::move(src2));
    agg2.Init();
    auto rows2 = pull(agg2);
    REQUIRE(rows2.size() == 5);
    for (auto &r : rows2) REQUIRE(r.cells[1] == "10000");
}

// 1M rows, k INT32 over 1,024 values, v INT64 in [0, 10^6): COUNT/SUM/MIN/MAX
// against a direct host computation; then Init() and a second execution.
static void test_plain_million_rows_and_reexecution() {
    const idx_t n = 1000000;
    std::mt19937_64 rng(0);
    auto src = std::make_unique<ColumnSource>(std::vector<LogicalType>{INTEGER_T, BIGINT_T}, n);
    src->ints.assign(2, std::vector<int64_t>(n));
    std::map<int64_t, std::tuple<int64_t, int64_t, int64_t, int64_t>> want;
    for (idx_t i = 0; i < n; i++) {
        const int64_t k = (int64_t)(rng() % 1024), v = (int64_t)(rng() % 1000000);
        src->ints[0][i] = k;
        src->ints[1][i] = v;
        auto it = want.find(k);
        if (it == want.end()) want[k] = std::make_tuple(1, v, v, v);
        else {
            auto &t = it->second;
            std::get<0>(t)++;
            std::get<1>(t) += v;
            std::get<2>(t) = std::min(std::get<2>(t), v);
            std::get<3>(t) = std::max(std::get<3>(t), v);
        }
    }
    PhysicalGpuHashAggregate agg({0}, {{GB_AGG_COUNT_STAR, -1}, {GB_AGG_SUM, 1}, {GB_AGG_MIN, 1}, {GB_AGG_MAX, 1}},
                                 {INTEGER_T, BIGINT_T, BIGINT_T, BIGINT_T, BIGINT_T}, {INTEGER_T, BIGINT_T}, {},
                                 1024);
    agg.children.push_back(std::move(src));
    for (int run = 0; run < 2; run++) {
        agg.Init();
        auto rows = pull(agg);
        REQUIRE(rows.size() == want.size());
        int bad = 0;
        for (auto &r : rows) {
            const auto &t = want[std::stoll(r.cells[0])];
            bad += r.cells[1] != std::to_string(std::get<0>(t)) || r.cells[2] != std::to_string(std::get<1>(t)) ||
                   r.cells[3] != std::to_string(std::get<2>(t)) || r.cells[4] != std::to_string(std::get<3>(t));
        }
        REQUIRE(bad == 0);
    }
}

static void test_nulls_filter_and_topn() {
    // k SMALLINT with NULLs, v INTEGER with NULLs; WHERE v >= 0;
    // SELECT k, COUNT(v), SUM(v) ... ORDER BY COUNT(v) DESC LIMIT 3
    const idx_t n = 5000;
    auto src = std::make_unique<ColumnSource>(std::vector<LogicalType>{SMALLINT_T, INTEGER_T}, n);
    src->ints.assign(2, std::vector<int64_t>(n));
    src->nulls.assign(2, std::vector<bool>(n, false));
    std::map<std::string, std::pair<int64_t, int64_t>> want;  // key → (count(v), sum(v))
    for (idx_t i = 0; i < n; i++) {
        const int64_t k = (int64_t)((i * 7) % 13), v = (int64_t)(i % 23) - 3;
        src->ints[0][i] = k;
        src->ints[1][i] = v;
        src->nulls[0][i] = (i % 17) == 0;
        src->nulls[1][i] = (i % 11) == 0;
        if (src->nulls[1][i] || v < 0) continue;  // the predicate drops NULL and negative v
        auto &w = want[src->nulls[0][i] ? "NULL" : std::to_string(k)];
        w.first++;
        w.second += v;
    }
    PhysicalGpuHashAggregate agg({0}, {{GB_AGG_COUNT, 1}, {GB_AGG_SUM, 1}}, {SMALLINT_T, BIGINT_T, BIGINT_T},
                                 {SMALLINT_T, INTEGER_T}, {{1, GB_CMP_GE, 0, 0.0}});
    agg.children.push_back(std::move(src));
    agg.Init();
    auto rows = pull(agg);
    REQUIRE(rows.size() == want.size());
    for (auto &r : rows) {
        auto it = want.find(r.cells[0]);
        REQUIRE(it != want.end());
        if (it != want.end())
            REQUIRE(r.cells[1] == std::to_string(it->second.first) && r.cells[2] == std::to_string(it->second.second));
    }
    // TopN: 3 rows with the largest COUNT(v), in descending order
    auto src2 = std::make_unique<ColumnSource>(std::vector<LogicalType>{INTEGER_T}, 1000);
    src2->ints.assign(1, std::vector<int64_t>(1000));
    for (idx_t i = 0; i < 1000; i++) src2->ints[0][i] = (int64_t)(i < 400 ? 7 : (i < 700 ? 3 : (i < 900 ? 9 : i)));
    PhysicalGpuHashAggregate top({0}, {{GB_AGG_COUNT_STAR, -1}}, {INTEGER_T, BIGINT_T}, {INTEGER_T});
    top.children.push_back(std::move(src2));
    top.SetTopNHint(1, false, 3);
    top.Init();
    auto t = pull(top);
    REQUIRE(t.size() == 3);
    if (t.size() == 3) {
        REQUIRE(t[0].cells == std::vector<std::string>({"7", "400"}));
        REQUIRE(t[1].cells == std::vector<std::string>({"3", "300"}));
        REQUIRE(t[2].cells == std::vector<std::string>({"9", "200"}));
    }
}

static void test_errors_are_reported() {
    bool threw = false;
    try {  // SUM over VARCHAR is not a GPU shape: an error, never a CPU fallback
        PhysicalGpuHashAggregate bad({0}, {{GB_AGG_SUM, 1}}, {INTEGER_T, BIGINT_T}, {INTEGER_T, VARCHAR_T});
    } catch (const GpuAggregateError &e) {
        threw = e.status == GB_ERR_UNSUPPORTED || e.status == GB_ERR_INVALID;
    }
    REQUIRE(threw);
    threw = false;
    try {  // declared result types must match the plan's
        auto src = std::make_unique<ColumnSource>(std::vector<LogicalType>{INTEGER_T, INTEGER_T}, 3);
        src->ints = {{1, 2, 3}, {4, 5, 6}};
        PhysicalGpuHashAggregate agg({0}, {{GB_AGG_SUM, 1}}, {INTEGER_T, INTEGER_T}, {INTEGER_T, INTEGER_T});
        agg.children.push_back(std::move(src));
        agg.Init();
        pull(agg);
    } catch (const GpuAggregateError &) {
        threw = true;
    }
    REQUIRE(threw);
}

static void test_count_distinct() {
    // SELECT DISTINCT x over (1, 1, 2, 2, 3) has 3 rows
    // (test_advanced_sql.cpp:11-18): COUNT(DISTINCT x) under a constant key
    auto src = std::make_unique<ColumnSource>(std::vector<LogicalType>{INTEGER_T, INTEGER_T}, 5);
    src->ints = {{0, 0, 0, 0, 0}, {1, 1, 2, 2, 3}};
    PhysicalGpuHashAggregate agg({0}, {{GB_AGG_COUNT_DISTINCT, 1}}, {INTEGER_T, BIGINT_T}, {INTEGER_T, INTEGER_T});
    agg.children.push_back(std::move(src));
    agg.Init();
    auto rows = pull(agg);
    REQUIRE(rows.size() == 1 && rows[0].cells[1] == "3");
    // grouped: NULL values never counted, a group of NULL values counts 0
    const idx_t n = 3000;
    auto src2 = std::make_unique<ColumnSource>(std::vector<LogicalType>{INTEGER_T, BIGINT_T}, n);
    src2->ints.assign(2, std::vector<int64_t>(n));
    src2->nulls.assign(2, std::vector<bool>(n, false));
    std::map<std::string, std::set<int64_t>> want;
    for (idx_t i = 0; i < n; i++) {
        const int64_t k = (int64_t)(i % 7), v = (int64_t)((i * 13) % 50);
        src2->ints[0][i] = k;
        src2->ints[1][i] = v;
        src2->nulls[1][i] = (i % 9) == 0 || k == 6;
        auto &w = want[std::to_string(k)];
        if (!src2->nulls[1][i]) w.insert(v);
    }
    PhysicalGpuHashAggregate agg2({0}, {{GB_AGG_COUNT_DISTINCT, 1}, {GB_AGG_COUNT_STAR, -1}},
                                  {INTEGER_T, BIGINT_T, BIGINT_T}, {INTEGER_T, BIGINT_T});
    agg2.children.push_back(std::move(src2));
    agg2.Init();
    auto rows2 = pull(agg2);
    REQUIRE(rows2.size() == want.size());
    for (auto &r : rows2) {
        auto it = want.find(r.cells[0]);
        REQUIRE(it != want.end());
        if (it != want.end()) REQUIRE(r.cells[1] == std::to_string(it->second.size()));
    }
}

int main() {
    test_hash_aggregate_known_answer();
    test_emp_group_by_dept();
    test_parallel_sum_and_counts();
    test_plain_million_rows_and_reexecution();
    test_nulls_filter_and_topn();
    test_errors_are_reported();
    test_count_distinct();
    if (g_fail) {
        std::fprintf(stderr, "%d check(s) failed\n", g_fail);
        return 1;
    }
    std::printf("all operator tests passed\n");
    return 0;
}
