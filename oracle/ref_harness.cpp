// ref_harness.cpp — runs one GROUP BY through the reference engine itself.
//
// TEST INFRASTRUCTURE ONLY: linked against the reference library that
// oracle/ref.mk builds from the reference's sources; it pins the oracle and
// generates golden vectors.  The product never links or loads it.
//
// It uses only the reference's public programmatic API:
//   Database / Connection            include/slothdb/main/connection.hpp:90-128
//   Connection::CreateTable + Append include/slothdb/main/connection.hpp:104-108
//   DataChunk / Vector / ValidityMask include/slothdb/common/types/*.hpp
//   Connection::Query -> QueryResult (chunks of typed vectors)
//
// Usage: ref_harness <spec> <out>
// spec (text, one directive per line):
//   rows <n>
//   col <name> <SMALLINT|INTEGER|BIGINT|DOUBLE|VARCHAR> <data file> [<null file>|-] [<offsets file>]
//       data: raw little-endian values (VARCHAR: the bytes, offsets: int64[n+1]);
//       null: one byte per row, 1 = NULL
//   query <SQL to the end of the line>
//   repeat <r>            (times the query r times; the median is reported)
// Columns are appended as table "t" in 2048-row chunks.  The result is written
// to <out> as text: a header line of type names, then one tab-separated line
// per row (\N = NULL, doubles with 17 significant digits).  stdout gets
// "ms <median query ms>" and "rows <result rows>".
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "slothdb/main/connection.hpp"
#include "slothdb/main/database.hpp"

using namespace slothdb;

struct ColSpec {
    std::string name, type, data, nulls, offs;
};

static std::vector<char> read_file(const std::string &path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        fprintf(stderr, "cannot open %s\n", path.c_str());
        exit(2);
    }
    return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

static LogicalType type_of(const std::string &t) {
    if (t == "SMALLINT") return LogicalType::SMALLINT();
    if (t == "INTEGER") return LogicalType::INTEGER();
    if (t == "BIGINT") return LogicalType::BIGINT();
    if (t == "DOUBLE") return LogicalType::DOUBLE();
    if (t == "VARCHAR") return LogicalType::VARCHAR();
    fprintf(stderr, "unknown type %s\n", t.c_str());
    exit(2);
}

static size_t width_of(const std::string &t) {
    if (t == "SMALLINT") return 2;
    if (t == "INTEGER") return 4;
    return 8;
}

static void write_value(FILE *o, const Value &v) {
    if (v.IsNull()) {
        fputs("\\N", o);
        return;
    }
    switch (v.type().id()) {
    case LogicalTypeId::DOUBLE: fprintf(o, "%.17g", v.GetValue<double>()); break;
    case LogicalTypeId::FLOAT: fprintf(o, "%.9g", (double)v.GetValue<float>()); break;
    case LogicalTypeId::SMALLINT: fprintf(o, "%d", (int)v.GetValue<int16_t>()); break;
    case LogicalTypeId::INTEGER: fprintf(o, "%d", v.GetValue<int32_t>()); break;
    case LogicalTypeId::BIGINT: fprintf(o, "%lld", (long long)v.GetValue<int64_t>()); break;
    default: fputs(v.ToString().c_str(), o); break;
    }
}

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: ref_harness <spec> <out>\n");
        return 2;
    }
    std::ifstream spec(argv[1]);
    std::string line, query;
    long long rows = 0;
    int repeat = 1;
    std::vector<ColSpec> cols;
    while (std::getline(spec, line)) {
        std::istringstream ls(line);
        std::string d;
        ls >> d;
        if (d == "rows") ls >> rows;
        else if (d == "repeat") ls >> repeat;
        else if (d == "query") {
            std::getline(ls, query);
            query.erase(0, query.find_first_not_of(' '));
        } else if (d == "col") {
            ColSpec c;
            ls >> c.name >> c.type >> c.data;
            ls >> c.nulls >> c.offs;
            if (c.nulls == "-") c.nulls.clear();
            cols.push_back(c);
        }
    }
    Database db;
    Connection con(db);
    if (!cols.empty()) {
        std::vector<ColumnDefinition> defs;
        std::vector<LogicalType> types;
        for (auto &c : cols) {
            defs.emplace_back(c.name, type_of(c.type));
            types.push_back(type_of(c.type));
        }
        con.CreateTable("t", defs);
        std::vector<std::vector<char>> data, nulls, offs;
        for (auto &c : cols) {
            data.push_back(read_file(c.data));
            nulls.push_back(c.nulls.empty() ? std::vector<char>() : read_file(c.nulls));
            offs.push_back(c.offs.empty() ? std::vector<char>() : read_file(c.offs));
        }
        for (long long r0 = 0; r0 < rows; r0 += VECTOR_SIZE) {
            const long long n = std::min<long long>(VECTOR_SIZE, rows - r0);
            DataChunk chunk;
            chunk.Initialize(types);
            for (size_t ci = 0; ci < cols.size(); ci++) {
                Vector &v = chunk.GetVector(ci);
                const bool has_nulls = !nulls[ci].empty();
                if (cols[ci].type == "VARCHAR") {
                    const int64_t *o = (const int64_t *)offs[ci].data();
                    for (long long i = 0; i < n; i++) {
                        const long long r = r0 + i;
                        if (has_nulls && nulls[ci][r]) {
                            v.SetValue(i, Value());
                            v.GetValidity().SetInvalid(i);
                        } else {
                            v.SetValue(i, Value::VARCHAR(std::string(data[ci].data() + o[r], o[r + 1] - o[r])));
                        }
                    }
                } else {
                    const size_t w = width_of(cols[ci].type);
                    memcpy(v.GetData(), data[ci].data() + (size_t)r0 * w, (size_t)n * w);
                    if (has_nulls)
                        for (long long i = 0; i < n; i++)
                            if (nulls[ci][r0 + i]) v.GetValidity().SetInvalid(i);
                }
            }
            chunk.SetCardinality(n);
            con.Append("t", chunk);
        }
    }
    std::vector<double> ms;
    QueryResult res;
    for (int i = 0; i < repeat; i++) {
        auto t0 = std::chrono::steady_clock::now();
        res = con.Query(query);
        res.MaterialiseRows();
        auto t1 = std::chrono::steady_clock::now();
        ms.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
    }
    std::sort(ms.begin(), ms.end());
    FILE *o = fopen(argv[2], "w");
    if (!o) return 2;
    for (size_t c = 0; c < res.column_types.size(); c++)
        fprintf(o, "%s%s", c ? "\t" : "", res.column_types[c].ToString().c_str());
    fputc('\n', o);
    const idx_t nr = res.RowCount();
    for (idx_t r = 0; r < nr; r++) {
        for (idx_t c = 0; c < res.ColumnCount(); c++) {
            if (c) fputc('\t', o);
            write_value(o, res.GetValue(r, c));
        }
        fputc('\n', o);
    }
    fclose(o);
    printf("ms %.3f\nrows %llu\n", ms[ms.size() / 2], (unsigned long long)nr);
    return 0;
}
