// Drop-in check of the C++ boundary: the reference's join unit tests
// (tests/unit_tests.cpp:10-371 of eleanalt/hash-join-optimizer) written
// against include/plan.h and run through Contest::build_context / execute /
// destroy_context of libhjgb300.so, exactly as the reference harness calls
// them.  Inputs are built with ColumnInserter; results are decoded from the
// returned pages and compared as sorted rows.  Prints "ok" on success.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <optional>
#include <stdexcept>
#include <string>
#include <vector>

#include "plan.h"

using Cell = std::optional<std::string>;  // NULL = nullopt; INT32 printed as decimal
using Row  = std::vector<Cell>;

struct In {
    std::vector<DataType>          types;
    std::vector<std::vector<Cell>> rows;  // cells as text; INT32 parsed
};

static ColumnarTable make_table(const In& t) {
    ColumnarTable out;
    out.num_rows = t.rows.size();
    for (size_t c = 0; c < t.types.size(); ++c) {
        out.columns.emplace_back(t.types[c]);
        Column& col = out.columns.back();
        if (t.types[c] == DataType::INT32) {
            ColumnInserter<int32_t> ins(col);
            for (auto& r : t.rows) r[c] ? ins.insert(int32_t(std::stol(*r[c]))) : ins.insert_null();
            ins.finalize();
        } else {
            ColumnInserter<std::string> ins(col);
            for (auto& r : t.rows) r[c] ? ins.insert(*r[c]) : ins.insert_null();
            ins.finalize();
        }
    }
    return out;
}

static std::vector<Row> rows_of(const ColumnarTable& t) {
    std::vector<Row> rows(t.num_rows, Row(t.columns.size()));
    for (size_t c = 0; c < t.columns.size(); ++c) {
        size_t r = 0;
        for (Page* pg : t.columns[c].pages) {
            const auto*    p  = reinterpret_cast<const uint8_t*>(pg->data);
            uint16_t       nr, nn;
            std::memcpy(&nr, p, 2);
            std::memcpy(&nn, p + 2, 2);
            if (nr == 0xffff) {
                rows.at(r++)[c] = std::string(reinterpret_cast<const char*>(p + 4), nn);
                continue;
            }
            if (nr == 0xfffe) {
                *rows.at(r - 1)[c] += std::string(reinterpret_cast<const char*>(p + 4), nn);
                continue;
            }
            const uint8_t* bm = p + PAGE_SIZE - (nr + 7) / 8;
            uint16_t       d = 0, start = 0;
            for (uint16_t i = 0; i < nr; ++i, ++r) {
                if (!(bm[i / 8] >> (i % 8) & 1)) continue;
                if (t.columns[c].type == DataType::INT32) {
                    int32_t v;
                    std::memcpy(&v, p + 4 + 4 * d++, 4);
                    rows.at(r)[c] = std::to_string(v);
                } else {
                    uint16_t end;
                    std::memcpy(&end, p + 4 + 2 * d++, 2);
                    rows.at(r)[c] = std::string(reinterpret_cast<const char*>(p + 4 + 2 * nn + start), end - start);
                    start = end;
                }
            }
        }
        if (r != t.num_rows) throw std::runtime_error("column " + std::to_string(c) + " row count mismatch");
    }
    std::sort(rows.begin(), rows.end());
    return rows;
}

static std::vector<Row> sorted(std::vector<Row> r) {
    std::sort(r.begin(), r.end());
    return r;
}

static int failures = 0;

static void check(const char* name, Plan& plan, void* ctx, std::vector<Row> truth, size_t ncols) {
    ColumnarTable out = Contest::execute(plan, ctx);
    auto          got = rows_of(out);
    if (out.num_rows != truth.size() || out.columns.size() != ncols || got != sorted(truth)) {
        std::printf("FAIL %s: %zu rows\n", name, out.num_rows);
        ++failures;
    }
}

int main() {
    using S     = std::string;
    const auto I = DataType::INT32, V = DataType::VARCHAR;
    const Cell N;  // NULL
    void*      ctx = Contest::build_context();
    auto one = [](std::initializer_list<Cell> c) { return std::vector<Cell>(c); };

    {  // empty join
        Plan p;
        p.new_scan_node(0, {{0, I}});
        p.new_scan_node(1, {{0, I}});
        p.new_join_node(true, 0, 1, 0, 0, {{0, I}, {1, I}});
        p.new_input(make_table({{I}, {}}));
        p.new_input(make_table({{I}, {}}));
        p.root = 2;
        check("empty", p, ctx, {}, 2);
    }
    {  // duplicate keys + NULL keys (unit_tests.cpp:163-200)
        In t{{I}, {one({S("1")}), one({S("1")}), one({N}), one({S("2")}), one({S("3")})}};
        Plan p;
        p.new_scan_node(0, {{0, I}});
        p.new_scan_node(1, {{0, I}});
        p.new_join_node(true, 0, 1, 0, 0, {{0, I}, {1, I}});
        p.new_input(make_table(t));
        p.new_input(make_table(t));
        p.root = 2;
        check("null_keys", p, ctx,
              {{S("1"), S("1")}, {S("1"), S("1")}, {S("1"), S("1")}, {S("1"), S("1")}, {S("2"), S("2")},
               {S("3"), S("3")}},
              2);
    }
    for (bool build_left : {true, false}) {  // unit_tests.cpp:202-282
        In t{{I, V},
             {one({S("1"), S("xxx")}), one({S("1"), S("yyy")}), one({N, S("zzz")}), one({S("2"), S("uuu")}),
              one({S("3"), S("vvv")})}};
        Plan p;
        p.new_scan_node(0, {{0, I}});
        p.new_scan_node(1, {{1, V}, {0, I}});
        p.new_join_node(build_left, 0, 1, 0, 1, {{0, I}, {2, I}, {1, V}});
        p.new_input(make_table(t));
        p.new_input(make_table(t));
        p.root = 2;
        check(build_left ? "multiple_columns" : "build_on_right", p, ctx,
              {{S("1"), S("1"), S("xxx")}, {S("1"), S("1"), S("xxx")}, {S("1"), S("1"), S("yyy")},
               {S("1"), S("1"), S("yyy")}, {S("2"), S("2"), S("uuu")}, {S("3"), S("3"), S("vvv")}},
              3);
    }
    {  // 3-way join with VARCHAR on both sides (unit_tests.cpp:323-371)
        Plan p;
        p.new_scan_node(0, {{0, I}, {1, V}});
        p.new_scan_node(1, {{0, I}, {1, V}});
        p.new_scan_node(2, {{0, I}, {1, V}});
        p.new_join_node(false, 0, 1, 0, 0, {{0, I}, {1, V}});
        p.new_join_node(false, 3, 2, 0, 0, {{0, I}, {1, V}, {3, V}});
        p.new_input(make_table({{I, V}, {one({S("1"), S("a")}), one({S("2"), S("b")}), one({S("3"), S("c")})}}));
        p.new_input(make_table({{I, V}, {one({S("1"), S("x")}), one({S("2"), S("y")})}}));
        p.new_input(make_table({{I, V}, {one({S("1"), S("u")}), one({S("2"), S("v")}), one({S("3"), S("w")})}}));
        p.root = 4;
        check("three_way", p, ctx, {{S("1"), S("a"), S("u")}, {S("2"), S("b"), S("v")}}, 3);
    }
    {  // the reference's exception classes cross the boundary
        Plan p;
        p.new_scan_node(0, {{0, V}});
        p.new_scan_node(1, {{0, V}});
        p.new_join_node(true, 0, 1, 0, 0, {{0, V}});
        p.new_input(make_table({{V}, {one({S("a")})}}));
        p.new_input(make_table({{V}, {one({S("a")})}}));
        p.root = 2;
        bool thrown = false;
        try {
            Contest::execute(p, ctx);
        } catch (const std::runtime_error& e) {
            thrown = std::string(e.what()).find("int32") != std::string::npos;
        }
        if (!thrown) {
            std::printf("FAIL runtime_error\n");
            ++failures;
        }
    }
    Contest::destroy_context(ctx);
    if (failures) return 1;
    std::printf("ok\n");
    return 0;
}
