// Test infrastructure (oracle only) -- never linked into the shipped library.
//
// C ABI over the UNMODIFIED reference sources of eleanalt/hash-join-optimizer
// (src/execute.cpp, src/build_table.cpp, src/statement.cpp, src/csv_parser.cpp
// and include/*.h, compiled where they lie by oracle/Makefile into
// oracle/_ref/libhjref.so).  It lets the tests run the reference's own
// Contest::execute, Table::to_columnar, UnchainedHash and
// PartitionedDirectoryHash on the same flat plan descriptors (include/hj_api.h)
// the GPU engine takes, so the oracle restatement and the GPU results can be
// pinned against the real thing.
#include <cstring>
#include <exception>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include <plan.h>
#include <table.h>

// The reference keeps UnchainedHash's directory private; the known-answer
// export below needs to read it.  Layout is unchanged by this.
#define private public
#include <unchained.h>
#undef private
#include <partitioned_directory_hash.h>

#include "../include/hj_api.h"
#include "oracle_result.h"

namespace {

// Input columns borrow the caller's pages.  A reference `Column` frees its
// pages unless it holds a MappedMemory, so each borrowed column gets a
// zero-length mapping whose refcount keeps the pages alive and untouched.
ColumnarTable borrow_table(const hj_table_desc& t) {
    ColumnarTable out;
    out.num_rows = t.num_rows;
    for (uint32_t c = 0; c < t.num_columns; ++c) {
        const hj_column_desc& cd = t.columns[c];
        out.columns.emplace_back(static_cast<DataType>(cd.type));
        Column& col = out.columns.back();
        col.assign_mapped_memory(new MappedMemory(nullptr, 0));
        for (uint64_t p = 0; p < cd.num_pages; ++p)
            col.pages.push_back(reinterpret_cast<Page*>(const_cast<void*>(cd.pages[p])));
    }
    return out;
}

Plan to_plan(const hj_plan_desc& d) {
    Plan plan;
    for (uint32_t i = 0; i < d.num_nodes; ++i) {
        const hj_node_desc& n = d.nodes[i];
        if (n.num_filters) throw std::invalid_argument("the reference's Plan has no scan filters");
        std::vector<std::tuple<size_t, DataType>> attrs;
        for (uint32_t a = 0; a < n.num_attrs; ++a)
            attrs.emplace_back(size_t(n.attrs[a].index), static_cast<DataType>(n.attrs[a].type));
        if (n.kind == HJ_NODE_SCAN)
            plan.new_scan_node(n.base_table_id, std::move(attrs));
        else
            plan.new_join_node(n.build_left != 0, n.left, n.right, n.left_attr, n.right_attr,
                               std::move(attrs));
    }
    for (uint32_t i = 0; i < d.num_inputs; ++i) plan.inputs.push_back(borrow_table(d.inputs[i]));
    plan.root = d.root;
    return plan;
}

void fill_result(const ColumnarTable& t, oracle_result* out) {
    out->num_rows    = t.num_rows;
    out->num_columns = uint32_t(t.columns.size());
    out->types       = new int32_t[t.columns.size() + 1];
    out->num_pages   = new uint64_t[t.columns.size() + 1];
    out->pages       = new uint8_t*[t.columns.size() + 1];
    for (size_t c = 0; c < t.columns.size(); ++c) {
        const Column& col = t.columns[c];
        out->types[c]     = int32_t(col.type);
        out->num_pages[c] = col.pages.size();
        out->pages[c]     = new uint8_t[col.pages.size() * PAGE_SIZE + 1];
        for (size_t p = 0; p < col.pages.size(); ++p)
            std::memcpy(out->pages[c] + p * PAGE_SIZE, col.pages[p]->data, PAGE_SIZE);
    }
}

int fail(oracle_result* out, int status, const char* what) {
    out->status = status;
    std::snprintf(out->error, sizeof(out->error), "%s", what);
    return status;
}

}  // namespace

extern "C" {

int ref_execute(const hj_plan_desc* desc, oracle_result* out) {
    std::memset(out, 0, sizeof(*out));
    try {
        Plan  plan = to_plan(*desc);
        void* ctx  = Contest::build_context();
        auto  res  = Contest::execute(plan, ctx);
        Contest::destroy_context(ctx);
        fill_result(res, out);
        return HJ_OK;
    } catch (const std::out_of_range& e) {
        return fail(out, HJ_ERR_OUT_OF_RANGE, e.what());
    } catch (const std::runtime_error& e) {
        return fail(out, HJ_ERR_RUNTIME, e.what());
    } catch (const std::exception& e) {
        return fail(out, HJ_ERR_INVALID, e.what());
    }
}

// The reference's binary table cache: DumpTable::dump (include/table.h:128-211)
// of a borrowed table into `path`, and Table::from_cache (src/build_table.cpp:
// 147-203) of a file into `out`.
int ref_dump_table(const hj_table_desc* t, const char* path) {
    try {
        ColumnarTable ct = borrow_table(*t);
        DumpTable     d(&ct);
        std::ofstream f(path, std::ios::binary);
        d.dump(f);
        return f.good() ? HJ_OK : HJ_ERR_RUNTIME;
    } catch (const std::exception&) {
        return HJ_ERR_RUNTIME;
    }
}

int ref_from_cache(const char* path, oracle_result* out) {
    std::memset(out, 0, sizeof(*out));
    try {
        fill_result(Table::from_cache(path), out);
        return HJ_OK;
    } catch (const std::exception& e) {
        return fail(out, HJ_ERR_RUNTIME, e.what());
    }
}

// Table::to_columnar of one INT32 column (valid[i] == 0 -> NULL).
int ref_to_columnar_int32(const int32_t* vals, const uint8_t* valid, uint64_t n,
                          oracle_result* out) {
    std::memset(out, 0, sizeof(*out));
    std::vector<std::vector<Data>> rows(n);
    for (uint64_t i = 0; i < n; ++i) {
        if (!valid || valid[i]) rows[i].emplace_back(vals[i]);
        else                    rows[i].emplace_back(std::monostate{});
    }
    Table t(std::move(rows), {DataType::INT32});
    fill_result(t.to_columnar(), out);
    return HJ_OK;
}

// Table::to_columnar of one VARCHAR column; string i = bytes[off[i], off[i+1]).
int ref_to_columnar_strings(const uint8_t* bytes, const uint64_t* off, const uint8_t* valid,
                            uint64_t n, oracle_result* out) {
    std::memset(out, 0, sizeof(*out));
    std::vector<std::vector<Data>> rows(n);
    for (uint64_t i = 0; i < n; ++i) {
        if (!valid || valid[i])
            rows[i].emplace_back(std::string(reinterpret_cast<const char*>(bytes) + off[i],
                                             off[i + 1] - off[i]));
        else
            rows[i].emplace_back(std::monostate{});
    }
    Table t(std::move(rows), {DataType::VARCHAR});
    fill_result(t.to_columnar(), out);
    return HJ_OK;
}

// UnchainedHash<int32_t, uint32_t> over `keys` (payload = row index): copies the
// directory (dir_size + 1 words) to dir_out and returns dir_size in *dir_size.
int ref_unchained_directory(const int32_t* keys, uint64_t n, uint64_t* dir_out, uint64_t cap,
                            uint64_t* dir_size) {
    Contest::UnchainedHash<int32_t, uint32_t> h;
    for (uint64_t i = 0; i < n; ++i) h.build_insert(keys[i], uint32_t(i));
    h.finalize_build();
    *dir_size = h.dir_size_;
    if (h.directory_.size() > cap) return HJ_ERR_CAPACITY;
    std::copy(h.directory_.begin(), h.directory_.end(), dir_out);
    return HJ_OK;
}

// UnchainedHash probe of each key: number of payloads the callback receives.
int ref_unchained_counts(const int32_t* build, uint64_t nb, const int32_t* probe, uint64_t np,
                         uint64_t* counts) {
    Contest::UnchainedHash<int32_t, uint32_t> h;
    for (uint64_t i = 0; i < nb; ++i) h.build_insert(build[i], uint32_t(i));
    h.finalize_build();
    for (uint64_t i = 0; i < np; ++i) {
        uint64_t c = 0;
        h.probe(probe[i], [&](uint32_t) { ++c; });
        counts[i] = c;
    }
    return HJ_OK;
}

// PartitionedDirectoryHash (the table execute() builds, src/execute.cpp:64-83):
// directory words [-1 .. 2^dir_bits) after build with `threads` partitions.
int ref_pdh_directory(const int32_t* keys, uint64_t n, uint64_t threads, uint32_t dir_bits,
                      uint64_t* dir_out) {
    Contest::PartitionedDirectoryHash idx;
    idx.init(threads, dir_bits);
    struct Opt {
        bool     has;
        uint32_t v;
        bool     has_value() const { return has; }
        uint32_t value() const { return v; }
    };
    idx.build(n, threads, [&](size_t r) { return Opt{true, uint32_t(keys[r])}; });
    std::copy(idx.directory_store.begin(), idx.directory_store.end(), dir_out);
    return HJ_OK;
}

}  // extern "C"
