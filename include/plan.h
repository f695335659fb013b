// Plan / paged-columnar-table API of the SIGMOD-2025 contest, as used by the
// join path of eleanalt/hash-join-optimizer (include/plan.h:28-405 there).
//
// Every type that crosses `Contest::execute` keeps the reference's member
// order and types, so a harness compiled against the reference's plan.h links
// against this library unchanged:
//   MappedMemory            plan.h:28-64    {addr, length, refs}
//   ScanNode / JoinNode     plan.h:78-88
//   PlanNode                plan.h:90-98    {variant<ScanNode,JoinNode>, output_attrs}
//   Page                    plan.h:102-106  8192 bytes, alignas(8)
//   Column                  plan.h:108-161  {type, vector<Page*>, MappedMemory*}
//   ColumnarTable           plan.h:163-166  {num_rows, columns}
//   Plan                    plan.h:173-210  {nodes, inputs, root} + builders
//   Contest::*              plan.h:398-405
//
// Page format (the reference's readers, src/build_table.cpp:513-637):
//   INT32    u16 num_rows @0, u16 num_non_null @2, int32 values of the non-NULL
//            rows packed from +4, validity bitmap of ceil(num_rows/8) bytes
//            ending at byte 8192 (bit i of byte i/8 = row i is non-NULL).
//   VARCHAR  u16 num_rows @0, u16 num_non_null @2, u16 cumulative end offsets of
//            the non-NULL strings from +4, string bytes right after the offsets,
//            bitmap at the tail as for INT32.  A string longer than 8185 bytes
//            is stored alone on a 0xffff page (u16 byte count @2, bytes from +4)
//            continued on 0xfffe pages.
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <string>
#include <string_view>
#include <tuple>
#include <variant>
#include <vector>

#include <sys/mman.h>

#include "attribute.h"

class MappedMemory {
public:
    void*  addr;
    size_t length;
    size_t refs;

    MappedMemory(void* addr, size_t length)
    : addr(addr), length(length), refs(0) {}

    MappedMemory(const MappedMemory&)            = delete;
    MappedMemory& operator=(const MappedMemory&) = delete;

    MappedMemory(MappedMemory&& o) noexcept
    : addr(o.addr), length(o.length), refs(o.refs) {
        o.addr = nullptr;
        o.length = 0;
        o.refs = 0;
    }

    MappedMemory& operator=(MappedMemory&& o) noexcept {
        if (this != &o) {
            addr   = o.addr;
            length = o.length;
            refs   = o.refs;
            o.addr = nullptr;
            o.length = 0;
            o.refs = 0;
        }
        return *this;
    }

    ~MappedMemory() {
        if (addr != nullptr) munmap(addr, length);
    }
};

enum class NodeType {
    HashJoin,
    Scan,
};

struct ScanNode {
    size_t base_table_id;
};

struct JoinNode {
    bool   build_left;
    size_t left;
    size_t right;
    size_t left_attr;
    size_t right_attr;
};

struct PlanNode {
    std::variant<ScanNode, JoinNode>          data;
    std::vector<std::tuple<size_t, DataType>> output_attrs;

    PlanNode(std::variant<ScanNode, JoinNode> data,
             std::vector<std::tuple<size_t, DataType>> output_attrs)
    : data(std::move(data)), output_attrs(std::move(output_attrs)) {}
};

constexpr size_t PAGE_SIZE = 8192;

struct alignas(8) Page {
    std::byte data[PAGE_SIZE];
};

struct Column {
    DataType           type;
    std::vector<Page*> pages;
    MappedMemory*      mapped_memory;

    Page* new_page() {
        auto* p = new Page;
        pages.push_back(p);
        return p;
    }

    void assign_mapped_memory(MappedMemory* m) {
        mapped_memory = m;
        mapped_memory->refs++;
    }

    Column(DataType data_type)
    : type(data_type), pages(), mapped_memory(nullptr) {}

    Column(Column&& o) noexcept
    : type(o.type), pages(std::move(o.pages)), mapped_memory(o.mapped_memory) {
        o.pages.clear();
        o.mapped_memory = nullptr;
    }

    Column& operator=(Column&& o) noexcept {
        if (this != &o) {
            release();
            type  = o.type;
            pages = std::move(o.pages);
            o.pages.clear();
            mapped_memory   = o.mapped_memory;
            o.mapped_memory = nullptr;
        }
        return *this;
    }

    Column(const Column&)            = delete;
    Column& operator=(const Column&) = delete;

    ~Column() { release(); }

private:
    // Pages of a mapped column belong to the mapping; otherwise each page was
    // allocated by `new_page` and is owned here.
    void release() {
        if (mapped_memory != nullptr) {
            if (--mapped_memory->refs == 0) delete mapped_memory;
            mapped_memory = nullptr;
            pages.clear();
            return;
        }
        for (auto* p : pages) delete p;
        pages.clear();
    }
};

struct ColumnarTable {
    size_t              num_rows{0};
    std::vector<Column> columns;
};

std::tuple<std::vector<std::vector<Data>>, std::vector<DataType>> from_columnar(
    const ColumnarTable& table);
ColumnarTable from_table(const std::vector<std::vector<Data>>& table,
                         const std::vector<DataType>&          data_types);

struct Plan {
    std::vector<PlanNode>      nodes;
    std::vector<ColumnarTable> inputs;
    size_t                     root;

    size_t new_join_node(bool build_left, size_t left, size_t right, size_t left_attr,
                         size_t right_attr,
                         std::vector<std::tuple<size_t, DataType>> output_attrs) {
        JoinNode j{build_left, left, right, left_attr, right_attr};
        nodes.emplace_back(j, std::move(output_attrs));
        return nodes.size() - 1;
    }

    size_t new_scan_node(size_t base_table_id,
                         std::vector<std::tuple<size_t, DataType>> output_attrs) {
        ScanNode s{base_table_id};
        nodes.emplace_back(s, std::move(output_attrs));
        return nodes.size() - 1;
    }

    size_t new_input(ColumnarTable input) {
        inputs.emplace_back(std::move(input));
        return inputs.size() - 1;
    }
};

// Page writers with the reference's packing rules (plan.h:212-396): a value is
// appended while the page, including it, still fits in 8192 bytes; fixed-width
// data starts at max(4, sizeof(T)); strings longer than 8185 bytes go to
// 0xffff/0xfffe long-string pages.
template <class T>
struct ColumnInserter {
    Column&              column;
    size_t               last_page_idx = 0;
    uint16_t             num_rows      = 0;
    size_t               data_end      = data_begin();
    std::vector<uint8_t> bitmap;

    static constexpr size_t data_begin() { return sizeof(T) < 4 ? 4 : sizeof(T); }

    explicit ColumnInserter(Column& c) : column(c) { bitmap.resize(PAGE_SIZE); }

    std::byte* get_page() {
        if (last_page_idx == column.pages.size()) column.new_page();
        return column.pages[last_page_idx]->data;
    }

    void save_page() {
        auto* page = get_page();
        const uint16_t non_null = uint16_t((data_end - data_begin()) / sizeof(T));
        std::memcpy(page, &num_rows, 2);
        std::memcpy(page + 2, &non_null, 2);
        const size_t bm = (num_rows + 7) / 8;
        std::memcpy(page + PAGE_SIZE - bm, bitmap.data(), bm);
        ++last_page_idx;
        num_rows = 0;
        data_end = data_begin();
    }

    void set_bit(size_t i, bool on) {
        if (on) bitmap[i / 8] |= uint8_t(1u << (i % 8));
        else    bitmap[i / 8] &= uint8_t(~(1u << (i % 8)));
    }

    void insert(T value) {
        if (data_end + 4 + num_rows / 8 + 1 > PAGE_SIZE) save_page();
        std::memcpy(get_page() + data_end, &value, sizeof(T));
        data_end += sizeof(T);
        set_bit(num_rows, true);
        ++num_rows;
    }

    void insert_null() {
        if (data_end + num_rows / 8 + 1 > PAGE_SIZE) save_page();
        set_bit(num_rows, false);
        ++num_rows;
    }

    void finalize() {
        if (num_rows != 0) save_page();
    }
};

template <>
struct ColumnInserter<std::string> {
    Column&              column;
    size_t               last_page_idx = 0;
    uint16_t             num_rows      = 0;
    uint16_t             data_size     = 0;
    size_t               offset_end    = 4;
    std::vector<char>    data;
    std::vector<uint8_t> bitmap;

    static constexpr size_t offset_begin() { return 4; }

    explicit ColumnInserter(Column& c) : column(c) {
        data.resize(PAGE_SIZE);
        bitmap.resize(PAGE_SIZE);
    }

    std::byte* get_page() {
        if (last_page_idx == column.pages.size()) column.new_page();
        return column.pages[last_page_idx]->data;
    }

    void save_long_string(std::string_view v) {
        size_t off = 0;
        bool   first = true;
        while (off < v.size()) {
            auto*          page = get_page();
            const uint16_t tag  = first ? 0xffff : 0xfffe;
            first               = false;
            const uint16_t len  = uint16_t(std::min(v.size() - off, PAGE_SIZE - 4));
            std::memcpy(page, &tag, 2);
            std::memcpy(page + 2, &len, 2);
            std::memcpy(page + 4, v.data() + off, len);
            off += len;
            ++last_page_idx;
        }
    }

    void save_page() {
        auto*          page     = get_page();
        const uint16_t non_null = uint16_t((offset_end - offset_begin()) / 2);
        std::memcpy(page, &num_rows, 2);
        std::memcpy(page + 2, &non_null, 2);
        std::memcpy(page + offset_end, data.data(), data_size);
        const size_t bm = (num_rows + 7) / 8;
        std::memcpy(page + PAGE_SIZE - bm, bitmap.data(), bm);
        ++last_page_idx;
        num_rows   = 0;
        data_size  = 0;
        offset_end = offset_begin();
    }

    void set_bit(size_t i, bool on) {
        if (on) bitmap[i / 8] |= uint8_t(1u << (i % 8));
        else    bitmap[i / 8] &= uint8_t(~(1u << (i % 8)));
    }

    void insert(std::string_view v) {
        if (v.size() > PAGE_SIZE - 7) {
            if (num_rows > 0) save_page();
            save_long_string(v);
            return;
        }
        if (offset_end + 2 + data_size + v.size() + num_rows / 8 + 1 > PAGE_SIZE) save_page();
        std::memcpy(data.data() + data_size, v.data(), v.size());
        data_size = uint16_t(data_size + v.size());
        std::memcpy(get_page() + offset_end, &data_size, 2);
        offset_end += 2;
        set_bit(num_rows, true);
        ++num_rows;
    }

    void insert_null() {
        if (offset_end + data_size + num_rows / 8 + 1 > PAGE_SIZE) save_page();
        set_bit(num_rows, false);
        ++num_rows;
    }

    void finalize() {
        if (num_rows != 0) save_page();
    }
};

namespace Contest {

void* build_context();
void  destroy_context(void*);

ColumnarTable execute(const Plan& plan, void* context);

}  // namespace Contest
