// Column data types of the SIGMOD-2025 contest API.
//
// Layout-compatible with the reference's `DataType` (include/attribute.h:8-13
// of eleanalt/hash-join-optimizer): an `enum class` with the same four
// enumerators in the same order, so a `Plan` built against either header has
// the same bytes.  `Data` is the row-table cell type the reference declares in
// include/statement.h:13 (same alternatives, same order).
#pragma once

#include <cstdint>
#include <string>
#include <variant>

enum class DataType {
    INT32,    // 4-byte signed integer
    INT64,    // 8-byte signed integer
    FP64,     // 8-byte IEEE double
    VARCHAR,  // byte string of any length
};

using Data = std::variant<int32_t, int64_t, double, std::string, std::monostate>;

struct Attribute {
    DataType    type;
    std::string name;
};
