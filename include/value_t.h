// 64-bit tagged values and string references of the join engine.
//
// The bit layouts are a contract with the reference (include/value_t.h:7-127 of
// eleanalt/hash-join-optimizer) and are kept identical:
//
//   StrRef   bit 61      long-string flag (string spans 0xffff/0xfffe pages)
//            bits 51..60 input table id      (10 bits)
//            bits 41..50 input column index  (10 bits)
//            bits 23..40 page index          (18 bits)
//            bits  7..22 offset index        (16 bits: ordinal of the string
//                                             among the page's non-NULL rows)
//            bits  0..6  zero padding
//   value_t  bits 63..62 tag: 01 INT32, 10 StrRef, 00 NULL
//            INT32 payload in bits 0..31 (two's complement, zero-extended)
//
// Encoders throw std::out_of_range on a field overflow, as the reference does
// (value_t.h:36-47); the device side checks the same limits on the host before
// any StrRef is formed.  Everything here is usable from CUDA device code.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>

#if defined(__CUDACC__)
#define HJ_HD __host__ __device__ __forceinline__
#else
#define HJ_HD inline
#endif

struct StrRef {
    uint64_t ref = 0;

    static constexpr uint64_t LONGSTR_BIT = 1ull << 61;

    static constexpr int TABLE_LEN  = 10;
    static constexpr int COLUMN_LEN = 10;
    static constexpr int PAGE_LEN   = 18;
    static constexpr int OFFSET_LEN = 16;
    static constexpr int PADDING    = 7;

    static constexpr int OFFSET_SHIFT = PADDING;
    static constexpr int PAGE_SHIFT   = OFFSET_SHIFT + OFFSET_LEN;
    static constexpr int COLUMN_SHIFT = PAGE_SHIFT + PAGE_LEN;
    static constexpr int TABLE_SHIFT  = COLUMN_SHIFT + COLUMN_LEN;

    static constexpr uint64_t TABLE_MASK  = (1ull << TABLE_LEN) - 1;
    static constexpr uint64_t COLUMN_MASK = (1ull << COLUMN_LEN) - 1;
    static constexpr uint64_t PAGE_MASK   = (1ull << PAGE_LEN) - 1;
    static constexpr uint64_t OFFSET_MASK = (1ull << OFFSET_LEN) - 1;

    StrRef() = default;

    StrRef(bool is_long, uint64_t table, uint64_t col, uint64_t page, uint64_t off_idx) {
        encode(is_long, table, col, page, off_idx);
    }

    static void check_field(const char* what, uint64_t v, uint64_t mask) {
        if (v > mask) {
            throw std::out_of_range(std::string("StrRef ") + what + " overflow: "
                                    + std::to_string(v) + " > " + std::to_string(mask));
        }
    }

    // Same contract as the reference: ORs the fields into `ref` (callers start
    // from a cleared reference), throwing before any bit is written.
    void encode(bool is_long = false, uint64_t table = 0, uint64_t col = 0,
                uint64_t page = 0, uint64_t off_idx = 0) {
        check_field("table", table, TABLE_MASK);
        check_field("column", col, COLUMN_MASK);
        check_field("page", page, PAGE_MASK);
        check_field("offset", off_idx, OFFSET_MASK);
        ref |= pack(is_long, table, col, page, off_idx);
    }

    // Unchecked packing for code that has already validated the field ranges
    // (device kernels; fields are validated on the host per column).
    static HJ_HD uint64_t pack(bool is_long, uint64_t table, uint64_t col, uint64_t page,
                               uint64_t off_idx) {
        return (is_long ? LONGSTR_BIT : 0ull) | ((table & TABLE_MASK) << TABLE_SHIFT)
             | ((col & COLUMN_MASK) << COLUMN_SHIFT) | ((page & PAGE_MASK) << PAGE_SHIFT)
             | ((off_idx & OFFSET_MASK) << OFFSET_SHIFT);
    }

    void clear() { ref = 0; }

    HJ_HD size_t get_table() const { return (ref >> TABLE_SHIFT) & TABLE_MASK; }
    HJ_HD size_t get_column() const { return (ref >> COLUMN_SHIFT) & COLUMN_MASK; }
    HJ_HD size_t get_page() const { return (ref >> PAGE_SHIFT) & PAGE_MASK; }
    HJ_HD size_t get_offset() const { return (ref >> OFFSET_SHIFT) & OFFSET_MASK; }
    HJ_HD bool   is_long() const { return (ref & LONGSTR_BIT) != 0; }
};

struct value_t {
    // tag in bits 63..62: 01 INT32, 10 StrRef, 00 NULL
    uint64_t value = 0;

    static constexpr uint64_t TAG_MASK   = 3ull << 62;
    static constexpr uint64_t TAG_INT32  = 1ull << 62;
    static constexpr uint64_t TAG_STRREF = 1ull << 63;

    HJ_HD void parse_int32(int32_t num) { value = uint64_t(uint32_t(num)) | TAG_INT32; }
    HJ_HD void parse_strref(StrRef str) { value = (str.ref & ~TAG_MASK) | TAG_STRREF; }

    HJ_HD bool is_int32() const { return (value >> 62) == 1; }
    HJ_HD bool is_strref() const { return (value >> 62) == 2; }
    HJ_HD bool is_null() const { return (value >> 62) == 0; }

    HJ_HD int32_t get_int32() const { return int32_t(uint32_t(value)); }
    HJ_HD StrRef  get_strref() const {
        StrRef r;
        r.ref = value & ~TAG_MASK;
        return r;
    }
};

static_assert(sizeof(StrRef) == 8 && sizeof(value_t) == 8, "tagged values are 64-bit");
