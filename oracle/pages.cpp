// Test infrastructure (oracle only): host writers of the reference page
// format, restating the reference's column writers so that a process can build
// input tables without the engine library (the reference arm of bench.py).
//
// Rules restated (include/plan.h:212-396, ColumnInserter<int32_t> /
// ColumnInserter<std::string>, as used by Table::to_columnar,
// src/build_table.cpp:657-882):
//   * INT32: a value is appended while 4 + 4 * (values + 1) + (rows / 8 + 1)
//     stays within 8192 bytes, a NULL while 4 + 4 * values + (rows / 8 + 1)
//     does; header (u16 rows, u16 values), values from byte 4, bitmap at the
//     page end (bit i of byte i / 8).
//   * VARCHAR: a string of more than 8185 bytes closes the open page and is
//     written on one 0xffff page plus 0xfffe continuation pages of up to 8188
//     bytes each; otherwise it is appended while 4 + 2 * (strings + 1) +
//     bytes + len + (rows / 8 + 1) fits; offsets are the u16 end of each string
//     after the offset array.
// Bytes the reference leaves uninitialised are zero.
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr size_t kPage = 8192;

void put16(uint8_t* p, uint16_t v) { std::memcpy(p, &v, 2); }

// Pages grown one at a time into a caller buffer (counting only when the
// buffer is absent or full).
struct Sink {
    uint8_t* out;
    uint64_t cap;
    uint64_t used = 0;
    uint8_t* page() {
        uint8_t* p = (out && used < cap) ? out + used * kPage : nullptr;
        if (p) std::memset(p, 0, kPage);
        ++used;
        return p;
    }
};

}  // namespace

extern "C" {

// values[n] with optional valid[n] (0 = NULL) -> INT32 pages.  Returns 0, or 6
// (capacity) when `out` has fewer than the needed pages; *num_pages is the need.
int oracle_pages_from_int32(const int32_t* values, const uint8_t* valid, uint64_t n, void* out,
                            uint64_t capacity_pages, uint64_t* num_pages) {
    Sink                 sink{static_cast<uint8_t*>(out), capacity_pages};
    std::vector<int32_t> vals;
    std::vector<uint8_t> bits;  // one byte per row of the open page
    auto flush = [&] {
        if (bits.empty()) return;
        if (uint8_t* pg = sink.page()) {
            put16(pg, uint16_t(bits.size()));
            put16(pg + 2, uint16_t(vals.size()));
            std::memcpy(pg + 4, vals.data(), vals.size() * 4);
            uint8_t* bm = pg + kPage - (bits.size() + 7) / 8;
            for (size_t i = 0; i < bits.size(); ++i)
                if (bits[i]) bm[i / 8] |= uint8_t(1u << (i % 8));
        }
        vals.clear();
        bits.clear();
    };
    for (uint64_t r = 0; r < n; ++r) {
        const bool   on   = !valid || valid[r];
        const size_t need = 4 + 4 * (vals.size() + (on ? 1 : 0)) + (bits.size() / 8 + 1);
        if (need > kPage) flush();
        if (on) vals.push_back(values[r]);
        bits.push_back(on);
    }
    flush();
    *num_pages = sink.used;
    return (out && sink.used > capacity_pages) ? 6 : 0;
}

// Strings bytes[offsets[i] .. offsets[i + 1]) with optional valid[n] -> VARCHAR pages.
int oracle_pages_from_strings(const uint8_t* bytes, const uint64_t* offsets, const uint8_t* valid,
                              uint64_t n, void* out, uint64_t capacity_pages, uint64_t* num_pages) {
    Sink                  sink{static_cast<uint8_t*>(out), capacity_pages};
    std::vector<uint8_t>  data;
    std::vector<uint16_t> ends;
    std::vector<uint8_t>  bits;
    auto flush = [&] {
        if (bits.empty()) return;
        if (uint8_t* pg = sink.page()) {
            put16(pg, uint16_t(bits.size()));
            put16(pg + 2, uint16_t(ends.size()));
            std::memcpy(pg + 4, ends.data(), ends.size() * 2);
            std::memcpy(pg + 4 + ends.size() * 2, data.data(), data.size());
            uint8_t* bm = pg + kPage - (bits.size() + 7) / 8;
            for (size_t i = 0; i < bits.size(); ++i)
                if (bits[i]) bm[i / 8] |= uint8_t(1u << (i % 8));
        }
        data.clear();
        ends.clear();
        bits.clear();
    };
    for (uint64_t r = 0; r < n; ++r) {
        const bool     on  = !valid || valid[r];
        const uint64_t len = on ? offsets[r + 1] - offsets[r] : 0;
        if (on && len > kPage - 7) {
            flush();
            for (uint64_t o = 0; o < len; o += kPage - 4) {
                const uint64_t part = len - o < kPage - 4 ? len - o : kPage - 4;
                if (uint8_t* pg = sink.page()) {
                    put16(pg, o == 0 ? 0xffff : 0xfffe);
                    put16(pg + 2, uint16_t(part));
                    std::memcpy(pg + 4, bytes + offsets[r] + o, part);
                }
            }
            continue;
        }
        const size_t need = 4 + 2 * (ends.size() + (on ? 1 : 0)) + data.size() + len + (bits.size() / 8 + 1);
        if (need > kPage) flush();
        if (on) {
            data.insert(data.end(), bytes + offsets[r], bytes + offsets[r] + len);
            ends.push_back(uint16_t(data.size()));
        }
        bits.push_back(on);
    }
    flush();
    *num_pages = sink.used;
    return (out && sink.used > capacity_pages) ? 6 : 0;
}

}  // extern "C"
