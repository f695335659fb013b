// Host page writers: dense arrays -> the reference's page format.
//
// They pack exactly as the reference's writers do (Table::to_columnar,
// src/build_table.cpp:657-882, and ColumnInserter, include/plan.h:212-396): a
// row is appended while the page including it fits in 8192 bytes; INT32 data
// from +4; VARCHAR strings longer than 8185 bytes on 0xffff/0xfffe pages.
// Bytes the reference leaves uninitialised are zero here.
#include <cstdint>
#include <cstring>

#include "../../include/hj_api.h"

namespace {

constexpr uint64_t kPage = 8192;

struct PageOut {
    uint8_t* out;
    uint64_t cap;
    uint64_t n = 0;
    uint8_t* next() {
        uint8_t* p = (out && n < cap) ? out + n * kPage : nullptr;
        if (p) std::memset(p, 0, kPage);
        ++n;
        return p;
    }
};

inline void w16(uint8_t* p, uint16_t v) { std::memcpy(p, &v, 2); }

}  // namespace

extern "C" {

int hj_pages_from_int32(const int32_t* values, const uint8_t* valid, uint64_t n, void* out,
                        uint64_t capacity_pages, uint64_t* num_pages) {
    if (!num_pages || (n > 0 && !values)) return HJ_ERR_INVALID;
    PageOut  po{static_cast<uint8_t*>(out), capacity_pages};
    uint32_t rows = 0, data = 0;  // rows and non-NULL values on the open page
    uint64_t start = 0;           // first row of the open page
    auto save = [&](uint64_t end) {
        uint8_t* pg = po.next();
        if (pg) {
            w16(pg, uint16_t(rows));
            w16(pg + 2, uint16_t(data));
            uint8_t* bm = pg + kPage - (rows + 7) / 8;
            uint32_t d  = 0;
            for (uint64_t r = start; r < end; ++r) {
                const uint32_t i = uint32_t(r - start);
                if (!valid || valid[r]) {
                    std::memcpy(pg + 4 + 4 * size_t(d++), &values[r], 4);
                    bm[i / 8] |= uint8_t(1u << (i % 8));
                }
            }
        }
        rows = data = 0;
        start       = end;
    };
    for (uint64_t r = 0; r < n; ++r) {
        const bool on = !valid || valid[r];
        if (on ? 4 + (data + 1) * 4 + (rows / 8 + 1) > kPage : 4 + data * 4 + (rows / 8 + 1) > kPage)
            save(r);
        data += on;
        ++rows;
    }
    if (rows) save(n);
    *num_pages = po.n;
    return (out && po.n > capacity_pages) ? HJ_ERR_CAPACITY : HJ_OK;
}

int hj_pages_from_strings(const uint8_t* bytes, const uint64_t* offsets, const uint8_t* valid,
                          uint64_t n, void* out, uint64_t capacity_pages, uint64_t* num_pages) {
    if (!num_pages || (n > 0 && !offsets)) return HJ_ERR_INVALID;
    PageOut  po{static_cast<uint8_t*>(out), capacity_pages};
    uint32_t rows = 0, nn = 0, dbytes = 0;
    uint64_t start = 0;
    auto save = [&](uint64_t end) {
        uint8_t* pg = po.next();
        if (pg) {
            w16(pg, uint16_t(rows));
            w16(pg + 2, uint16_t(nn));
            uint8_t* bm  = pg + kPage - (rows + 7) / 8;
            uint8_t* dat = pg + 4 + 2 * size_t(nn);
            uint32_t k = 0, off = 0;
            for (uint64_t r = start; r < end; ++r) {
                const uint32_t i = uint32_t(r - start);
                if (!valid || valid[r]) {
                    const uint64_t len = offsets[r + 1] - offsets[r];
                    std::memcpy(dat + off, bytes + offsets[r], len);
                    off += uint32_t(len);
                    w16(pg + 4 + 2 * size_t(k++), uint16_t(off));
                    bm[i / 8] |= uint8_t(1u << (i % 8));
                }
            }
        }
        rows = nn = dbytes = 0;
        start              = end;
    };
    for (uint64_t r = 0; r < n; ++r) {
        const bool     on  = !valid || valid[r];
        const uint64_t len = on ? offsets[r + 1] - offsets[r] : 0;
        if (on && len > kPage - 7) {  // long string: its own 0xffff/0xfffe pages
            if (rows) save(r);
            for (uint64_t o = 0; o < len; o += kPage - 4) {
                uint8_t* pg = po.next();
                if (!pg) continue;
                const uint64_t part = len - o < kPage - 4 ? len - o : kPage - 4;
                w16(pg, o == 0 ? 0xffff : 0xfffe);
                w16(pg + 2, uint16_t(part));
                std::memcpy(pg + 4, bytes + offsets[r] + o, part);
            }
            start = r + 1;
            continue;
        }
        const uint64_t after = on ? 4 + (nn + 1) * 2 + (dbytes + len) + (rows / 8 + 1)
                                  : 4 + nn * 2 + dbytes + (rows / 8 + 1);
        if (after > kPage) save(r);
        if (on) {
            ++nn;
            dbytes += uint32_t(len);
        }
        ++rows;
    }
    if (rows) save(n);
    *num_pages = po.n;
    return (out && po.n > capacity_pages) ? HJ_ERR_CAPACITY : HJ_OK;
}

}  // extern "C"
