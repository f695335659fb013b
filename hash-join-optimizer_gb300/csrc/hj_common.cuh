// Shared device/host definitions of the GB300 join engine.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "../../include/hj_api.h"

namespace hj {

constexpr int      kPage       = 8192;
constexpr int      kDenseRows  = 1984;        // rows of a full INT32 page (no NULLs)
constexpr uint64_t kFib        = 11400714819323198485ull;  // 2^64 / golden ratio

// Multiprocessors of the current device (152 on a GB300: 2 dies x 76), read
// once per device from cudaDevAttrMultiProcessorCount; grids are sized in
// multiples of it.
int num_sms();

// Engine error carrying an HJ_* status; converted to a return code at the C ABI.
struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define HJ_CUDA(call)                                                                        \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            throw ::hj::Error(HJ_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Kernels launched by this library in this process (every launch site ends
// with HJ_LAUNCH_CHECK, which counts it).
extern std::atomic<uint64_t> g_kernel_launches;

#define HJ_LAUNCH_CHECK()                                        \
    do {                                                         \
        ::hj::g_kernel_launches.fetch_add(1, std::memory_order_relaxed); \
        HJ_CUDA(cudaGetLastError());                             \
    } while (0)

// Unchained-table hash of a join key: libstdc++'s std::hash<int32_t> (the
// sign-extended value) times the Fibonacci constant, as
// UnchainedHash::hash_key (include/unchained.h:56-66 of the reference).
__host__ __device__ __forceinline__ uint64_t fib_hash(int32_t key) {
    return uint64_t(int64_t(key)) * kFib;
}

// Bucket (directory slot) of a hash: its top `bits` bits (0 bits -> slot 0).
__host__ __device__ __forceinline__ uint64_t bucket_of(uint64_t h, uint32_t bits) {
    return bits == 0 ? 0 : (h >> (64 - bits));
}

// 16-bit Bloom mask of a hash: one bit per nibble of its low 16 bits
// (UnchainedHash::bloom_mask, include/unchained.h:110-117).
__host__ __device__ __forceinline__ uint32_t bloom_mask(uint64_t h) {
    const uint32_t s = uint32_t(h) & 0xffffu;
    return (1u << (s & 15)) | (1u << ((s >> 4) & 15)) | (1u << ((s >> 8) & 15))
         | (1u << ((s >> 12) & 15));
}

// Bucket summary: the engine's probe-side companion of a directory word (the
// directory itself keeps UnchainedHash's layout).  One 8-byte load gives the
// probe everything a bucket of one key needs:
//   bits  0..31  first key of the bucket's tuples (0 when empty)
//   bits 32..47  the bucket's 16-bit Bloom tag (the directory word's low bits)
//   bits 48..62  tuples in the bucket, saturated at kSumLenMax
//   bit  63      the bucket holds more than one distinct key ("mixed")
// An empty bucket's summary is 0.
constexpr uint32_t kSumLenMax = 0x7fffu;

__host__ __device__ __forceinline__ uint64_t make_summary(int32_t head, uint32_t bloom, uint32_t len, bool mixed) {
    const uint64_t l = len < kSumLenMax ? len : kSumLenMax;
    return uint64_t(uint32_t(head)) | (uint64_t(bloom & 0xffffu) << 32) | (l << 48) | (uint64_t(mixed) << 63);
}
__host__ __device__ __forceinline__ int32_t  sum_head(uint64_t w) { return int32_t(uint32_t(w)); }
__host__ __device__ __forceinline__ uint32_t sum_bloom(uint64_t w) { return uint32_t(w >> 32) & 0xffffu; }
__host__ __device__ __forceinline__ uint32_t sum_len(uint64_t w) { return uint32_t(w >> 48) & kSumLenMax; }
__host__ __device__ __forceinline__ bool     sum_mixed(uint64_t w) { return (w >> 63) != 0; }

__device__ __forceinline__ bool bit_valid(const uint32_t* bm, uint64_t i) {
    return bm == nullptr || ((__ldg(bm + (i >> 5)) >> (i & 31)) & 1u);
}

__device__ __forceinline__ uint16_t ld16(const uint8_t* p) {
    return uint16_t(p[0]) | uint16_t(uint16_t(p[1]) << 8);
}

// An INT32 base column on the device, in one of three forms:
//  * direct: the raw input pages, every page but the last dense with 1984 rows
//    (the reference's column_t "direct" mode, include/column_t.h:46-66): row r
//    is int32 number r % 1984 after the 4-byte header of page r / 1984;
//  * plain:  int32 values, NULLs marked in an optional validity bitmap;
//  * tagged: one value_t per row (tag 01 + value, 0 = NULL), so a random
//    gather fetches value and validity with one load.
struct IntCol {
    const uint8_t*  pages  = nullptr;
    const int32_t*  plain  = nullptr;
    const uint32_t* valid  = nullptr;  // with `plain` only
    const uint64_t* tagged = nullptr;
};

__device__ __forceinline__ bool int_get(const IntCol& c, uint64_t r, int32_t& v) {
    if (c.tagged) {
        const uint64_t t = __ldg(c.tagged + r);
        v                = int32_t(uint32_t(t));
        return (t >> 62) == 1;
    }
    if (c.plain) {
        v = __ldg(c.plain + r);
        return bit_valid(c.valid, r);
    }
    // page of row r: a 32-bit division by the constant for rows below 2^32
    // (every column the engine reads), the 64-bit one above
    uint64_t p;
    if ((r >> 32) == 0) p = uint32_t(r) / uint32_t(kDenseRows);
    else                p = r / uint64_t(kDenseRows);
    v = __ldg(reinterpret_cast<const int32_t*>(c.pages + p * kPage + 4) + (r - p * uint64_t(kDenseRows)));
    return true;
}

// Scan predicates (hj_filter) over INT32 base columns, AND-combined.
constexpr int kMaxFilters = HJ_MAX_SCAN_FILTERS;
struct Filt {
    IntCol  col;
    int32_t op;
    int32_t val;
};
struct Filters {
    int  n = 0;
    Filt f[kMaxFilters];
};

// Comparisons as truth tables over a value's state: 0 greater than the
// literal, 1 equal, 2 less, 3 NULL.  NULL never compares true; IS_NULL /
// IS_NOT_NULL test validity (the reference's bitmap & comparison).
__host__ __device__ __forceinline__ uint32_t cmp_table(int32_t op) {
    switch (op) {
        case HJ_CMP_EQ: return 0x2u;
        case HJ_CMP_NEQ: return 0x5u;
        case HJ_CMP_LT: return 0x4u;
        case HJ_CMP_GT: return 0x1u;
        case HJ_CMP_LEQ: return 0x6u;
        case HJ_CMP_GEQ: return 0x3u;
        case HJ_CMP_IS_NULL: return 0x8u;
        default: return 0x7u;  // HJ_CMP_IS_NOT_NULL
    }
}
__device__ __forceinline__ uint32_t cmp_state(bool valid, int32_t v, int32_t x) {
    return valid ? (v < x ? 2u : (v == x ? 1u : 0u)) : 3u;
}
__device__ __forceinline__ bool cmp_ok(int32_t op, bool valid, int32_t v, int32_t x) {
    return (cmp_table(op) >> cmp_state(valid, v, x)) & 1u;
}

// Does base row r pass every filter?
__device__ __forceinline__ bool filt_pass(const Filters& F, uint64_t r) {
    for (int i = 0; i < F.n; ++i) {
        int32_t    v     = 0;
        const bool valid = int_get(F.f[i].col, r, v);
        if (!cmp_ok(F.f[i].op, valid, v, F.f[i].val)) return false;
    }
    return true;
}

// A VARCHAR base column is decoded to one 64-bit locator per row: 0 = NULL;
// otherwise bit 63 set, bit 62 = long string (0xffff page + 0xfffe pages),
// bits 40..61 = byte length (saturated at 2^22 - 1 for long strings, whose
// length is then re-read from their pages), bits 0..39 = byte offset of the
// string (normal) or of its 0xffff page (long) in the column's page buffer.
constexpr uint64_t kLocValid   = 1ull << 63;
constexpr uint64_t kLocLong    = 1ull << 62;
constexpr uint64_t kLocLenMax  = (1ull << 22) - 1;

__host__ __device__ __forceinline__ uint64_t make_loc(uint64_t off, uint64_t len, bool is_long) {
    return kLocValid | (is_long ? kLocLong : 0) | ((len < kLocLenMax ? len : kLocLenMax) << 40)
         | (off & ((1ull << 40) - 1));
}
__host__ __device__ __forceinline__ uint64_t loc_off(uint64_t loc) { return loc & ((1ull << 40) - 1); }
__host__ __device__ __forceinline__ uint64_t loc_len_field(uint64_t loc) { return (loc >> 40) & kLocLenMax; }

// Byte length of a long string starting at the 0xffff page `pg` (its page and
// the 0xfffe pages after it).
__device__ __forceinline__ uint32_t long_len(const uint8_t* base, uint64_t pg, uint64_t npages) {
    uint32_t len = *reinterpret_cast<const uint16_t*>(base + pg * kPage + 2);
    for (uint64_t q = pg + 1; q < npages; ++q) {
        const uint8_t* nx = base + q * kPage;
        if (*reinterpret_cast<const uint16_t*>(nx) != 0xfffe) break;
        len += *reinterpret_cast<const uint16_t*>(nx + 2);
    }
    return len;
}

inline unsigned div_up(uint64_t a, uint64_t b) { return unsigned((a + b - 1) / b); }

}  // namespace hj
