// Page decode: reference-format input pages in HBM -> dense device columns.
//
// This is the device form of copy_scan (src/execute.cpp:265-369 of the
// reference): INT32 pages become int32 values + a validity bitmap, VARCHAR
// pages become one value_t per row holding StrRef(table, column, page,
// ordinal-among-non-NULL) exactly as the reference encodes it, long strings
// (0xffff page) become one row and 0xfffe continuation pages none.
#include "../../include/value_t.h"
#include "hj_block.cuh"
#include "hj_common.cuh"
#include "hj_kernels.h"

namespace hj {
namespace {

constexpr int kDecThreads = 256;

__global__ void k_page_headers(const uint8_t* __restrict__ pages, uint64_t num_pages, int32_t type,
                               uint32_t* __restrict__ rows, uint32_t* __restrict__ non_null,
                               uint32_t* __restrict__ flags) {
    const uint64_t p = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= num_pages) return;
    const uint8_t* pg = pages + p * kPage;
    const uint16_t nr = *reinterpret_cast<const uint16_t*>(pg);
    const uint16_t nn = *reinterpret_cast<const uint16_t*>(pg + 2);
    uint32_t r = 0, v = 0, f = 0;
    if (type == HJ_INT32) {
        r = nr;
        v = nn;
        f = nr != nn ? 1u : 0u;
    } else if (type == HJ_VARCHAR) {
        if (nr == 0xffff) {
            r = 1;
            v = 1;
        } else if (nr != 0xfffe) {
            r = nr;
            v = nn;
            f = nr != nn ? 1u : 0u;
        }
        if (p > StrRef::PAGE_MASK && v > 0) f |= 2u;
    }
    rows[p]     = r;
    non_null[p] = v;
    flags[p]    = f;
}

// ORs the validity of 32 consecutive rows starting at global row g into the
// bitmap (the 32 rows may straddle two words).
__device__ __forceinline__ void or_bits(uint32_t* bm, uint64_t g, uint32_t ballot) {
    if (ballot == 0) return;
    const uint64_t w  = g >> 5;
    const unsigned sh = unsigned(g & 31);
    atomicOr(bm + w, ballot << sh);
    if (sh != 0 && (ballot >> (32 - sh)) != 0) atomicOr(bm + w + 1, ballot >> (32 - sh));
}

__global__ void __launch_bounds__(kDecThreads)
    k_decode_int32(const uint8_t* __restrict__ pages, const uint64_t* __restrict__ row_start,
                   int32_t* __restrict__ vals, uint32_t* __restrict__ valid) {
    __shared__ uint32_t sm[33];
    const uint64_t  p    = blockIdx.x;
    const uint8_t*  pg   = pages + p * kPage;
    const uint32_t  nr   = *reinterpret_cast<const uint16_t*>(pg);
    const uint32_t  nn   = *reinterpret_cast<const uint16_t*>(pg + 2);
    const int32_t*  data = reinterpret_cast<const int32_t*>(pg + 4);
    const uint8_t*  bm   = pg + kPage - (nr + 7) / 8;
    const uint64_t  r0   = row_start[p];
    if (nr == nn) {  // dense page: rows are the packed values
        for (uint32_t i = threadIdx.x; i < nr; i += blockDim.x) vals[r0 + i] = data[i];
        if (valid) {
            for (uint32_t c = 0; c < nr; c += blockDim.x) {
                const uint32_t i = c + threadIdx.x;
                const uint32_t b = __ballot_sync(0xffffffffu, i < nr);
                if ((threadIdx.x & 31) == 0) or_bits(valid, r0 + c + (threadIdx.x & ~31u), b);
            }
        }
        return;
    }
    uint32_t rank_base = 0;
    for (uint32_t c = 0; c < nr; c += blockDim.x) {
        const uint32_t i  = c + threadIdx.x;
        const bool     on = i < nr && ((bm[i >> 3] >> (i & 7)) & 1u);
        uint32_t       total;
        const uint32_t rank = rank_base + block_exclusive_scan<uint32_t>(on ? 1u : 0u, sm, &total);
        // a well-formed page has rank < num_non_null <= 2047; never read past it
        if (i < nr) vals[r0 + i] = (on && rank < (kPage - 4) / 4) ? data[rank] : 0;
        const uint32_t b = __ballot_sync(0xffffffffu, on);
        if (valid && (threadIdx.x & 31) == 0) or_bits(valid, r0 + c + (threadIdx.x & ~31u), b);
        rank_base += total;
    }
}

__global__ void __launch_bounds__(kDecThreads)
    k_decode_varchar(const uint8_t* __restrict__ pages, const uint64_t* __restrict__ row_start,
                     uint32_t table_id, uint32_t column, uint64_t* __restrict__ refs,
                     uint32_t* __restrict__ valid) {
    __shared__ uint32_t sm[33];
    const uint64_t p  = blockIdx.x;
    const uint8_t* pg = pages + p * kPage;
    const uint32_t nr = *reinterpret_cast<const uint16_t*>(pg);
    const uint64_t r0 = row_start[p];
    if (nr == 0xfffe) return;
    if (nr == 0xffff) {
        if (threadIdx.x == 0) {
            refs[r0] = StrRef::pack(true, table_id, column, p, 0) | value_t::TAG_STRREF;
            atomicOr(valid + (r0 >> 5), 1u << (r0 & 31));
        }
        return;
    }
    const uint8_t* bm        = pg + kPage - (nr + 7) / 8;
    uint32_t       rank_base = 0;
    for (uint32_t c = 0; c < nr; c += blockDim.x) {
        const uint32_t i  = c + threadIdx.x;
        const bool     on = i < nr && ((bm[i >> 3] >> (i & 7)) & 1u);
        uint32_t       total;
        const uint32_t rank = rank_base + block_exclusive_scan<uint32_t>(on ? 1u : 0u, sm, &total);
        if (i < nr)
            refs[r0 + i] = on ? (StrRef::pack(false, table_id, column, p, rank) | value_t::TAG_STRREF)
                              : 0ull;
        const uint32_t b = __ballot_sync(0xffffffffu, on);
        if ((threadIdx.x & 31) == 0) or_bits(valid, r0 + c + (threadIdx.x & ~31u), b);
        rank_base += total;
    }
}

}  // namespace

void launch_page_headers(const uint8_t* pages, uint64_t num_pages, int32_t type, uint32_t* rows,
                         uint32_t* non_null, uint32_t* flags, cudaStream_t st) {
    if (num_pages == 0) return;
    k_page_headers<<<div_up(num_pages, 256), 256, 0, st>>>(pages, num_pages, type, rows, non_null,
                                                           flags);
    HJ_LAUNCH_CHECK();
}

void launch_decode_int32(const uint8_t* pages, uint64_t num_pages, const uint64_t* row_start,
                         int32_t* vals, uint32_t* valid, cudaStream_t st) {
    if (num_pages == 0) return;
    k_decode_int32<<<unsigned(num_pages), kDecThreads, 0, st>>>(pages, row_start, vals, valid);
    HJ_LAUNCH_CHECK();
}

void launch_decode_varchar(const uint8_t* pages, uint64_t num_pages, const uint64_t* row_start,
                           uint32_t table_id, uint32_t column, uint64_t* refs, uint32_t* valid,
                           cudaStream_t st) {
    if (num_pages == 0) return;
    k_decode_varchar<<<unsigned(num_pages), kDecThreads, 0, st>>>(pages, row_start, table_id,
                                                                  column, refs, valid);
    HJ_LAUNCH_CHECK();
}

}  // namespace hj
