// Page decode: reference-format input pages in HBM -> device columns.
//
// The device form of copy_scan (src/execute.cpp:265-369 of the reference).
// A dense INT32 column whose pages hold 1984 rows each needs no decode at
// all: kernels read it in place, like the reference's column_t direct mode.
// Other columns are decoded once per query:
//  * INT32 with NULLs -> value_t per row (tag 01 + value, 0 = NULL), exactly
//    the reference's value_t encoding (include/value_t.h:92-127);
//  * INT32 without NULLs but irregular pages -> plain int32;
//  * VARCHAR -> a 64-bit byte locator per row (see hj_common.cuh): the
//    StrRef(table, column, page, ordinal) of the reference resolved to where
//    the bytes are, so the final page writer gathers them with one load.
//    The bytes themselves stay in the input pages until that writer runs.
#include <algorithm>

#include "../../include/value_t.h"
#include "hj_block.cuh"
#include "hj_common.cuh"
#include "hj_kernels.h"

namespace hj {
namespace {

constexpr int kDecThreads = 256;

__global__ void k_page_rows(const uint8_t* __restrict__ pages, uint64_t num_pages, int32_t type,
                            uint32_t* __restrict__ rows) {
    const uint64_t p = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= num_pages) return;
    const uint16_t nr = *reinterpret_cast<const uint16_t*>(pages + p * kPage);
    uint32_t       r  = nr;
    if (type == HJ_VARCHAR) r = nr == 0xffff ? 1u : (nr == 0xfffe ? 0u : nr);
    rows[p] = r;
}

// INT32 pages: one block per page (grid-stride over pages).  The page, which
// is almost all values and bitmap, is copied into
// shared memory with one 16-byte load per thread per 4 KB (all in flight
// together); a warp scan of the bitmap words' popcounts gives every 32-row
// group its first non-NULL rank; then thread t decodes rows t, t + 256, ...
// from shared memory (rank = group base + popcount of the lower bits) and
// stores them coalesced.  No global load depends on another.
constexpr uint32_t kMaxWords = (kPage * 8 + 31) / 32;  // bitmap words of a page, at most

struct PageSmem {
    uint4    img[kPage / 16];
    uint32_t base[kMaxWords];  // non-NULL rows before each 32-row group
};

// Copies page `pg` into s.img and fills s.base for its nr rows; returns the
// bitmap's byte offset within the page.  Ends with a block barrier.
__device__ __forceinline__ uint32_t stage_page(const uint8_t* __restrict__ pg, uint32_t nr, PageSmem& s) {
    const uint4* src = reinterpret_cast<const uint4*>(pg);
    uint4        v[kPage / 16 / kDecThreads];
#pragma unroll
    for (int k = 0; k < kPage / 16 / kDecThreads; ++k) v[k] = __ldg(src + threadIdx.x + k * kDecThreads);
#pragma unroll
    for (int k = 0; k < kPage / 16 / kDecThreads; ++k) s.img[threadIdx.x + k * kDecThreads] = v[k];
    __syncthreads();
    const uint8_t* b    = reinterpret_cast<const uint8_t*>(s.img);
    const uint32_t bm0  = kPage - (nr + 7) / 8;
    const uint32_t nw   = (nr + 31) / 32;
    if (threadIdx.x < 32) {
        uint32_t run = 0;
        for (uint32_t w0 = 0; w0 < nw; w0 += 32) {
            const uint32_t w = w0 + threadIdx.x;
            uint32_t       c = 0;
            if (w < nw) {
                // bits of rows 32w .. 32w + 31 (bytes past the page's rows are 0 or masked)
                uint32_t word = 0;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const uint32_t byte = 4 * w + k;
                    if (bm0 + byte < kPage) word |= uint32_t(b[bm0 + byte]) << (8 * k);
                }
                const uint32_t valid = nr - 32 * w >= 32 ? 0xffffffffu : ((1u << (nr - 32 * w)) - 1u);
                c = __popc(word & valid);
            }
            const uint32_t inc = warp_inclusive_scan<uint32_t>(c);
            if (w < nw) s.base[w] = run + inc - c;
            run += __shfl_sync(0xffffffffu, inc, 31);
        }
    }
    __syncthreads();
    return bm0;
}

// Row i of the staged page: its validity and non-NULL rank.
__device__ __forceinline__ bool row_rank(const PageSmem& s, uint32_t bm0, uint32_t i, uint32_t& rank) {
    const uint8_t* b    = reinterpret_cast<const uint8_t*>(s.img);
    const uint32_t w    = i >> 5, l = i & 31;
    uint32_t       word = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t byte = 4 * w + k;
        if (bm0 + byte < kPage) word |= uint32_t(b[bm0 + byte]) << (8 * k);
    }
    rank = s.base[w] + __popc(word & ((1u << l) - 1u));
    return (word >> l) & 1u;
}

// VARCHAR pages: one warp per page (grid-stride over pages), 4 x 32 rows at a
// time -- only the offsets and the bitmap are read, never the string bytes,
// which make up most of such a page.  Each non-NULL row's rank among the
// page's non-NULL rows comes from ballots of the bitmap bits, so no
// block-wide barrier is needed.  The bitmap bytes of the 4
// steps are loaded together, then the 4 values (fetch), then stored, so each
// lane has 4 independent loads in flight instead of one dependent chain.
template <class Fetch, class Store>
__device__ __forceinline__ void warp_rows(const uint8_t* pg, uint32_t nr, Fetch&& fetch, Store&& store) {
    constexpr int  kU        = 4;
    const unsigned lane      = threadIdx.x & 31;
    const unsigned lt        = (1u << lane) - 1;
    const uint8_t* bm        = pg + kPage - (nr + 7) / 8;
    uint32_t       rank_base = 0;
    for (uint32_t c = 0; c < nr; c += 32 * kU) {
        bool on[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const uint32_t i = c + 32 * u + lane;
            on[u]            = i < nr && ((bm[i >> 3] >> (i & 7)) & 1u);
        }
        uint32_t rank[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const unsigned bal = __ballot_sync(0xffffffffu, on[u]);
            rank[u]            = rank_base + __popc(bal & lt);
            rank_base += __popc(bal);
        }
        uint64_t v[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) v[u] = fetch(on[u], rank[u]);
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const uint32_t i = c + 32 * u + lane;
            if (i < nr) store(i, v[u]);
        }
    }
}

__device__ __forceinline__ uint64_t global_warp() {
    return (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
}
__device__ __forceinline__ uint64_t total_warps() { return (uint64_t(gridDim.x) * blockDim.x) >> 5; }

__global__ void __launch_bounds__(kDecThreads)
    k_decode_int32_tagged(const uint8_t* __restrict__ pages, uint64_t num_pages,
                          const uint64_t* __restrict__ row_start, uint64_t* __restrict__ out) {
    __shared__ PageSmem s;
    for (uint64_t p = blockIdx.x; p < num_pages; p += gridDim.x) {
        const uint8_t* pg  = pages + p * kPage;
        const uint32_t nr  = *reinterpret_cast<const uint16_t*>(pg);
        const uint32_t bm0 = stage_page(pg, nr, s);
        const int32_t* data = reinterpret_cast<const int32_t*>(reinterpret_cast<const uint8_t*>(s.img) + 4);
        uint64_t*      o    = out + row_start[p];
        for (uint32_t i = threadIdx.x; i < nr; i += kDecThreads) {
            uint32_t   rank;
            const bool on = row_rank(s, bm0, i, rank);
            // a well-formed page has rank < num_non_null <= 2047; never read past it
            o[i] = (on && rank < (kPage - 4) / 4) ? (uint64_t(uint32_t(data[rank])) | value_t::TAG_INT32) : 0ull;
        }
        __syncthreads();  // the next page overwrites the image
    }
}

__global__ void __launch_bounds__(kDecThreads)
    k_decode_int32_plain(const uint8_t* __restrict__ pages, uint64_t num_pages,
                         const uint64_t* __restrict__ row_start, int32_t* __restrict__ out) {
    for (uint64_t p = global_warp(); p < num_pages; p += total_warps()) {
        const uint8_t* pg   = pages + p * kPage;
        const uint32_t nr   = min(uint32_t(*reinterpret_cast<const uint16_t*>(pg)), uint32_t((kPage - 4) / 4));
        const int32_t* data = reinterpret_cast<const int32_t*>(pg + 4);
        int32_t*       o    = out + row_start[p];
        for (uint32_t i = threadIdx.x & 31; i < nr; i += 32) o[i] = __ldg(data + i);
    }
}

__global__ void __launch_bounds__(kDecThreads, 8)
    k_decode_varchar_loc(const uint8_t* __restrict__ pages, uint64_t num_pages,
                         const uint64_t* __restrict__ row_start, uint64_t* __restrict__ out) {
    for (uint64_t p = global_warp(); p < num_pages; p += total_warps()) {
        const uint8_t* pg = pages + p * kPage;
        const uint32_t nr = *reinterpret_cast<const uint16_t*>(pg);
        if (nr == 0xfffe) continue;
        if (nr == 0xffff) {
            if ((threadIdx.x & 31) == 0) out[row_start[p]] = make_loc(p * kPage, long_len(pages, p, num_pages), true);
            continue;
        }
        const uint32_t  nn    = *reinterpret_cast<const uint16_t*>(pg + 2);
        const uint16_t* offs  = reinterpret_cast<const uint16_t*>(pg + 4);
        const uint64_t  data0 = p * kPage + 4 + 2 * uint64_t(nn);
        uint64_t*       o     = out + row_start[p];
        warp_rows(
            pg, nr,
            [&](bool on, uint32_t rank) {
                uint64_t v = 0;
                if (on && rank < nn && rank < (kPage - 4) / 2) {
                    const uint32_t start = rank == 0 ? 0u : offs[rank - 1];
                    v                    = make_loc(data0 + start, uint32_t(offs[rank]) - start, false);
                }
                return v;
            },
            [&](uint32_t i, uint64_t v) { o[i] = v; });
    }
}

// one block per page
unsigned block_page_grid(uint64_t num_pages) {
    return unsigned(std::max<uint64_t>(1, std::min<uint64_t>(num_pages, uint64_t(num_sms()) * 8)));
}

// one warp per page: kDecThreads / 32 pages per block
unsigned page_grid(uint64_t num_pages) {
    const uint64_t blocks = (num_pages + kDecThreads / 32 - 1) / (kDecThreads / 32);
    return unsigned(std::max<uint64_t>(1, std::min<uint64_t>(blocks, uint64_t(num_sms()) * 8)));
}

}  // namespace

void launch_page_rows(const uint8_t* pages, uint64_t num_pages, int32_t type, uint32_t* rows, cudaStream_t st) {
    if (num_pages == 0) return;
    k_page_rows<<<div_up(num_pages, 256), 256, 0, st>>>(pages, num_pages, type, rows);
    HJ_LAUNCH_CHECK();
}

void launch_decode_int32_tagged(const uint8_t* pages, uint64_t num_pages, const uint64_t* row_start,
                                uint64_t* out, cudaStream_t st) {
    if (num_pages == 0) return;
    k_decode_int32_tagged<<<block_page_grid(num_pages), kDecThreads, 0, st>>>(pages, num_pages, row_start, out);
    HJ_LAUNCH_CHECK();
}

void launch_decode_int32_plain(const uint8_t* pages, uint64_t num_pages, const uint64_t* row_start,
                               int32_t* out, cudaStream_t st) {
    if (num_pages == 0) return;
    k_decode_int32_plain<<<page_grid(num_pages), kDecThreads, 0, st>>>(pages, num_pages, row_start, out);
    HJ_LAUNCH_CHECK();
}

void launch_decode_varchar_loc(const uint8_t* pages, uint64_t num_pages, const uint64_t* row_start,
                               uint64_t* out, cudaStream_t st) {
    if (num_pages == 0) return;
    k_decode_varchar_loc<<<page_grid(num_pages), kDecThreads, 0, st>>>(pages, num_pages, row_start, out);
    HJ_LAUNCH_CHECK();
}

}  // namespace hj
