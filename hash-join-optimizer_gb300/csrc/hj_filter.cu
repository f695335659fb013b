// Scan predicates: order-preserving compaction of the base rows that pass a
// scan's filters into a row-id vector (hj_filter, include/hj_api.h).
//
// The reference applies a scan's Comparison while loading the table and
// hands execute() only the passing rows, in order (src/build_table.cpp:
// 321-370).  Here the passing rows become the scan's row ids.  (With option
// fuse_filters a filtered probe side skips this and k_probe_count, in
// hj_probe.cu, evaluates the predicate on the raw rows instead.)
//
// Two passes over 4096-row tiles (8 warps x 16 steps x 32 rows):
//  * k_filter_mask evaluates the filters and writes one pass bit per row (the
//    32-row ballots) and a count per tile.  A warp issues the loads of its 16
//    rows per lane before it compares any of them, so 16 loads per thread are
//    in flight; the column is read once.
//  * after an exclusive scan of the tile counts, k_filter_emit reads only the
//    bit words and writes each passing row's id at its rank, so the ids come
//    out in base-row order.
#include <algorithm>

#include "hj_block.cuh"
#include "hj_common.cuh"
#include "hj_kernels.h"

namespace hj {
namespace {

constexpr int kFT        = 256;                 // threads: 8 warps
constexpr int kFStep     = 16;                  // 32-row steps per warp
constexpr int kFTile     = kFT * kFStep;        // rows per tile
constexpr int kFWords    = kFTile / 32;         // bit words per tile
constexpr int kWarpWords = kFStep;              // bit words per warp

// Values and validity of column c at rows r0 + 32 k (k < lim <= S); the
// loads are issued together.  Steps at or past lim read as NULL.  The S rows
// span fewer than kDenseRows rows, so a dense column's rows lie on at most
// two pages.
template <int S>
__device__ __forceinline__ uint32_t load_steps(const IntCol& c, uint64_t r0, uint32_t lim, int32_t (&v)[S]) {
    static_assert(32 * S <= kDenseRows && S < 32, "steps span at most two pages");
    uint32_t valid = 0;
    if (c.tagged) {
        const uint64_t* t = c.tagged + r0;
#pragma unroll
        for (int k = 0; k < S; ++k) {
            const uint64_t x = uint32_t(k) < lim ? __ldg(t + 32 * k) : 0;
            v[k]             = int32_t(uint32_t(x));
            valid |= uint32_t((x >> 62) == 1) << k;
        }
    } else if (c.plain) {
        const int32_t* q = c.plain + r0;
#pragma unroll
        for (int k = 0; k < S; ++k) v[k] = uint32_t(k) < lim ? __ldg(q + 32 * k) : 0;
        valid = (1u << lim) - 1u;
        if (c.valid) {  // the bits of rows r0 + 32 k: bit (r0 & 31) of consecutive words
            const uint32_t* b = c.valid + (r0 >> 5);
            uint32_t        m = 0;
#pragma unroll
            for (int k = 0; k < S; ++k) m |= (uint32_t(k) < lim ? (__ldg(b + k) >> (r0 & 31)) & 1u : 0u) << k;
            valid &= m;
        }
    } else {  // dense pages read in place; steps from kb on lie on the next page
        const uint64_t p0   = r0 / uint64_t(kDenseRows);
        const uint32_t rem0 = uint32_t(r0 - p0 * uint64_t(kDenseRows));
        const uint32_t kb   = (uint32_t(kDenseRows) - rem0 + 31) / 32;
        const int32_t* q0   = reinterpret_cast<const int32_t*>(c.pages + p0 * kPage + 4) + rem0;
        const int32_t* q1   = q0 + (kPage / 4 - kDenseRows);  // same step index on the next page
#pragma unroll
        for (int k = 0; k < S; ++k) {
            v[k] = 0;
            if (uint32_t(k) < lim && uint32_t(k) < kb) v[k] = __ldg(q0 + 32 * k);
        }
#pragma unroll
        for (int k = 0; k < S; ++k)
            if (uint32_t(k) < lim && uint32_t(k) >= kb) v[k] = __ldg(q1 + 32 * k);
        valid = (1u << lim) - 1u;
    }
    return valid;
}

__global__ void __launch_bounds__(kFT, 4)
    k_filter_mask(Filters F, uint64_t n, uint64_t nwords, uint64_t ntiles, uint32_t* __restrict__ words,
                  uint32_t* __restrict__ cnt) {
    __shared__ uint32_t wt[kFT / 32];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t r0   = tile * kFTile + uint64_t(warp) * (kFStep * 32) + lane;
        // steps of this lane with a row below n
        const uint32_t lim  = r0 >= n ? 0u : uint32_t((n - r0 + 31) / 32 < kFStep ? (n - r0 + 31) / 32 : kFStep);
        uint32_t       keep = (1u << lim) - 1u;
        for (int i = 0; i < F.n; ++i) {
            int32_t        v[kFStep];
            const uint32_t valid = load_steps<kFStep>(F.f[i].col, r0, lim, v);
            const uint32_t tt = cmp_table(F.f[i].op);
            const int32_t  x  = F.f[i].val;
            uint32_t       ok = 0;
#pragma unroll
            for (int k = 0; k < kFStep; ++k) ok |= ((tt >> cmp_state((valid >> k) & 1u, v[k], x)) & 1u) << k;
            keep &= ok;
        }
        uint32_t mine = 0, wc = 0;
#pragma unroll
        for (int k = 0; k < kFStep; ++k) {
            const uint32_t m = __ballot_sync(0xffffffffu, (keep >> k) & 1u);
            if (lane == unsigned(k)) mine = m;
            wc += __popc(m);
        }
        const uint64_t w = tile * kFWords + uint64_t(warp) * kWarpWords + lane;
        if (lane < unsigned(kWarpWords) && w < nwords) words[w] = mine;
        if (lane == 0) wt[warp] = wc;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (int q = 0; q < kFT / 32; ++q) t += wt[q];
            cnt[tile] = t;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kFT)
    k_filter_emit(const uint32_t* __restrict__ words, uint64_t nwords, uint64_t ntiles,
                  const uint64_t* __restrict__ off, uint32_t* __restrict__ rid) {
    __shared__ uint32_t wt[kFT / 32];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t w0   = tile * kFWords + uint64_t(warp) * kWarpWords;
        const uint32_t word = (lane < unsigned(kWarpWords) && w0 + lane < nwords) ? __ldg(words + w0 + lane) : 0u;
        const uint32_t c    = __popc(word);
        uint32_t       inc  = c;  // inclusive scan over the warp's words
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, d);
            if (lane >= unsigned(d)) inc += y;
        }
        if (lane == 31) wt[warp] = inc;
        __syncthreads();
        uint64_t pos = off[tile];
        for (unsigned q = 0; q < warp; ++q) pos += wt[q];
        const uint32_t excl = inc - c;
#pragma unroll
        for (int k = 0; k < kWarpWords; ++k) {
            const uint32_t wk = __shfl_sync(0xffffffffu, word, k);
            const uint32_t pk = __shfl_sync(0xffffffffu, excl, k);
            if ((wk >> lane) & 1u)
                rid[pos + pk + __popc(wk & ((1u << lane) - 1))] = uint32_t((w0 + k) * 32 + lane);
        }
        __syncthreads();
    }
}

}  // namespace

uint64_t filter_compact(const Filters& f, uint64_t n, uint32_t* rid_out, uint64_t* pinned, cudaStream_t st) {
    if (n == 0) return 0;
    if (n > 0xffffffffull) throw Error(HJ_ERR_INVALID, "a filtered scan has more than 2^32 rows");
    const uint64_t ntiles = (n + kFTile - 1) / kFTile;
    const uint64_t nwords = (n + 31) / 32;
    const unsigned grid   = unsigned(std::min<uint64_t>(ntiles, uint64_t(num_sms()) * 8));
    uint32_t*      words  = dalloc_n<uint32_t>(nwords, st);
    uint32_t*      cnt    = dalloc_n<uint32_t>(ntiles, st);
    uint64_t*      off    = dalloc_n<uint64_t>(ntiles + 1, st);
    k_filter_mask<<<grid, kFT, 0, st>>>(f, n, nwords, ntiles, words, cnt);
    HJ_LAUNCH_CHECK();
    scan_exclusive_u32_to_u64(cnt, off, ntiles, st);
    k_filter_emit<<<grid, kFT, 0, st>>>(words, nwords, ntiles, off, rid_out);
    HJ_LAUNCH_CHECK();
    readback(pinned, off + ntiles, sizeof(uint64_t), true, st);  // page-locked scratch
    HJ_CUDA(cudaStreamSynchronize(st));
    const uint64_t kept = pinned[0];
    dfree(words, st);
    dfree(cnt, st);
    dfree(off, st);
    return kept;
}

}  // namespace hj
