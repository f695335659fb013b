// Scan predicates: order-preserving compaction of the base rows that pass a
// scan's filters into a row-id vector (hj_filter, include/hj_api.h).
//
// The reference applies a scan's Comparison while loading the table and
// hands execute() only the passing rows, in order (src/build_table.cpp:
// 321-370).  A filtered scan on the probe side of a join needs no compaction
// at all: k_probe_count evaluates the predicate on the raw rows (hj_probe.cu).
// Everywhere else the passing rows become the scan's row ids here.
//
// Two passes over 2048-row tiles (8 warps x 8 steps x 32 rows): count per
// tile, exclusive scan, then each warp writes its passing rows at ballot
// ranks, so the ids come out in base-row order.
#include <algorithm>

#include "hj_block.cuh"
#include "hj_common.cuh"
#include "hj_kernels.h"

namespace hj {
namespace {

constexpr int kFT    = 256;           // threads: 8 warps
constexpr int kFStep = 8;             // 32-row steps per warp
constexpr int kFTile = kFT * kFStep;  // rows per tile

template <bool WRITE>
__global__ void __launch_bounds__(kFT)
    k_filter_pass(Filters F, uint64_t n, uint64_t ntiles, uint32_t* __restrict__ cnt,
                  const uint64_t* __restrict__ off, uint32_t* __restrict__ rid) {
    __shared__ uint32_t wt[kFT / 32];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t base = tile * kFTile;
        unsigned       m[kFStep];
        uint32_t       wc = 0;
#pragma unroll
        for (int k = 0; k < kFStep; ++k) {
            const uint64_t r    = base + (uint64_t(warp) * kFStep + k) * 32 + lane;
            const bool     pass = r < n && filt_pass(F, r);
            m[k]                = __ballot_sync(0xffffffffu, pass);
            wc += __popc(m[k]);
        }
        if (lane == 0) wt[warp] = wc;
        __syncthreads();
        if (!WRITE) {
            if (threadIdx.x == 0) {
                uint32_t t = 0;
                for (int w = 0; w < kFT / 32; ++w) t += wt[w];
                cnt[tile] = t;
            }
        } else {
            uint64_t pos = off[tile];
            for (unsigned w = 0; w < warp; ++w) pos += wt[w];
#pragma unroll
            for (int k = 0; k < kFStep; ++k) {
                if ((m[k] >> lane) & 1u)
                    rid[pos + __popc(m[k] & ((1u << lane) - 1))] =
                        uint32_t(base + (uint64_t(warp) * kFStep + k) * 32 + lane);
                pos += __popc(m[k]);
            }
        }
        __syncthreads();
    }
}

}  // namespace

uint64_t filter_compact(const Filters& f, uint64_t n, uint32_t* rid_out, uint64_t* pinned, cudaStream_t st) {
    if (n == 0) return 0;
    if (n > 0xffffffffull) throw Error(HJ_ERR_INVALID, "a filtered scan has more than 2^32 rows");
    const uint64_t ntiles = (n + kFTile - 1) / kFTile;
    const unsigned grid   = unsigned(std::min<uint64_t>(ntiles, uint64_t(kSMs) * 8));
    uint32_t*      cnt    = dalloc_n<uint32_t>(ntiles, st);
    uint64_t*      off    = dalloc_n<uint64_t>(ntiles + 1, st);
    k_filter_pass<false><<<grid, kFT, 0, st>>>(f, n, ntiles, cnt, nullptr, nullptr);
    HJ_LAUNCH_CHECK();
    scan_exclusive_u32_to_u64(cnt, off, ntiles, st);
    k_filter_pass<true><<<grid, kFT, 0, st>>>(f, n, ntiles, nullptr, off, rid_out);
    HJ_LAUNCH_CHECK();
    HJ_CUDA(cudaMemcpyAsync(pinned, off + ntiles, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    HJ_CUDA(cudaStreamSynchronize(st));
    const uint64_t kept = pinned[0];
    dfree(cnt, st);
    dfree(off, st);
    return kept;
}

}  // namespace hj
