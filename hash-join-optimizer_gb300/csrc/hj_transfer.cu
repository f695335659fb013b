// Host <-> HBM page transfers by the GPU itself, for systems whose GPU reads
// and writes pageable host memory through the CPU's page tables (address
// translation services, as on Grace-Blackwell: cudaDevAttrPageableMemoryAccess).
// The input pages of a ColumnarTable are separate host allocations; instead of
// gathering them into pinned staging memory with host threads, one kernel
// reads each page through its pointer over the chip-to-chip link and writes it
// to a contiguous HBM buffer, noting the page header on the way; result pages
// go back the same way, straight into the caller's pages.
#include <algorithm>

#include "hj_common.cuh"
#include "hj_kernels.h"

namespace hj {
namespace {

constexpr int kTT = 256;

__device__ __forceinline__ void copy_page(uint8_t* dst, const uint8_t* src) {
    const unsigned lane = threadIdx.x & 31;
    if ((reinterpret_cast<uintptr_t>(src) & 15) == 0 && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
        const uint4* s = reinterpret_cast<const uint4*>(src);
        uint4*       d = reinterpret_cast<uint4*>(dst);
#pragma unroll 4
        for (uint32_t k = lane; k < kPage / 16; k += 32) d[k] = s[k];
    } else {  // pages are only guaranteed 8-byte aligned (alignas(8) Page)
        const uint2* s = reinterpret_cast<const uint2*>(src);
        uint2*       d = reinterpret_cast<uint2*>(dst);
#pragma unroll 4
        for (uint32_t k = lane; k < kPage / 8; k += 32) d[k] = s[k];
    }
}

// One warp per page: host page -> HBM; header fields into nr / nn.
__global__ void __launch_bounds__(kTT)
    k_gather_host_pages(const uint8_t* const* __restrict__ src, uint64_t n, uint8_t* __restrict__ dst,
                        uint16_t* __restrict__ nr, uint16_t* __restrict__ nn) {
    const uint64_t gw = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = (uint64_t(gridDim.x) * blockDim.x) >> 5;
    for (uint64_t p = gw; p < n; p += nw) {
        const uint8_t* s = src[p];
        copy_page(dst + p * kPage, s);
        if ((threadIdx.x & 31) == 0) {
            const uint32_t h = *reinterpret_cast<const uint32_t*>(s);
            nr[p]            = uint16_t(h);
            nn[p]            = uint16_t(h >> 16);
        }
    }
}

// One warp per page: HBM -> host page dst[p] (or dst_contig + p * 8192).
__global__ void __launch_bounds__(kTT)
    k_scatter_host_pages(const uint8_t* __restrict__ src, uint64_t n, uint8_t* const* __restrict__ dst,
                         uint8_t* __restrict__ dst_contig) {
    const uint64_t gw = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = (uint64_t(gridDim.x) * blockDim.x) >> 5;
    for (uint64_t p = gw; p < n; p += nw) copy_page(dst ? dst[p] : dst_contig + p * kPage, src + p * kPage);
}

unsigned warp_grid(uint64_t pages) {
    const uint64_t blocks = (pages + kTT / 32 - 1) / (kTT / 32);
    return unsigned(std::max<uint64_t>(1, std::min<uint64_t>(blocks, uint64_t(kSMs) * 16)));
}

}  // namespace

void launch_gather_host_pages(const void* const* host_pages, uint64_t n, uint8_t* dst, uint16_t* nr, uint16_t* nn,
                              cudaStream_t st) {
    if (n == 0) return;
    k_gather_host_pages<<<warp_grid(n), kTT, 0, st>>>(reinterpret_cast<const uint8_t* const*>(host_pages), n, dst,
                                                      nr, nn);
    HJ_LAUNCH_CHECK();
}

void launch_scatter_host_pages(const uint8_t* src, uint64_t n, void* const* host_pages, void* host_contig,
                               cudaStream_t st) {
    if (n == 0) return;
    k_scatter_host_pages<<<warp_grid(n), kTT, 0, st>>>(src, n, reinterpret_cast<uint8_t* const*>(host_pages),
                                                       static_cast<uint8_t*>(host_contig));
    HJ_LAUNCH_CHECK();
}

}  // namespace hj
