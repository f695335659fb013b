// Host <-> HBM page transfers by the GPU itself, for systems whose GPU reads
// and writes pageable host memory through the CPU's page tables (address
// translation services, as on Grace-Blackwell: cudaDevAttrPageableMemoryAccess).
// The input pages of a ColumnarTable are separate host allocations; instead of
// gathering them into pinned staging memory with host threads, one kernel
// reads each page through its pointer over the chip-to-chip link and writes it
// to a contiguous HBM buffer, noting the page header on the way; result pages
// go back the same way, straight into the caller's pages.
//
// Page-locked host memory (cudaHostRegister / cudaHostAlloc, hj_host_register)
// goes through the copy engines instead: one cudaMemcpyAsync per run of
// consecutive pages, which leaves the SMs to the kernels of other plans and
// lets uploads and result downloads of different plans overlap in both
// directions of the link.
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

// Header fields of n device pages (after a copy-engine upload).
__global__ void k_page_headers(const uint8_t* __restrict__ pages, uint64_t n, uint16_t* __restrict__ nr,
                               uint16_t* __restrict__ nn) {
    for (uint64_t p = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < n; p += uint64_t(gridDim.x) * blockDim.x) {
        const uint32_t h = *reinterpret_cast<const uint32_t*>(pages + p * kPage);
        nr[p]            = uint16_t(h);
        nn[p]            = uint16_t(h >> 16);
    }
}

// Device -> host bytes by the SMs (host memory the GPU can write).
__global__ void k_readback(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, uint64_t n) {
    const uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x, T = uint64_t(gridDim.x) * blockDim.x;
    if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 3) == 0) {
        const uint64_t w = n / 4;
        for (uint64_t i = t; i < w; i += T)
            reinterpret_cast<uint32_t*>(dst)[i] = reinterpret_cast<const uint32_t*>(src)[i];
        for (uint64_t i = 4 * w + t; i < n; i += T) dst[i] = src[i];
    } else {
        for (uint64_t i = t; i < n; i += T) dst[i] = src[i];
    }
}

bool page_locked(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();  // not a CUDA-known pointer: pageable
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

unsigned warp_grid(uint64_t pages) {
    const uint64_t blocks = (pages + kTT / 32 - 1) / (kTT / 32);
    return unsigned(std::max<uint64_t>(1, std::min<uint64_t>(blocks, uint64_t(num_sms()) * 16)));
}

}  // namespace

std::vector<PageRun> locked_runs(const void* const* pages, uint64_t n, size_t max_runs) {
    std::vector<PageRun> runs;
    for (uint64_t i = 0; i < n;) {
        const uint8_t* a = static_cast<const uint8_t*>(pages[i]);
        uint64_t       j = i + 1;
        while (j < n && static_cast<const uint8_t*>(pages[j]) == a + (j - i) * kPage) ++j;
        if (runs.size() == max_runs || !page_locked(a) || !page_locked(a + (j - i) * kPage - 1)) return {};
        runs.push_back(PageRun{i, j - i});
        i = j;
    }
    return runs;
}

bool locked_range(const void* p, uint64_t bytes) {
    return bytes > 0 && page_locked(p) && page_locked(static_cast<const uint8_t*>(p) + bytes - 1);
}

void readback(void* host, const void* dev, uint64_t bytes, bool kernel, cudaStream_t st) {
    if (bytes == 0) return;
    if (!kernel) {
        HJ_CUDA(cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, st));
        return;
    }
    const unsigned grid = unsigned(std::max<uint64_t>(1, std::min<uint64_t>((bytes / 4 + kTT - 1) / kTT, uint64_t(num_sms()))));
    k_readback<<<grid, kTT, 0, st>>>(static_cast<const uint8_t*>(dev), static_cast<uint8_t*>(host), bytes);
    HJ_LAUNCH_CHECK();
}

void launch_page_headers(const uint8_t* pages, uint64_t n, uint16_t* nr, uint16_t* nn, cudaStream_t st) {
    if (n == 0) return;
    const unsigned grid = unsigned(std::max<uint64_t>(1, std::min<uint64_t>((n + kTT - 1) / kTT, uint64_t(num_sms()) * 4)));
    k_page_headers<<<grid, kTT, 0, st>>>(pages, n, nr, nn);
    HJ_LAUNCH_CHECK();
}

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
