// Device-wide exclusive prefix sums (reduce-then-scan, 4096 items per block).
#include "hj_block.cuh"
#include "hj_common.cuh"
#include "hj_kernels.h"

namespace hj {
namespace {

constexpr int kScanThreads = 512;
constexpr int kScanItems   = 8;
constexpr int kScanTile    = kScanThreads * kScanItems;

template <class Tin>
__global__ void __launch_bounds__(kScanThreads) k_block_sums(const Tin* __restrict__ in, uint64_t n,
                                                             uint64_t* __restrict__ sums) {
    __shared__ uint64_t sm[33];
    const uint64_t base = uint64_t(blockIdx.x) * kScanTile + uint64_t(threadIdx.x) * kScanItems;
    uint64_t       s    = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
        if (base + i < n) s += uint64_t(in[base + i]);
    uint64_t total;
    block_exclusive_scan<uint64_t>(s, sm, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

template <class Tin>
__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const Tin* __restrict__ in,
                                                             uint64_t* __restrict__ out, uint64_t n,
                                                             const uint64_t* __restrict__ block_off) {
    __shared__ uint64_t sm[33];
    const uint64_t base = uint64_t(blockIdx.x) * kScanTile + uint64_t(threadIdx.x) * kScanItems;
    uint64_t       v[kScanItems];
    uint64_t       s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = base + i < n ? uint64_t(in[base + i]) : 0;
        s += v[i];
    }
    uint64_t total;
    uint64_t run = block_exclusive_scan<uint64_t>(s, sm, &total);
    run += block_off ? block_off[blockIdx.x] : 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n) out[base + i] = run;
        run += v[i];
    }
    if (threadIdx.x == 0 && blockIdx.x == gridDim.x - 1)
        out[n] = (block_off ? block_off[blockIdx.x] : 0) + total;
}

template <class Tin>
void scan_impl(const Tin* in, uint64_t* out, uint64_t n, cudaStream_t st) {
    if (n == 0) {
        HJ_CUDA(cudaMemsetAsync(out, 0, sizeof(uint64_t), st));
        return;
    }
    const uint64_t blocks = (n + kScanTile - 1) / kScanTile;
    if (blocks == 1) {
        k_scan_apply<Tin><<<1, kScanThreads, 0, st>>>(in, out, n, nullptr);
        HJ_LAUNCH_CHECK();
        return;
    }
    uint64_t* sums = dalloc_n<uint64_t>(blocks, st);
    uint64_t* offs = dalloc_n<uint64_t>(blocks + 1, st);
    k_block_sums<Tin><<<unsigned(blocks), kScanThreads, 0, st>>>(in, n, sums);
    HJ_LAUNCH_CHECK();
    scan_impl<uint64_t>(sums, offs, blocks, st);
    k_scan_apply<Tin><<<unsigned(blocks), kScanThreads, 0, st>>>(in, out, n, offs);
    HJ_LAUNCH_CHECK();
    dfree(sums, st);
    dfree(offs, st);
}

}  // namespace

void scan_exclusive_u32_to_u64(const uint32_t* in, uint64_t* out, uint64_t n, cudaStream_t st) {
    scan_impl<uint32_t>(in, out, n, st);
}

void scan_exclusive_u64(const uint64_t* in, uint64_t* out, uint64_t n, cudaStream_t st) {
    scan_impl<uint64_t>(in, out, n, st);
}

size_t scan_tmp_words(uint64_t n) {
    const uint64_t blocks = (n + kScanTile - 1) / kScanTile;
    return blocks <= 1 ? 0 : size_t(2 * blocks + 1) + scan_tmp_words(blocks);
}

namespace {

template <class Tin>
void scan_into_impl(const Tin* in, uint64_t* out, uint64_t n, uint64_t* tmp, cudaStream_t st) {
    if (n == 0) {
        HJ_CUDA(cudaMemsetAsync(out, 0, sizeof(uint64_t), st));
        return;
    }
    const uint64_t blocks = (n + kScanTile - 1) / kScanTile;
    if (blocks == 1) {
        k_scan_apply<Tin><<<1, kScanThreads, 0, st>>>(in, out, n, nullptr);
        HJ_LAUNCH_CHECK();
        return;
    }
    if (blocks > 0x7fffffffull) throw Error(HJ_ERR_INVALID, "scan too large");
    uint64_t* sums = tmp;
    uint64_t* offs = tmp + blocks;
    k_block_sums<Tin><<<unsigned(blocks), kScanThreads, 0, st>>>(in, n, sums);
    HJ_LAUNCH_CHECK();
    scan_into_impl<uint64_t>(sums, offs, blocks, tmp + 2 * blocks + 1, st);
    k_scan_apply<Tin><<<unsigned(blocks), kScanThreads, 0, st>>>(in, out, n, offs);
    HJ_LAUNCH_CHECK();
}

}  // namespace

void scan_exclusive_u32_to_u64_into(const uint32_t* in, uint64_t* out, uint64_t n, uint64_t* tmp,
                                    cudaStream_t st) {
    scan_into_impl<uint32_t>(in, out, n, tmp, st);
}

}  // namespace hj
