// Warp- and block-level building blocks (scans, aggregated atomics).
#pragma once

#include <cstdint>

namespace hj {

template <class T>
__device__ __forceinline__ T warp_inclusive_scan(T v) {
    const unsigned lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T n = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= unsigned(d)) v += n;
    }
    return v;
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    return v;
}

// Block-wide exclusive scan; `smem` holds >= 33 T.  Returns the exclusive
// prefix of the calling thread and writes the block total to *total.
// Every thread of the block must call it.
template <class T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* smem, T* total) {
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned nwarps = (blockDim.x + 31) >> 5;
    T inc = warp_inclusive_scan(v);
    if (lane == 31) smem[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        T w  = lane < nwarps ? smem[lane] : T(0);
        T wi = warp_inclusive_scan(w);
        if (lane < nwarps) smem[lane] = wi - w;
        if (lane == nwarps - 1) smem[32] = wi;
    }
    __syncthreads();
    T r = smem[warp] + inc - v;
    if (total) *total = smem[32];
    __syncthreads();
    return r;
}

// Adds `v` to smem counter addr[slot] once per distinct slot in the warp
// (lanes in `active`), returning the old value plus this lane's rank among
// the lanes with the same slot.  Used where Zipf-skewed keys make many lanes
// of a warp hit the same counter.
__device__ __forceinline__ uint32_t warp_agg_atomic_add(uint32_t* addr, uint32_t slot,
                                                         unsigned active) {
    const unsigned peers = __match_any_sync(active, slot);
    const unsigned lane  = threadIdx.x & 31;
    const int      leader = __ffs(peers) - 1;
    const uint32_t rank  = __popc(peers & ((1u << lane) - 1));
    uint32_t       base  = 0;
    if (int(lane) == leader) base = atomicAdd(addr + slot, uint32_t(__popc(peers)));
    base = __shfl_sync(peers, base, leader);
    return base + rank;
}

// OR `bits` into smem word addr[slot], once per distinct slot of the warp.
__device__ __forceinline__ void warp_agg_atomic_or(uint32_t* addr, uint32_t slot, uint32_t bits,
                                                   unsigned active) {
    const unsigned peers  = __match_any_sync(active, slot);
    const unsigned lane   = threadIdx.x & 31;
    const int      leader = __ffs(peers) - 1;
    const uint32_t acc    = __reduce_or_sync(peers, bits);
    if (int(lane) == leader) atomicOr(addr + slot, acc);
}

}  // namespace hj
