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
constexpr int      kSMs        = 152;         // GB300: 2 dies x 76 SMs

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

__device__ __forceinline__ bool bit_valid(const uint32_t* bm, uint64_t i) {
    return bm == nullptr || ((__ldg(bm + (i >> 5)) >> (i & 31)) & 1u);
}

__device__ __forceinline__ uint16_t ld16(const uint8_t* p) {
    return uint16_t(p[0]) | uint16_t(uint16_t(p[1]) << 8);
}

inline unsigned div_up(uint64_t a, uint64_t b) { return unsigned((a + b - 1) / b); }

}  // namespace hj
