// Allocation-free probe entry point (hj_table_probe_noalloc).
//
// Some callers cannot allocate device memory while they call us: engines that
// hand all device memory to their own sub-allocator under a fixed budget,
// embedders whose CUDA memory pool must not grow after start-up, and latency-
// critical paths where an allocation's cost or failure is not acceptable.
// hj_table_probe allocates its hit lists and prefix-sum temporaries per call;
// this variant takes them from one file-scope device array instead, so the
// call itself allocates nothing.
//
// The array below is part of the library image: every GPU that loads the
// library holds it (HJ_NOALLOC_SCRATCH_BYTES) until the process exits.  In
// host code its name is only a host-side stand-in, so its device address is
// looked up once per device (with that device current) through
// cudaGetSymbolAddress and passed to the kernels.  That lookup happens in the
// first call on each device, so that first call should come before any
// stream capture.  The address belongs to the device's primary context (the
// runtime's); it is kept until the process exits, so neither a non-primary
// driver-API context nor a call after cudaDeviceReset is supported.  All
// calls share the array and it keeps the last call's
// contents; the counters that must start at zero are cleared on every call.
// Two calls whose GPU work overlaps (different streams, or different contexts
// on one device) race on the array and must be serialised by the caller.
#include <mutex>

#include "hj_common.cuh"
#include "hj_kernels.h"

namespace hj {
namespace {

constexpr uint64_t kNoAllocMaxProbeRows = HJ_NOALLOC_MAX_PROBE_ROWS;
constexpr size_t   kNoAllocScratchBytes = HJ_NOALLOC_SCRATCH_BYTES;

static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex    g_mu;
uint8_t*      g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on `device` (current), looked up once.
uint8_t* scratch_on(int device) {
    if (device < 0 || device >= kMaxDevices) throw Error(HJ_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_scratch_addr[device]) {
        void*             p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr)
            throw Error(HJ_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ")
                                         + cudaGetErrorString(e));
        g_scratch_addr[device] = static_cast<uint8_t*>(p);
    }
    return g_scratch_addr[device];
}

}  // namespace
}  // namespace hj

static_assert(HJ_NOALLOC_SCRATCH_BYTES >= 88ull * HJ_NOALLOC_MAX_PROBE_ROWS + 16384,
              "scratch array too small for the probe row limit");

extern "C" int hj_table_probe_noalloc(hj_context* c, const hj_hash_table* t, const int32_t* keys,
                                      const uint32_t* valid, uint64_t n, uint32_t* out_probe_rows,
                                      uint32_t* out_build_rows, uint64_t capacity,
                                      uint64_t* num_matches) {
    if (!c || !t || !num_matches || (n > 0 && !keys)) return HJ_ERR_INVALID;
    *num_matches = 0;
    try {
        if (n > hj::kNoAllocMaxProbeRows) {
            const std::string m = "hj_table_probe_noalloc: " + std::to_string(n) + " probe rows exceed the limit of "
                                + std::to_string(hj::kNoAllocMaxProbeRows) + " (use hj_table_probe)";
            hj::context_set_error(c, m.c_str());
            return HJ_ERR_INVALID;
        }
        const int dev = hj::context_device(c);
        HJ_CUDA(cudaSetDevice(dev));
        uint8_t*           scratch = hj::scratch_on(dev);
        const cudaStream_t st      = hj::context_stream(c);
        hj::IntCol col;
        col.plain = keys;
        col.valid = valid;
        const hj::KeyCol pk{col, nullptr, n};
        if (hj::probe_scratch_bytes(n) > hj::kNoAllocScratchBytes)
            throw hj::Error(HJ_ERR_INVALID, "probe scratch exceeds the static array");
        const int rc = hj::probe_into_scratch(hj::hash_table_of(t), pk, hj::context_probe_params(c), scratch,
                                              hj::kNoAllocScratchBytes, out_probe_rows, out_build_rows,
                                              capacity, num_matches, st);
        HJ_CUDA(cudaStreamSynchronize(st));
        if (rc == HJ_ERR_CAPACITY) hj::context_set_error(c, "output capacity too small");
        return rc;
    } catch (const hj::Error& e) {
        hj::context_set_error(c, e.what());
        return e.status;
    } catch (const std::exception& e) {
        hj::context_set_error(c, e.what());
        return HJ_ERR_INVALID;
    }
}
