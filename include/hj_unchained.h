/* UnchainedHash-shaped C++ adapter over the GPU hash table of libhjgb300.so.
 *
 * Code written against the reference's HASH_ALGO=unchained table
 * (include/unchained.h:14-247 of eleanalt/hash-join-optimizer, selected by
 * CMakeLists.txt:173-187) calls clear / reserve / build_insert /
 * finalize_build / probe(key, cb).  This class keeps those names, argument
 * meanings and the callback form for INT32 keys, and runs the table on the
 * GPU:
 *   build_insert   appends (key, payload) on the host, as the reference
 *                  appends tuples (unchained.h:155-161);
 *   finalize_build uploads the keys and builds the table with
 *                  hj_table_build (directory of next_pow2(#tuples) words, the
 *                  reference's directory words for the same keys);
 *   probe(key, cb) calls cb(payload) for every inserted tuple with an equal
 *                  key, as unchained.h:220-246 does; one probe is one GPU
 *                  round trip, so code that probes many keys should call
 *                  probe_batch, which probes them in one call and reports
 *                  matches as cb(index of the probe key, payload).
 * Matches of one key come in the table's bucket order, not necessarily in
 * insertion order (the reference promises no order either).
 * Errors throw std::runtime_error carrying hj_last_error's message.
 *
 * Needs the CUDA runtime (cuda_runtime.h, -lcudart) and libhjgb300.so. */
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "hj_api.h"

namespace hjgb300 {

template <typename Key, typename Payload>
class UnchainedHash {
    static_assert(sizeof(Key) == 4 && Key(-1) < Key(0), "the GPU table takes INT32 keys");

public:
    /* ctx: the engine context whose device and stream the table uses; it must
     * outlive the table. */
    explicit UnchainedHash(hj_context* ctx) : ctx_(ctx) {
        if (!ctx_) throw std::runtime_error("UnchainedHash: null hj_context");
        stream_ = static_cast<cudaStream_t>(hj_context_stream(ctx_));
    }
    ~UnchainedHash() { clear(); }
    UnchainedHash(const UnchainedHash&)            = delete;
    UnchainedHash& operator=(const UnchainedHash&) = delete;

    void clear() {
        if (table_) hj_table_free(table_);
        table_ = nullptr;
        keys_.clear();
        payloads_.clear();
        release_probe_buffers();
        if (d_keys_) cudaFree(d_keys_);
        d_keys_ = nullptr;
    }
    void reserve(uint32_t expected_build_size) {
        keys_.reserve(expected_build_size);
        payloads_.reserve(expected_build_size);
    }
    void build_insert(const Key& key, const Payload& payload) {
        if (table_) throw std::runtime_error("UnchainedHash: build_insert after finalize_build");
        keys_.push_back(int32_t(key));
        payloads_.push_back(payload);
    }
    void finalize_build() {
        if (table_) throw std::runtime_error("UnchainedHash: finalize_build called twice");
        if (keys_.empty()) return;  // no tuples: every probe misses, as in the reference
        check(cudaMalloc(reinterpret_cast<void**>(&d_keys_), keys_.size() * sizeof(int32_t)), "cudaMalloc");
        copy(d_keys_, keys_.data(), keys_.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
        check_rc(hj_table_build(ctx_, d_keys_, nullptr, keys_.size(), -1, &table_));
    }
    template <typename Callback>
    void probe(const Key& key, Callback&& cb) const {
        probe_batch(&key, 1, [&](size_t, const Payload& p) { cb(p); });
    }
    /* Probes n host keys in one GPU call; cb(i, payload) per match of keys[i]. */
    template <typename Callback>
    void probe_batch(const Key* keys, size_t n, Callback&& cb) const {
        if (!table_ || n == 0) return;
        reserve_probe(n, probe_cap_ ? probe_cap_ : n);
        copy(d_pkeys_, keys, n * sizeof(int32_t), cudaMemcpyHostToDevice);
        uint64_t   found = 0;
        int        rc    = hj_table_probe(ctx_, table_, d_pkeys_, nullptr, n, d_prow_, d_brow_, probe_cap_, &found);
        if (rc == HJ_ERR_CAPACITY) {  // grow the match buffers to the exact count and probe again
            reserve_probe(n, found);
            rc = hj_table_probe(ctx_, table_, d_pkeys_, nullptr, n, d_prow_, d_brow_, probe_cap_, &found);
        }
        check_rc(rc);
        std::vector<uint32_t> prow(found), brow(found);
        if (found) {
            copy(prow.data(), d_prow_, found * sizeof(uint32_t), cudaMemcpyDeviceToHost);
            copy(brow.data(), d_brow_, found * sizeof(uint32_t), cudaMemcpyDeviceToHost);
        }
        for (uint64_t m = 0; m < found; ++m) cb(size_t(prow[m]), payloads_[brow[m]]);
    }
    /* The directory words (2^bits + 1 of (first tuple << 16 | Bloom tag)), for
     * comparison with the reference's directory_. */
    std::vector<uint64_t> directory() const {
        if (!table_) return {};
        uint32_t        bits = 0;
        uint64_t        nt   = 0;
        const uint64_t* dir  = nullptr;
        const int32_t*  tk   = nullptr;
        const uint32_t* tr   = nullptr;
        check_rc(hj_table_info(table_, &bits, &nt, &dir, &tk, &tr));
        std::vector<uint64_t> out((size_t(1) << bits) + 1);
        copy(out.data(), dir, out.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost);
        return out;
    }
    size_t size() const { return keys_.size(); }

private:
    static void check(cudaError_t e, const char* what) {
        if (e != cudaSuccess) throw std::runtime_error(std::string("UnchainedHash: ") + what + ": " + cudaGetErrorString(e));
    }
    // copies on the context's stream, so they order with the engine's kernels
    void copy(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) const {
        check(cudaMemcpyAsync(dst, src, bytes, kind, stream_), "cudaMemcpyAsync");
        check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
    }
    void check_rc(int rc) const {
        if (rc != HJ_OK) throw std::runtime_error(std::string("UnchainedHash: ") + hj_last_error(ctx_));
    }
    void reserve_probe(size_t n, uint64_t cap) const {
        if (n > pkeys_cap_) {
            if (d_pkeys_) cudaFree(d_pkeys_);
            d_pkeys_ = nullptr;
            check(cudaMalloc(reinterpret_cast<void**>(&d_pkeys_), n * sizeof(int32_t)), "cudaMalloc");
            pkeys_cap_ = n;
        }
        if (cap == 0) cap = 1;
        if (cap > probe_cap_) {
            if (d_prow_) cudaFree(d_prow_);
            if (d_brow_) cudaFree(d_brow_);
            d_prow_ = d_brow_ = nullptr;
            check(cudaMalloc(reinterpret_cast<void**>(&d_prow_), cap * sizeof(uint32_t)), "cudaMalloc");
            check(cudaMalloc(reinterpret_cast<void**>(&d_brow_), cap * sizeof(uint32_t)), "cudaMalloc");
            probe_cap_ = cap;
        }
    }
    void release_probe_buffers() {
        for (void* p : {static_cast<void*>(d_pkeys_), static_cast<void*>(d_prow_), static_cast<void*>(d_brow_)})
            if (p) cudaFree(p);
        d_pkeys_ = nullptr;
        d_prow_ = d_brow_ = nullptr;
        pkeys_cap_ = probe_cap_ = 0;
    }

    hj_context*          ctx_;
    cudaStream_t         stream_ = nullptr;
    hj_hash_table*       table_ = nullptr;
    std::vector<int32_t> keys_;
    std::vector<Payload> payloads_;
    int32_t*             d_keys_ = nullptr;
    mutable int32_t*     d_pkeys_ = nullptr;
    mutable uint32_t*    d_prow_  = nullptr;
    mutable uint32_t*    d_brow_  = nullptr;
    mutable size_t       pkeys_cap_ = 0;
    mutable uint64_t     probe_cap_ = 0;
};

}  // namespace hjgb300
