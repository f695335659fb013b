// Batched execution of many independent joins (hj_batch_execute), and the
// synthetic instance generator the batched form is measured on
// (hj_batch_generate).
//
// An instance is a chain R0 x R1 x ... x Rm-1 of INT32 equi-joins on one key:
// R0 is probed against R1, the result against R2, and so on.  Every relation is
// (key, payload) with INT32 values and no NULLs.  An instance's result is
// summarised by its row count and an order-independent checksum: the sum mod
// 2^64, over its result rows, of a 64-bit fingerprint of key, payload0 ...
// payloadm-1 (fp_start / fp_add / fp_final below; the same on every path and
// in the oracle).
//
// Batched path: because every join of an instance is on the same key, one
// radix partitioning of the key serves the whole chain.  All relations of all
// instances are partitioned together (one histogram, scan and scatter pass),
// then each work item -- (instance, partition, chunk of R0 rows) -- builds the
// partition of every build relation as a shared-memory table and runs its R0
// rows through the whole chain in registers; no intermediate is written.  The
// kernels are persistent: grids sized to the resident capacity pull work
// items from device-side queues (atomic counters), so instances of very
// different sizes share the SMs evenly, and the whole batch runs without host
// synchronisation, captured and launched as one CUDA graph.  A partition too
// large for shared memory (heavy duplicate keys) flags its instance, which is
// then recomputed on the plain path.
//
// Plain path: the instances one at a time through the engine's regular
// radix-partitioned table build and two-pass probe (hj_build.cu, hj_probe.cu),
// with a host readback of each join's match count -- what a caller without
// batching runs.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "hj_block.cuh"
#include "hj_common.cuh"
#include "hj_kernels.h"

namespace hj {
namespace {


constexpr uint64_t kGold = 0x9e3779b97f4a7c15ull;

// splitmix64's output function (Steele, Lea, Flood 2014; constants as published by Vigna).
__host__ __device__ __forceinline__ uint64_t sm_fin(uint64_t x) {
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}
// Row fingerprint: a fold state over the row's values, one multiply per value
// (state' = (state ^ uint32(v)) * 0x9e3779b97f4a7c15, starting from the key
// xor 0x243f6a8885a308d3), finished by splitmix64's output function.  Joined
// rows carry the state; a result row contributes fp_final(state).
__host__ __device__ __forceinline__ uint64_t fp_add(uint64_t st, int32_t v) {
    return (st ^ uint64_t(uint32_t(v))) * kGold;
}
__host__ __device__ __forceinline__ uint64_t fp_start(int32_t key, int32_t payload0) {
    return fp_add((uint64_t(uint32_t(key)) ^ 0x243f6a8885a308d3ull) * kGold, payload0);
}
__host__ __device__ __forceinline__ uint64_t fp_final(uint64_t st) { return sm_fin(st); }

// ---- generator --------------------------------------------------------------
// Instance relations from (seed, instance, relation): key domain [0, 2b) with
// b = build rows; relation j >= 1 holds b distinct keys perm_j(0 .. b-1), where
// perm_j(x) = (x * 2654435761 + c_j) mod 2b is a bijection of [0, 2b)
// (2654435761 is a prime above 2b); the probe relation R0 draws each key from
// R1's keys with probability match_q24 / 2^24 and from the other half of the
// domain otherwise.  Payloads are uniform 32-bit values.
constexpr uint64_t kPermMul = 2654435761ull;

__host__ __device__ __forceinline__ uint64_t gen_base(uint64_t seed, uint32_t inst, uint32_t rel, uint32_t which) {
    return sm_fin(sm_fin(seed + kGold * (uint64_t(inst) + 1)) + 0xd1b54a32d192ed03ull * (uint64_t(rel) * 4 + which + 1));
}
__host__ __device__ __forceinline__ uint64_t gen_val(uint64_t base, uint64_t row) {
    return sm_fin(base + kGold * (row + 1));
}

__global__ void k_batch_generate(uint64_t seed, uint32_t inst, uint32_t rel, uint64_t b, uint32_t thr, uint64_t rows,
                                 int32_t* __restrict__ keys, int32_t* __restrict__ pay) {
    const uint64_t D      = 2 * b;
    const uint64_t bk     = gen_base(seed, inst, rel, 0);
    const uint64_t bp     = gen_base(seed, inst, rel, 1);
    const uint64_t bx     = gen_base(seed, inst, rel, 2);
    const uint64_t c      = gen_base(seed, inst, rel == 0 ? 1 : rel, 3) % D;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t r = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < rows; r += stride) {
        uint64_t x = r;
        if (rel == 0) {
            const bool hit = (gen_val(bk, r) >> 40) < thr;
            x              = gen_val(bx, r) % b + (hit ? 0 : b);
        }
        keys[r] = int32_t((x * kPermMul + c) % D);
        pay[r]  = int32_t(uint32_t(gen_val(bp, r)));
    }
}

// ---- batched path: one multi-way partitioned pass ---------------------------
// Every relation of an instance joins on the same key, so one partitioning of
// the key serves the whole chain: partition l of R0 meets only partition l of
// R1, R2, ...  Instance i gets p_i partition bits (about `part_rows` build
// rows per partition summed over its build relations); a row belongs to
// partition top_p_i(hash(key)).
//   1. row counts per (relation, partition), all relations of all instances
//      (8192-row items round robin; counts kept per block until its
//      relation changes)                                     k_bpart_hist
//   2. exclusive scan -> partition offsets in one partitioned buffer
//   3. rows into partition order                             k_bpart_scatter
//      (block-local counting sort in shared memory, payloads staged by
//      cp.async meanwhile, one global range reservation per (block,
//      partition), runs written out coalesced as (key, payload) pairs)
//   4. join work list: (instance partition, chunk of its R0 rows)
//                                                            k_bjoin_plan
//   5. per work item: the partition of every build relation becomes a
//      shared-memory table, and each R0 row walks the chain through them in
//      registers -- no intermediate results are written    k_bjoin
// A partition whose build rows exceed the shared-memory capacity (heavy
// duplicates) flags its instance, which is then recomputed on the plain path.
constexpr int      kPT         = 512;   // threads of the partition and join blocks
constexpr uint32_t kPartItem   = 8192;  // rows per partition-pass work item
constexpr uint32_t kJoinChunk  = 8192;  // least R0 rows per join work item (else 16 per build row)
constexpr uint32_t kMaxPartBits = 11;
constexpr uint32_t kMaxRel     = 8;     // relations per instance

struct RelInst {  // one relation of one instance
    const int32_t* keys;
    const int32_t* pay;
    uint64_t       rows;
    uint64_t       item_base;  // first partition-pass item
    uint64_t       part_base;  // global partition id of its partition 0
    uint32_t       pbits;
    uint32_t       inst;
};

struct InstInfo {
    uint64_t part_base;  // global partition id of (R0, partition 0); relation j, partition l: + j * 2^pbits + l
    uint64_t ip_base;    // first instance-partition entry of the join plan (2^pbits entries)
    uint32_t nrel;
    uint32_t pbits;
};

// Top 32 bits of fib_hash(k) in 32-bit arithmetic: with k sign-extended to 64
// bits, hi32(k * C) = umulhi(k, C_lo) + k * C_hi - (k < 0 ? C_lo : 0) (mod 2^32).
// Partition and bucket bits (at most 11 + 14) all come from these 32 bits.
__device__ __forceinline__ uint32_t fib_hi(int32_t k) {
    constexpr uint32_t CL = uint32_t(kFib), CH = uint32_t(kFib >> 32);
    const uint32_t     kl = uint32_t(k);
    return __umulhi(kl, CL) + kl * CH - (k < 0 ? CL : 0u);
}
__device__ __forceinline__ uint32_t part_of(int32_t k, uint32_t pbits) {
    return pbits ? fib_hi(k) >> (32 - pbits) : 0u;
}

// Largest i < n with key(i) <= t, for keys ascending in i (entries without
// work share their key with the next entry, so this is the owner of t).
template <class F>
__device__ __forceinline__ uint32_t owner(uint32_t n, uint64_t t, F key) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (key(mid) <= t) lo = mid;
        else               hi = mid;
    }
    return lo;
}

// The block's next work item from the queue (uniform across the block).
__device__ __forceinline__ uint64_t next_item(unsigned long long* q, unsigned long long* sh) {
    __syncthreads();
    if (threadIdx.x == 0) *sh = atomicAdd(q, 1ull);
    __syncthreads();
    return *sh;
}

// In-place scan of n shared-memory counters (exclusive or inclusive).  Warp w
// scans one contiguous slice 32 counters at a time (lane l touches counter
// i + l: no bank conflicts), then the slices are offset by the scanned slice
// totals.  `wsum` holds >= 32 words.  Every thread of the block must call it.
__device__ __forceinline__ void smem_scan(uint32_t* a, uint32_t n, bool inclusive, uint32_t* wsum) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const uint32_t per  = ((n + 31) / 32 + nw - 1) / nw * 32;
    const uint32_t b = min(n, warp * per), e = min(n, b + per);
    uint32_t       carry = 0;
    for (uint32_t i = b; i < e; i += 32) {
        const uint32_t idx = i + lane;
        const uint32_t v   = idx < e ? a[idx] : 0u;
        const uint32_t inc = warp_inclusive_scan(v);
        if (idx < e) a[idx] = carry + (inclusive ? inc : inc - v);
        carry += __shfl_sync(0xffffffffu, inc, 31);
    }
    if (lane == 0) wsum[warp] = carry;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = lane < nw ? wsum[lane] : 0u;
        const uint32_t x = warp_inclusive_scan(w);
        if (lane < nw) wsum[lane] = x - w;
    }
    __syncthreads();
    const uint32_t off = wsum[warp];
    if (off)
        for (uint32_t i = b + lane; i < e; i += 32) a[i] += off;
    __syncthreads();
}

// 0. the relation of every partition-pass item, so that the histogram and
// scatter blocks find an item's relation with one load instead of a binary
// search of dependent loads each
__global__ void k_item_rel(const RelInst* __restrict__ R, uint32_t nr, uint64_t items, uint32_t* __restrict__ rmap) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < items; t += stride)
        rmap[t] = owner(nr, t, [&](uint32_t i) { return R[i].item_base; });
}

// 1. per (relation, partition) row counts
__global__ void __launch_bounds__(kPT)
    k_bpart_hist(const RelInst* __restrict__ R, const uint32_t* __restrict__ rmap, uint64_t items,
                 uint32_t* __restrict__ cnt) {
    // Items of equal size go to the blocks round robin (no queue, no barrier
    // per item).  The block's counts accumulate in shared memory over its items
    // of one relation and go to global memory when the relation changes (items
    // are numbered relation by relation), not once per item.
    extern __shared__ uint32_t hist[];
    uint32_t cur = ~0u;  // relation whose counts the shared histogram holds
    auto flush = [&]() {
        if (cur == ~0u) return;
        const RelInst& c = R[cur];
        for (uint32_t k = threadIdx.x; k < (1u << c.pbits); k += kPT)
            if (hist[k]) atomicAdd(cnt + c.part_base + k, hist[k]);
    };
    for (uint64_t t = blockIdx.x; t < items; t += gridDim.x) {
        const uint32_t ri = __ldg(rmap + t);
        const RelInst& s  = R[ri];
        const uint64_t r0 = (t - s.item_base) * kPartItem;
        const uint64_t r1 = min(s.rows, r0 + kPartItem);
        if (r0 >= r1) continue;
        if (s.pbits == 0) {
            if (threadIdx.x == 0) atomicAdd(cnt + s.part_base, uint32_t(r1 - r0));
            continue;
        }
        const uint32_t np2 = 1u << s.pbits;
        if (ri != cur) {
            __syncthreads();  // the last item's atomics are done
            flush();
            __syncthreads();
            for (uint32_t k = threadIdx.x; k < np2; k += kPT) hist[k] = 0;
            cur = ri;
            __syncthreads();
        }
        constexpr int kPer = kPartItem / kPT;
        int32_t       kv[kPer];
#pragma unroll
        for (int j = 0; j < kPer; ++j) {  // all loads in flight before the atomics
            const uint64_t r = r0 + threadIdx.x + uint64_t(j) * kPT;
            if (r < r1) kv[j] = __ldg(s.keys + r);
        }
#pragma unroll
        for (int j = 0; j < kPer; ++j)
            if (r0 + threadIdx.x + uint64_t(j) * kPT < r1) atomicAdd(&hist[part_of(kv[j], s.pbits)], 1u);
    }
    __syncthreads();
    flush();
}

// 4-byte global -> shared copy that completes asynchronously (cp.async);
// cp_async_wait_all waits for this thread's copies.
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    const uint32_t sa = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// 3. rows into partition order.  Shared memory: the item's payloads in row
// order (copied asynchronously while the keys are ranked), its keys sorted by
// partition with each one's row in the item, then per partition its count,
// its first sorted row and its global base.
__global__ void __launch_bounds__(kPT, 2)
    k_bpart_scatter(const RelInst* __restrict__ R, const uint32_t* __restrict__ rmap, uint64_t items,
                    unsigned long long* q,
                    const uint64_t* __restrict__ off, uint32_t* __restrict__ fill, uint32_t pmax,
                    int2* __restrict__ okp) {
    extern __shared__ __align__(16) unsigned char smem[];
    int32_t*  spay  = reinterpret_cast<int32_t*>(smem);   // row order
    int32_t*  skey  = spay + kPartItem;                    // partition order
    uint32_t* hist  = reinterpret_cast<uint32_t*>(skey + kPartItem);
    uint32_t* loff  = hist + (1u << pmax);
    uint64_t* gbase = reinterpret_cast<uint64_t*>(loff + (1u << pmax));
    uint16_t* sidx  = reinterpret_cast<uint16_t*>(gbase + (1u << pmax));  // partition order: row in the item
    __shared__ unsigned long long sh;
    __shared__ uint32_t           wsum[32];
    constexpr int kPer = kPartItem / kPT;
    static_assert(kPartItem <= 65536, "row in the item fits 16 bits");
    for (uint64_t t = next_item(q, &sh); t < items; t = next_item(q, &sh)) {
        const RelInst& s  = R[__ldg(rmap + t)];
        const uint64_t r0 = (t - s.item_base) * kPartItem;
        const uint64_t r1 = min(s.rows, r0 + kPartItem);
        if (r0 >= r1) continue;
        const uint32_t pb  = s.pbits;
        const uint32_t np2 = 1u << pb;
        for (uint32_t k = threadIdx.x; k < np2; k += kPT) hist[k] = 0;
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const uint32_t i = threadIdx.x + uint32_t(j) * kPT;
            if (r0 + i < r1) cp_async4(spay + i, s.pay + r0 + i);
        }
        __syncthreads();
        uint32_t pr[kPer];  // partition << 16 | rank in the partition
        int32_t  kv[kPer];
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const uint64_t r = r0 + threadIdx.x + uint64_t(j) * kPT;
            if (r < r1) kv[j] = __ldg(s.keys + r);
        }
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const uint64_t r = r0 + threadIdx.x + uint64_t(j) * kPT;
            if (r < r1) {
                const uint32_t k = part_of(kv[j], pb);
                pr[j]            = (k << 16) | atomicAdd(&hist[k], 1u);
            }
        }
        __syncthreads();
        // global ranges first (hist still holds the counts), then local offsets;
        // a thread's reservations four at a time, all four in flight before
        // any result is stored
        for (uint32_t k0 = threadIdx.x; k0 < np2; k0 += 4 * kPT) {
            uint64_t g[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t k = k0 + uint32_t(u) * kPT;
                const uint32_t c = k < np2 ? hist[k] : 0u;
                g[u]             = c ? off[s.part_base + k] + atomicAdd(fill + s.part_base + k, c) : 0ull;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t k = k0 + uint32_t(u) * kPT;
                if (k < np2 && hist[k]) gbase[k] = g[u];
            }
        }
        for (uint32_t k = threadIdx.x; k < np2; k += kPT) loff[k] = hist[k];
        __syncthreads();
        smem_scan(loff, np2, false, wsum);
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const uint32_t i = threadIdx.x + uint32_t(j) * kPT;
            if (r0 + i < r1) {
                const uint32_t pos = loff[pr[j] >> 16] + (pr[j] & 0xffffu);
                skey[pos]          = kv[j];
                sidx[pos]          = uint16_t(i);
            }
        }
        cp_async_wait_all();
        __syncthreads();
        const uint32_t m = uint32_t(r1 - r0);
        for (uint32_t j = threadIdx.x; j < m; j += kPT) {
            const int32_t  k   = skey[j];
            const uint32_t p   = part_of(k, pb);
            const uint64_t pos = gbase[p] + (j - loff[p]);
            okp[pos]           = make_int2(k, spay[sidx[j]]);
        }
        __syncthreads();  // the next item overwrites spay
    }
}

// R0 rows of one join work item: at least 16 per build row, so the table build
// is amortised (a partition of a probe side 10x its build side is then one
// item, its tables built once).
__device__ __forceinline__ uint64_t join_chunk(uint64_t build_rows) {
    const uint64_t c = 16 * build_rows;
    return c > kJoinChunk ? c : uint64_t(kJoinChunk);
}

__device__ __forceinline__ uint64_t part_rows(const uint64_t* off, uint64_t pid) { return off[pid + 1] - off[pid]; }

// 4. join work items per instance partition: chunks of its R0 rows (none when
// any relation's partition is empty: the chain then has no result there)
__global__ void k_bjoin_plan(const InstInfo* __restrict__ I, uint32_t n, uint64_t nip, const uint64_t* __restrict__ off,
                             uint32_t* __restrict__ jcnt) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t e = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < nip; e += stride) {
        const InstInfo& s   = I[owner(n, e, [&](uint32_t i) { return I[i].ip_base; })];
        const uint64_t  l   = e - s.ip_base;
        const uint64_t  np2 = 1ull << s.pbits;
        const uint64_t  n0  = part_rows(off, s.part_base + l);
        uint64_t        nb  = 0;
        bool            any_empty = n0 == 0;
        for (uint32_t j = 1; j < s.nrel; ++j) {
            const uint64_t c = part_rows(off, s.part_base + j * np2 + l);
            nb += c;
            any_empty |= c == 0;
        }
        const uint64_t cs = join_chunk(nb);
        jcnt[e]           = any_empty ? 0u : uint32_t((n0 + cs - 1) / cs);
    }
}

// 4b. the (instance partition, instance) of every join work item, written by
// each instance partition for its items (one load per item in the join)
__global__ void k_bjoin_map(const InstInfo* __restrict__ I, uint32_t n, uint64_t nip, const uint64_t* __restrict__ joff,
                            uint2* __restrict__ jmap) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t e = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < nip; e += stride) {
        const uint64_t a = joff[e], b = joff[e + 1];
        if (a == b) continue;
        const uint32_t ii = owner(n, e, [&](uint32_t i) { return I[i].ip_base; });
        for (uint64_t t = a; t < b; ++t) jmap[t] = make_uint2(uint32_t(e), ii);
    }
}

// 5. join.  Shared memory: the build rows of the item's partition in every
// build relation (keys, payloads; at most `cap` rows together), then per
// table its bucket bounds.  Table j (relation j + 1) has 2^bits_j buckets
// after a gap word; after one inclusive scan over all tables' counts and the
// scatter, bucket b of table j holds tuples [S[sb_j + b + 1], S[sb_j + b + 2]).
// Each R0 row looks its key up in every table (a cheap compare loop that
// notes the first match and the count), stops at the first table without it,
// and forms fingerprints only for complete matches; duplicate keys are
// enumerated by an odometer over the match lists.  In chains of three or more
// relations the rows that pass table 0 are queued per warp and looked up in
// the later tables 32 at a time.
__global__ void __launch_bounds__(kPT, 2)
    k_bjoin(const InstInfo* __restrict__ I, const uint2* __restrict__ jmap, uint64_t nip,
            const uint64_t* __restrict__ joff, unsigned long long* q, const uint64_t* __restrict__ off,
            const int2* __restrict__ kp, uint32_t cap, uint32_t scap, uint32_t max_bits, uint32_t load_q8,
            unsigned long long* __restrict__ rows, unsigned long long* __restrict__ sums, uint32_t* __restrict__ ovf) {
    extern __shared__ __align__(16) unsigned char smem[];
    int32_t*  skey = reinterpret_cast<int32_t*>(smem);
    int32_t*  spay = skey + cap;
    uint32_t* S    = reinterpret_cast<uint32_t*>(spay + cap);
    __shared__ unsigned long long sh;
    __shared__ unsigned long long red[33];
    __shared__ uint32_t           wsum[32];
    // table geometry of the current item: bits, rows, first S word, source offset
    __shared__ uint32_t g_tb[kMaxRel], g_tn[kMaxRel], g_ts[kMaxRel], g_words, g_nb, g_skip;
    __shared__ uint64_t g_src[kMaxRel];
    // per warp: rows that matched table 0 once, waiting for the later tables
    constexpr uint32_t  kRing = 64;
    __shared__ int32_t  ring_key[kPT / 32][kRing];
    __shared__ uint64_t ring_fp[kPT / 32][kRing];
    const uint32_t      lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t items = joff[nip];
    for (uint64_t t = next_item(q, &sh); t < items; t = next_item(q, &sh)) {
        const uint2     em  = jmap[t];
        const uint32_t  e   = em.x, ii = em.y;
        const InstInfo& s   = I[ii];
        const uint32_t  pb  = s.pbits;
        const uint32_t  nt  = s.nrel - 1;  // tables
        const uint64_t  np2 = 1ull << pb;
        const uint64_t  l   = e - s.ip_base;
        if (threadIdx.x == 0) {
            uint32_t nb = 0;
            for (uint32_t j = 0; j < nt; ++j) {
                const uint64_t pid  = s.part_base + (j + 1) * np2 + l;
                g_src[j]            = off[pid];
                g_tn[j]             = uint32_t(part_rows(off, pid));
                nb += g_tn[j];
                const uint32_t want = uint32_t((uint64_t(g_tn[j]) * 256 + load_q8 - 1) / load_q8);
                g_tb[j]             = min(max_bits, max(1u, want > 1 ? 32u - __clz(want - 1) : 1u));
            }
            uint32_t words = 0;
            for (;;) {  // shrink the largest tables until the bucket bounds fit
                uint32_t big = 0;
                words        = 0;
                for (uint32_t j = 0; j < nt; ++j) {
                    words += (1u << g_tb[j]) + 2;
                    if (g_tb[j] > g_tb[big]) big = j;
                }
                if (words <= scap || g_tb[big] == 1) break;
                --g_tb[big];
            }
            uint32_t w = 0;
            for (uint32_t j = 0; j < nt; ++j) {
                g_ts[j] = w;
                w += (1u << g_tb[j]) + 2;
            }
            g_words = words;
            g_nb    = nb;
            // a partition too large for shared memory: the plain path redoes the instance
            g_skip  = nb > cap || words > scap;
            if (g_skip) atomicOr(ovf + ii, 1u);
        }
        __syncthreads();
        if (g_skip) continue;
        const uint32_t words = g_words;
        auto bucket = [&](uint32_t j, int32_t k) { return (fib_hi(k) << pb) >> (32 - g_tb[j]); };
        // build the tables
        for (uint32_t w = threadIdx.x; w < words; w += kPT) S[w] = 0;
        __syncthreads();
        // four rows per thread in flight per step, loads before the atomics
        constexpr uint32_t kBU = 4;
        for (uint32_t j = 0; j < nt; ++j) {
            const uint32_t tn = g_tn[j];
            const int32_t* kj = reinterpret_cast<const int32_t*>(kp + g_src[j]);  // keys: even words
            for (uint32_t r = threadIdx.x; r < tn; r += kBU * kPT) {
                int32_t kk[kBU];
#pragma unroll
                for (uint32_t u = 0; u < kBU; ++u) kk[u] = r + u * kPT < tn ? __ldg(kj + 2 * (r + u * kPT)) : 0;
#pragma unroll
                for (uint32_t u = 0; u < kBU; ++u)
                    if (r + u * kPT < tn) atomicAdd(&S[g_ts[j] + bucket(j, kk[u]) + 1], 1u);
            }
        }
        __syncthreads();
        smem_scan(S, words, true, wsum);
        for (uint32_t j = 0; j < nt; ++j) {
            const uint32_t tn = g_tn[j];
            const int2* qj = kp + g_src[j];
            for (uint32_t r = threadIdx.x; r < tn; r += kBU * kPT) {
                int32_t kk[kBU], pv[kBU];
#pragma unroll
                for (uint32_t u = 0; u < kBU; ++u) {
                    const int2 v = r + u * kPT < tn ? __ldg(qj + r + u * kPT) : make_int2(0, 0);
                    kk[u]        = v.x;
                    pv[u]        = v.y;
                }
#pragma unroll
                for (uint32_t u = 0; u < kBU; ++u)
                    if (r + u * kPT < tn) {
                        const uint32_t pos = atomicSub(&S[g_ts[j] + bucket(j, kk[u]) + 1], 1u) - 1;
                        skey[pos]          = kk[u];
                        spay[pos]          = pv[u];
                    }
            }
        }
        __syncthreads();
        // probe the item's R0 rows
        const uint64_t p0 = off[s.part_base + l];
        const uint64_t cs = join_chunk(g_nb);
        const uint64_t x0 = p0 + (t - joff[e]) * cs;
        const uint32_t m  = uint32_t(min(p0 + part_rows(off, s.part_base + l), x0 + cs) - x0);
        const int2*    pq = kp + x0;
        unsigned long long my_rows = 0, my_sum = 0;
        // matches of key k in bucket word b: their count, and the first in `first`
        auto scan_bucket = [&](uint32_t b, int32_t k, uint32_t& first) {
            const uint32_t be = S[b + 2];
            uint32_t       cnt = 0, j1 = 0;
            for (uint32_t y = S[b + 1]; y < be; ++y)
                if (skey[y] == k) {
                    j1 = cnt ? j1 : y;
                    ++cnt;
                }
            first = j1;
            return cnt;
        };
        auto lookup = [&](uint32_t j, int32_t k, uint32_t& first) {
            return scan_bucket(g_ts[j] + bucket(j, k), k, first);
        };
        // table 0, which every row meets, with its geometry in registers
        const uint32_t ts0 = g_ts[0], sh0 = 32 - g_tb[0];
        auto lookup0 = [&](int32_t k, uint32_t& first) {
            return scan_bucket(ts0 + ((fib_hi(k) << pb) >> sh0), k, first);
        };
        // every combination of one match per table j0 .. nt-1 for key k, the
        // tables before j0 folded into fp (an odometer over the match lists)
        auto enumerate = [&](uint32_t j0, int32_t k, uint64_t fp) {
            uint32_t first[kMaxRel], pos[kMaxRel];
            uint64_t fpl[kMaxRel + 1];
            fpl[j0] = fp;
            for (uint32_t j = j0; j < nt; ++j) {
                if (!lookup(j, k, first[j])) return;
                pos[j]     = first[j];
                fpl[j + 1] = fp_add(fpl[j], spay[pos[j]]);
            }
            for (;;) {
                ++my_rows;
                my_sum += fp_final(fpl[nt]);
                int j = int(nt) - 1;
                for (; j >= int(j0); --j) {
                    const uint32_t be = S[g_ts[j] + bucket(uint32_t(j), k) + 2];
                    uint32_t       y  = pos[j] + 1;
                    while (y < be && skey[y] != k) ++y;
                    if (y < be) {
                        pos[j] = y;
                        break;
                    }
                    pos[j] = first[j];
                }
                if (j < int(j0)) break;
                for (uint32_t z = uint32_t(j); z < nt; ++z) fpl[z + 1] = fp_add(fpl[z], spay[pos[z]]);
            }
        };
        // the next row's key and payload are loaded while this row is looked up
        int2 q_next = threadIdx.x < m ? __ldg(pq + threadIdx.x) : make_int2(0, 0);
        if (nt == 1) {
            for (uint32_t x = threadIdx.x; x < m; x += kPT) {
                const int32_t k = q_next.x, pv = q_next.y;
                if (x + kPT < m) q_next = __ldg(pq + x + kPT);
                uint32_t       f;
                const uint32_t c = lookup0(k, f);
                if (c == 1) {
                    ++my_rows;
                    my_sum += fp_final(fp_add(fp_start(k, pv), spay[f]));
                } else if (c > 1) {
                    enumerate(0, k, fp_start(k, pv));
                }
            }
        } else {
            // Table 0 is looked up for every row.  Rows with one match there
            // queue up in the warp's ring (key and fold state) and the later
            // tables are looked up 32 queued rows at a time, so that lanes
            // whose row missed table 0 do not idle through them.
            int32_t*       qk   = ring_key[warp];
            uint64_t*      qf   = ring_fp[warp];
            uint32_t       qh = 0, qt = 0;  // ring head and tail (warp-uniform)
            auto drain = [&](uint32_t cnt) {
                __syncwarp();
                if (lane < cnt) {
                    const uint32_t slot = (qh + lane) % kRing;
                    const int32_t  k    = qk[slot];
                    uint64_t       fp   = qf[slot];
                    uint32_t       j = 1, c = 1;
                    for (; j < nt; ++j) {
                        uint32_t f;
                        c = lookup(j, k, f);
                        if (c != 1) break;
                        fp = fp_add(fp, spay[f]);
                    }
                    if (j == nt) {
                        ++my_rows;
                        my_sum += fp_final(fp);
                    } else if (c > 1) {
                        enumerate(j, k, fp);
                    }
                }
                qh += cnt;
                __syncwarp();
            };
            for (uint32_t x = threadIdx.x; x - lane < m; x += kPT) {  // warp-uniform bound
                const int32_t k = q_next.x, pv = q_next.y;
                if (x + kPT < m) q_next = __ldg(pq + x + kPT);
                uint32_t f = 0, c = 0;
                if (x < m) c = lookup0(k, f);
                if (c > 1) enumerate(0, k, fp_start(k, pv));
                const unsigned hm = __ballot_sync(0xffffffffu, c == 1);
                if (c == 1) {
                    const uint32_t slot = (qt + __popc(hm & ((1u << lane) - 1u))) % kRing;
                    qk[slot]            = k;
                    qf[slot]            = fp_add(fp_start(k, pv), spay[f]);
                }
                qt += __popc(hm);
                if (qt - qh >= 32) drain(32);
            }
            drain(qt - qh);
        }
        unsigned long long tr, tsum;
        block_exclusive_scan<unsigned long long>(my_rows, red, &tr);
        block_exclusive_scan<unsigned long long>(my_sum, red, &tsum);
        if (threadIdx.x == 0 && tr) {
            atomicAdd(rows + ii, tr);
            atomicAdd(sums + ii, tsum);
        }
    }
}

// ---- plain path helper --------------------------------------------------------
// (probe row, build row) pairs -> next (key, fold state) rows, or (okey null)
// the checksum of a last join.
__global__ void k_pairs_next(const uint32_t* __restrict__ prow, const uint32_t* __restrict__ brow, uint64_t n,
                             const int32_t* __restrict__ pkeys, const uint64_t* __restrict__ pfp,
                             const int32_t* __restrict__ ppay, const int32_t* __restrict__ bpay,
                             int32_t* __restrict__ okey, uint64_t* __restrict__ ofp, unsigned long long* __restrict__ sum) {
    unsigned long long acc    = 0;
    const uint64_t     stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t p  = prow[i];
        const int32_t  k  = pkeys[p];
        const uint64_t fp = pfp ? pfp[p] : fp_start(k, ppay[p]);
        const uint64_t nf = fp_add(fp, bpay[brow[i]]);
        if (okey) {
            okey[i] = k;
            ofp[i]  = nf;
        } else {
            acc += fp_final(nf);
        }
    }
    if (!okey) {
        acc = warp_sum(acc);
        if ((threadIdx.x & 31) == 0 && acc) atomicAdd(sum, acc);
    }
}

uint32_t ceil_log2u(uint64_t x) {
    uint32_t b = 0;
    while (b < 63 && (1ull << b) < x) ++b;
    return b;
}

// Blocks of `kernel` that fit on the GPU at once with `smem` dynamic shared
// memory (the grid of a persistent launch); raises the kernel's dynamic
// shared-memory limit first.  Not capturable: called before a capture.
template <class K>
int resident_grid(K kernel, size_t smem) {
    HJ_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int per_sm = 0;
    HJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kPT, smem));
    if (per_sm < 1) throw Error(HJ_ERR_INVALID, "batch: a kernel does not fit on an SM");
    return per_sm * num_sms();
}

}  // namespace

void launch_batch_generate(uint64_t seed, uint32_t instance, uint32_t relation, uint64_t build_rows,
                           uint32_t match_q24, uint64_t rows, int32_t* keys, int32_t* payload, cudaStream_t st) {
    if (build_rows == 0 || build_rows > (1ull << 30))
        throw Error(HJ_ERR_INVALID, "batch_generate: build rows must be in [1, 2^30]");
    if (relation > 0 && rows > build_rows)
        throw Error(HJ_ERR_INVALID, "batch_generate: a build relation has at most build_rows rows");
    if (match_q24 > (1u << 24)) throw Error(HJ_ERR_INVALID, "batch_generate: match rate above 2^24");
    if (rows == 0) return;
    if (!keys || !payload) throw Error(HJ_ERR_INVALID, "batch_generate: null output");
    const unsigned blocks = unsigned(std::min<uint64_t>(div_up(rows, 256), uint64_t(num_sms()) * 16));
    k_batch_generate<<<blocks, 256, 0, st>>>(seed, instance, relation, build_rows, match_q24, rows, keys, payload);
    HJ_LAUNCH_CHECK();
}

std::vector<uint32_t> batch_execute(const std::vector<BatchInstance>& B, const BatchOptions& o,
                                    std::vector<uint64_t>& rows, std::vector<uint64_t>& sums, cudaStream_t st) {
    const uint32_t n = uint32_t(B.size());
    rows.assign(n, 0);
    sums.assign(n, 0);
    if (n == 0) return {};
    if (!(o.load > 0.0 && o.load <= 8.0)) throw Error(HJ_ERR_INVALID, "batch: directory load out of range");
    if (o.part_rows_log2 < 8 || o.part_rows_log2 > 13)
        throw Error(HJ_ERR_INVALID, "batch: partition size must be 2^8 .. 2^13 build rows");
    for (const auto& b : B) {
        if (b.rels.size() < 2 || b.rels.size() > kMaxRel)
            throw Error(HJ_ERR_INVALID, "a batch instance needs 2 to 8 relations");
        for (const auto& r : b.rels) {
            if (r.rows > 0xffffffffull) throw Error(HJ_ERR_INVALID, "a batch relation has more than 2^32-1 rows");
            if (r.rows && (!r.keys || !r.payload)) throw Error(HJ_ERR_INVALID, "a batch relation lacks its columns");
        }
    }
    // shared-memory geometry: partitions of ~T build rows (all build relations
    // together), tables of up to 2T rows, bucket bounds for 2^max_bits buckets
    const uint64_t T        = 1ull << o.part_rows_log2;
    const uint32_t cap      = uint32_t(2 * T);
    const uint32_t max_bits = std::max<uint32_t>(1, ceil_log2u(uint64_t(std::ceil(double(T) / o.load))));
    const uint32_t scap     = (1u << max_bits) + 2 * kMaxRel;
    const uint32_t load_q8  = std::max<uint32_t>(1, uint32_t(std::lround(o.load * 256.0)));
    const size_t   join_smem = size_t(cap) * 8 + size_t(scap) * 4;
    if (join_smem > 200 * 1024) throw Error(HJ_ERR_INVALID, "batch: partition tables exceed shared memory");

    std::vector<RelInst>  hr;
    std::vector<InstInfo> hi(n);
    uint64_t pbase = 0, ipbase = 0, items = 0, total_rows = 0, r0_rows = 0;
    uint32_t pmax = 0;
    for (uint32_t i = 0; i < n; ++i) {
        uint64_t nb = 0;
        for (size_t j = 1; j < B[i].rels.size(); ++j) nb += B[i].rels[j].rows;
        const uint32_t p = nb > T ? std::min(kMaxPartBits, ceil_log2u((nb + T - 1) / T)) : 0;
        pmax             = std::max(pmax, p);
        InstInfo& s      = hi[i];
        s.part_base      = pbase;
        s.ip_base        = ipbase;
        s.nrel           = uint32_t(B[i].rels.size());
        s.pbits          = p;
        for (uint32_t j = 0; j < s.nrel; ++j) {
            const BatchRelation& br = B[i].rels[j];
            hr.push_back({br.keys, br.payload, br.rows, items, pbase + (uint64_t(j) << p), p, i});
            items += (br.rows + kPartItem - 1) / kPartItem;
            total_rows += br.rows;
        }
        r0_rows += B[i].rels[0].rows;
        pbase += uint64_t(s.nrel) << p;
        ipbase += 1ull << p;
    }
    const uint32_t nr = uint32_t(hr.size());

    std::vector<void*> owned;
    struct Release {
        std::vector<void*>& v;
        cudaStream_t        st;
        ~Release() {
            for (void* p : v) dfree(p, st);
        }
    } release{owned, st};
    auto take = [&](size_t bytes) {
        void* p = dalloc(bytes + 16, st);
        owned.push_back(p);
        return p;
    };
    auto* d_rows = static_cast<unsigned long long*>(take(n * 8));
    auto* d_sums = static_cast<unsigned long long*>(take(n * 8));
    auto* d_ovf  = static_cast<uint32_t*>(take(n * 4));
    auto* d_q    = static_cast<unsigned long long*>(take(4 * 8));
    auto* d_R    = static_cast<RelInst*>(take(nr * sizeof(RelInst)));
    auto* d_I    = static_cast<InstInfo*>(take(n * sizeof(InstInfo)));
    auto* cnt    = static_cast<uint32_t*>(take((pbase + 1) * 4));
    auto* fill   = static_cast<uint32_t*>(take((pbase + 1) * 4));
    auto* off    = static_cast<uint64_t*>(take((pbase + 2) * 8));
    auto* jcnt   = static_cast<uint32_t*>(take((ipbase + 1) * 4));
    auto* joff   = static_cast<uint64_t*>(take((ipbase + 2) * 8));
    auto* tmp    = static_cast<uint64_t*>(take((std::max(scan_tmp_words(pbase), scan_tmp_words(ipbase)) + 1) * 8));
    auto* pkp    = static_cast<int2*>(take(total_rows * 8));  // (key, payload) in partition order
    auto* rmap   = static_cast<uint32_t*>(take(items * 4));
    // join items: at most one per instance partition plus one per kJoinChunk R0 rows
    auto* jmap   = static_cast<uint2*>(take((ipbase + r0_rows / kJoinChunk + 1) * 8));
    HJ_CUDA(cudaMemcpyAsync(d_R, hr.data(), nr * sizeof(RelInst), cudaMemcpyHostToDevice, st));
    HJ_CUDA(cudaMemcpyAsync(d_I, hi.data(), n * sizeof(InstInfo), cudaMemcpyHostToDevice, st));
    HJ_CUDA(cudaStreamSynchronize(st));  // the host arrays stay alive until here

    // persistent grids (occupancy queries are not capturable: take them first)
    const size_t hist_smem = (size_t(1) << pmax) * 4;
    const size_t scat_smem = size_t(kPartItem) * 10 + (size_t(1) << pmax) * 16;
    const int    g_hist    = resident_grid(k_bpart_hist, hist_smem);
    const int    g_scat    = resident_grid(k_bpart_scatter, scat_smem);
    const int    g_join    = resident_grid(k_bjoin, join_smem);
    auto grid_for = [](int g, uint64_t work) { return unsigned(std::max<uint64_t>(1, std::min<uint64_t>(g, work))); };

    auto enqueue = [&]() {
        HJ_CUDA(cudaMemsetAsync(d_rows, 0, n * 8, st));
        HJ_CUDA(cudaMemsetAsync(d_sums, 0, n * 8, st));
        HJ_CUDA(cudaMemsetAsync(d_ovf, 0, n * 4, st));
        HJ_CUDA(cudaMemsetAsync(d_q, 0, 4 * 8, st));
        HJ_CUDA(cudaMemsetAsync(cnt, 0, (pbase + 1) * 4, st));
        HJ_CUDA(cudaMemsetAsync(fill, 0, (pbase + 1) * 4, st));
        if (items) {
            k_item_rel<<<unsigned(std::min<uint64_t>(div_up(items, 256), uint64_t(num_sms()) * 8)), 256, 0, st>>>(
                d_R, nr, items, rmap);
            HJ_LAUNCH_CHECK();
            k_bpart_hist<<<grid_for(g_hist, items), kPT, hist_smem, st>>>(d_R, rmap, items, cnt);
            HJ_LAUNCH_CHECK();
        }
        scan_exclusive_u32_to_u64_into(cnt, off, pbase, tmp, st);
        if (items) {
            k_bpart_scatter<<<grid_for(g_scat, items), kPT, scat_smem, st>>>(d_R, rmap, items, d_q + 1, off, fill,
                                                                             pmax, pkp);
            HJ_LAUNCH_CHECK();
        }
        k_bjoin_plan<<<unsigned(std::min<uint64_t>(div_up(ipbase, 256), uint64_t(num_sms()) * 8)), 256, 0, st>>>(
            d_I, n, ipbase, off, jcnt);
        HJ_LAUNCH_CHECK();
        scan_exclusive_u32_to_u64_into(jcnt, joff, ipbase, tmp, st);
        k_bjoin_map<<<unsigned(std::min<uint64_t>(div_up(ipbase, 256), uint64_t(num_sms()) * 8)), 256, 0, st>>>(
            d_I, n, ipbase, joff, jmap);
        HJ_LAUNCH_CHECK();
        // the item count lives on the device: launch the resident grid
        k_bjoin<<<unsigned(g_join), kPT, join_smem, st>>>(d_I, jmap, ipbase, joff, d_q + 2, off, pkp, cap,
                                                          scap, max_bits, load_q8, d_rows, d_sums, d_ovf);
        HJ_LAUNCH_CHECK();
    };
    if (o.graph) {
        cudaGraph_t g = nullptr;
        HJ_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        try {
            enqueue();
        } catch (...) {
            cudaStreamEndCapture(st, &g);
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            throw;
        }
        HJ_CUDA(cudaStreamEndCapture(st, &g));
        cudaGraphExec_t   ge = nullptr;
        const cudaError_t e  = cudaGraphInstantiate(&ge, g, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            throw Error(HJ_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
        }
        const cudaError_t le = cudaGraphLaunch(ge, st);
        const cudaError_t se = cudaStreamSynchronize(st);
        cudaGraphExecDestroy(ge);
        cudaGraphDestroy(g);
        HJ_CUDA(le);
        HJ_CUDA(se);
    } else {
        enqueue();
    }
    std::vector<uint32_t> ovf(n);
    HJ_CUDA(cudaMemcpyAsync(rows.data(), d_rows, n * 8, cudaMemcpyDeviceToHost, st));
    HJ_CUDA(cudaMemcpyAsync(sums.data(), d_sums, n * 8, cudaMemcpyDeviceToHost, st));
    HJ_CUDA(cudaMemcpyAsync(ovf.data(), d_ovf, n * 4, cudaMemcpyDeviceToHost, st));
    HJ_CUDA(cudaStreamSynchronize(st));
    std::vector<uint32_t> bad;
    for (uint32_t i = 0; i < n; ++i)
        if (ovf[i]) bad.push_back(i);
    return bad;
}

void plain_instance(const BatchInstance& b, const ProbeParams& prm, int dir_bits, int radix_bits, int dir_cap_bits,
                    uint64_t& rows, uint64_t& sum, cudaStream_t st) {
    rows = sum = 0;
    if (b.rels.size() < 2) throw Error(HJ_ERR_INVALID, "a batch instance needs at least two relations");
    std::vector<void*> owned;
    struct Release {
        std::vector<void*>& v;
        cudaStream_t        st;
        ~Release() {
            for (void* p : v) dfree(p, st);
        }
    } release{owned, st};
    auto take = [&](size_t bytes) {
        void* p = dalloc(bytes + 16, st);
        owned.push_back(p);
        return p;
    };
    auto*           d_sum = static_cast<unsigned long long*>(take(8));
    const int32_t*  pkeys = b.rels[0].keys;
    const int32_t*  ppay  = b.rels[0].payload;
    const uint64_t* pfp   = nullptr;
    uint64_t        np    = b.rels[0].rows;
    HJ_CUDA(cudaMemsetAsync(d_sum, 0, 8, st));
    for (size_t sg = 1; sg < b.rels.size() && np > 0; ++sg) {
        const BatchRelation& br   = b.rels[sg];
        const bool           last = sg + 1 == b.rels.size();
        if (br.rows == 0) break;
        IntCol bc;
        bc.plain = br.keys;
        IntCol pc;
        pc.plain = pkeys;
        const KeyCol pk{pc, nullptr, np};
        Table        t;
        build_table(KeyCol{bc, nullptr, br.rows}, dir_bits, radix_bits, t, prm.pinned, st, int64_t(br.rows),
                    dir_cap_bits);
        ProbePlan* pp    = nullptr;
        uint64_t   total = 0;
        uint32_t * pr = nullptr, *bw = nullptr;
        try {
            total = probe_count(t, pk, prm, &pp, st);
            pr    = static_cast<uint32_t*>(take(total * 4));
            bw    = static_cast<uint32_t*>(take(total * 4));
            const RidOut ro[2] = {{0, nullptr, pr}, {1, nullptr, bw}};
            if (total) probe_write(t, pk, pp, ro, 2, st);
        } catch (...) {
            if (pp) probe_free(pp, st);
            free_table(t, st);
            throw;
        }
        probe_free(pp, st);
        free_table(t, st);
        int32_t*  nk = last ? nullptr : static_cast<int32_t*>(take(total * 4));
        uint64_t* nf = last ? nullptr : static_cast<uint64_t*>(take(total * 8));
        if (total) {
            k_pairs_next<<<unsigned(std::min<uint64_t>(div_up(total, 256), uint64_t(num_sms()) * 8)), 256, 0, st>>>(
                pr, bw, total, pkeys, pfp, ppay, br.payload, nk, nf, d_sum);
            HJ_LAUNCH_CHECK();
        }
        pkeys = nk;
        pfp   = nf;
        ppay  = nullptr;
        np    = total;
        if (last) rows = total;
    }
    readback(prm.pinned, d_sum, 8, true, st);  // page-locked scratch
    HJ_CUDA(cudaStreamSynchronize(st));
    sum = prm.pinned[0];
}

}  // namespace hj
