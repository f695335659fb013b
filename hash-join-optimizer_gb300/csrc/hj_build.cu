// Unchained hash-table build on the GPU.
//
// Semantics of UnchainedHash::finalize_build (include/unchained.h:155-217 of
// the reference): Fibonacci hash, directory of 2^b words (default b =
// log2(next_pow2(#tuples))), word = (first adjacency-array index << 16) |
// 16-bit Bloom tag (OR of bloom_mask over the bucket's tuples), sentinel word
// 2^b = #tuples << 16; the adjacency array holds the tuples grouped by bucket.
// The directory words are therefore bit-identical to UnchainedHash's for the
// same key multiset (only the order of tuples inside a bucket may differ).
//
// The reference's live table, PartitionedDirectoryHash
// (include/partitioned_directory_hash.h:86-198), builds the same kind of
// adjacency array on the host with per-thread slab buffers
// (include/slab_allocator.h) and three phases.  Here the slabs are replaced by
// a two-level MSD radix partition:
//   1. k_part_hist      histogram of the top R hash bits (R = b - 12)
//   2. k_part_offsets   partition offsets and per-partition chunk counts
//   3. k_part_scatter   (key, row) pairs scattered to their partition
// Partitions of at most kFuseMax tuples are then built by one block each
// (k_bucket_local); the larger ones (Zipf-heavy keys) take steps 4-7, with
// their counters cleared first (k_bucket_zero):
//   4. k_bucket_count   per 8192-tuple chunk: shared-memory bucket counts and
//                       Bloom tags over the partition's 2^12 buckets
//   5. k_bucket_dir     per partition: prefix sum -> directory words
//   6. k_bucket_scatter per chunk: tuples to their final adjacency slots
//   7. k_bucket_mixed   flags buckets that hold more than one distinct key
// Shared-memory histograms per chunk keep Zipf-heavy keys (one key can own
// millions of tuples) off global atomics: a chunk adds one atomic per
// non-empty bucket, and warp-aggregated shared atomics absorb duplicates.
#include <algorithm>

#include "hj_block.cuh"
#include "hj_common.cuh"
#include "hj_kernels.h"

namespace hj {
namespace {

constexpr int kLocalBits   = 12;  // buckets per partition = 2^12 (16 KB of shared counters)
constexpr int kMaxRadix    = 14;
constexpr int kThreads     = 512;
constexpr int kItems       = 16;
constexpr int kTile        = kThreads * kItems;  // rows per partition-scatter tile
constexpr int kChunkTiles  = 1;
constexpr int kChunk       = kChunkTiles * kTile;  // tuples per bucket chunk
// Partitions of at most kFuseMax tuples are built by one block each
// (k_bucket_local); the chunked kernels take the larger ones.
constexpr uint32_t kFuseMax = 12288;

struct Geo {
    uint32_t b;  // directory bits
    uint32_t R;  // partition bits
    uint32_t L;  // local bucket bits = b - R
};

__device__ __forceinline__ bool load_key(const KeyCol& kc, uint64_t i, int32_t& key) {
    if (i >= kc.n) return false;
    return int_get(kc.col, kc.rid ? uint64_t(__ldg(kc.rid + i)) : i, key);
}

// 1. Partition histogram + count of valid keys.
__global__ void __launch_bounds__(kThreads)
    k_part_hist(KeyCol kc, uint32_t R, uint32_t* __restrict__ part_cnt,
                unsigned long long* __restrict__ n_valid) {
    extern __shared__ uint32_t hist[];
    const uint32_t P = 1u << R;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    uint32_t       mine = 0;
    constexpr int  kU   = 8;  // keys per thread loaded before any of them is counted
    const uint64_t step = uint64_t(gridDim.x) * blockDim.x * kU;
    for (uint64_t b0 = uint64_t(blockIdx.x) * blockDim.x * kU + threadIdx.x; b0 < kc.n; b0 += step) {
        int32_t key[kU];
        bool    ok[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) ok[u] = load_key(kc, b0 + uint64_t(u) * blockDim.x, key[u]);
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            if (ok[u]) {
                atomicAdd(hist + uint32_t(bucket_of(fib_hash(key[u]), R)), 1u);
                ++mine;
            }
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x)
        if (hist[i]) atomicAdd(part_cnt + i, hist[i]);
    mine = warp_sum(mine);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(n_valid, (unsigned long long)mine);
}

// 2. Exclusive scans of partition sizes and chunk counts (one block).  Only
//    the partitions k_bucket_local does not take are cut into chunks; each
//    chunk's partition is written to chunk_part, so a chunk kernel's block
//    finds its partition with one load.
__global__ void __launch_bounds__(1024)
    k_part_offsets(const uint32_t* __restrict__ part_cnt, uint32_t P, uint32_t* __restrict__ part_off,
                   uint32_t* __restrict__ part_cursor, uint32_t* __restrict__ chunk_off,
                   uint32_t* __restrict__ chunk_part) {
    __shared__ uint32_t sm[33];
    uint32_t            run_t = 0, run_c = 0;
    for (uint32_t base = 0; base < P; base += blockDim.x) {
        const uint32_t i  = base + threadIdx.x;
        const uint32_t c  = i < P ? part_cnt[i] : 0;
        const uint32_t ch = c > kFuseMax ? (c + kChunk - 1) / kChunk : 0u;
        uint32_t       tot_t, tot_c;
        const uint32_t et = block_exclusive_scan<uint32_t>(c, sm, &tot_t);
        const uint32_t ec = block_exclusive_scan<uint32_t>(ch, sm, &tot_c);
        if (i < P) {
            part_off[i]    = run_t + et;
            part_cursor[i] = run_t + et;
            chunk_off[i]   = run_c + ec;
        }
        run_t += tot_t;
        run_c += tot_c;
    }
    if (threadIdx.x == 0) {
        part_off[P]  = run_t;
        chunk_off[P] = run_c;
    }
    __syncthreads();
    for (uint32_t p = threadIdx.x; p < P; p += blockDim.x)
        for (uint32_t c = chunk_off[p]; c < chunk_off[p + 1]; ++c) chunk_part[c] = p;
}

// 3. Scatter (key, row) to partitions.  Each block owns a tile of kTile rows:
//    shared-memory counts give every item its rank in its partition within
//    the tile, one global atomic per (tile, non-empty partition) reserves the
//    partition's space, the items are placed partition by partition in shared
//    memory and then stored so that consecutive threads write consecutive
//    slots of a partition (runs instead of single 4-byte stores).
template <int kST>  // threads; a tile is kST * kItems rows
__global__ void __launch_bounds__(kST, 1024 / kST)
    k_part_scatter(KeyCol kc, uint32_t R, uint32_t* __restrict__ part_cursor,
                   int32_t* __restrict__ tkey, uint32_t* __restrict__ trow) {
    extern __shared__ uint32_t sh[];  // P counters / tile offsets, P global bases, staged items
    __shared__ uint32_t sm[33];
    const uint32_t P     = 1u << R;
    uint32_t*      off   = sh;                   // counts, then the tile's partition offsets
    uint32_t*      gbase = sh + P;               // global slot of each partition's first item
    int32_t*       sk    = reinterpret_cast<int32_t*>(sh + 2 * P);
    constexpr int  kT    = kST * kItems;
    uint32_t*      sr    = sh + 2 * P + kT;
    uint16_t*      sp    = reinterpret_cast<uint16_t*>(sh + 2 * P + 2 * kT);  // partition of each slot
    const uint64_t tile0 = uint64_t(blockIdx.x) * kT;
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) off[i] = 0;
    __syncthreads();
    int32_t  keys[kItems];
    uint32_t rank[kItems];
    uint32_t okmask = 0;
    // all of the thread's keys are loaded before any is counted
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const uint64_t i = tile0 + uint64_t(k) * kST + threadIdx.x;
        okmask |= uint32_t(load_key(kc, i, keys[k])) << k;
    }
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        const bool ok = (okmask >> k) & 1u;
        rank[k]       = ok ? atomicAdd(off + uint32_t(bucket_of(fib_hash(keys[k]), R)), 1u) : 0;
    }
    __syncthreads();
    // exclusive scan of the counts (thread t: partitions [t * per, (t + 1) * per))
    const uint32_t per = (P + kST - 1) / kST;
    uint32_t       run = 0;
    // the thread's reservations four at a time, all four in flight before any
    // result is stored
    for (uint32_t q0 = 0; q0 < per; q0 += 4) {
        uint32_t base[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t q = q0 + u, p = threadIdx.x * per + q;
            const uint32_t c = q < per && p < P ? off[p] : 0u;
            base[u]          = c ? atomicAdd(part_cursor + p, c) : 0u;
            run += c;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t q = q0 + u, p = threadIdx.x * per + q;
            if (q < per && p < P) gbase[p] = base[u];
        }
    }
    uint32_t       tot;
    const uint32_t ex = block_exclusive_scan<uint32_t>(run, sm, &tot);
    run               = ex;
    for (uint32_t q = 0; q < per; ++q) {
        const uint32_t p = threadIdx.x * per + q;
        if (p < P) {
            const uint32_t c = off[p];
            off[p]           = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        if ((okmask >> k) & 1u) {
            const uint32_t part = uint32_t(bucket_of(fib_hash(keys[k]), R));  // recomputed: fewer registers
            const uint32_t q    = off[part] + rank[k];
            sk[q]               = keys[k];
            sr[q]               = uint32_t(tile0 + uint64_t(k) * kST + threadIdx.x);
            sp[q]               = uint16_t(part);
        }
    }
    __syncthreads();
    for (uint32_t q = threadIdx.x; q < tot; q += blockDim.x) {
        const uint32_t p   = sp[q];
        const uint32_t pos = gbase[p] + (q - off[p]);
        tkey[pos]          = sk[q];
        trow[pos]          = sr[q];
    }
}


__device__ __forceinline__ bool fused_part(const uint32_t* part_off, uint32_t part) {
    return part_off[part + 1] - part_off[part] <= kFuseMax;
}

// Locates chunk `cid`: its partition and tuple range.  Returns false past the end.
__device__ __forceinline__ bool chunk_range(uint32_t cid, const uint32_t* chunk_off, const uint32_t* chunk_part,
                                            const uint32_t* part_off, uint32_t P, uint32_t& part,
                                            uint32_t& s, uint32_t& e, bool& single) {
    if (cid >= chunk_off[P]) return false;
    part             = chunk_part[cid];
    const uint32_t k = cid - chunk_off[part];
    s                = part_off[part] + k * kChunk;
    e                = min(part_off[part + 1], s + kChunk);
    single           = chunk_off[part + 1] - chunk_off[part] == 1;
    return true;
}

// Shared counter addr[slot] += 1 for each active lane, returning the lane's
// old value.  Lanes of a warp that all carry one slot (a Zipf-heavy key fills
// whole chunks) need one atomic; otherwise each lane adds on its own.
__device__ __forceinline__ uint32_t bucket_add(uint32_t* addr, uint32_t slot, unsigned act) {
    const unsigned lane   = threadIdx.x & 31;
    const int      leader = __ffs(act) - 1;
    // uniform when every active lane carries the leader's slot (a shuffle and
    // a vote: cheaper than a match instruction)
    const bool uni = __all_sync(act, slot == __shfl_sync(act, slot, leader));
    if (uni) {
        uint32_t  base   = 0;
        if (int(lane) == leader) base = atomicAdd(addr + slot, uint32_t(__popc(act)));
        return __shfl_sync(act, base, leader) + __popc(act & ((1u << lane) - 1));
    }
    return atomicAdd(addr + slot, 1u);
}

// Zeroes the bucket counters and Bloom tags of the partitions cut into more
// than one chunk (k_bucket_count accumulates those with global atomics; a
// single-chunk partition's are stored whole, and k_bucket_local's partitions
// use neither).  One block per partition.
__global__ void __launch_bounds__(256)
    k_bucket_zero(Geo g, const uint32_t* __restrict__ chunk_off, const uint32_t* __restrict__ part_off,
                  uint32_t* __restrict__ gcnt, uint32_t* __restrict__ gbloom) {
    const uint32_t part = blockIdx.x;
    if (fused_part(part_off, part) || chunk_off[part + 1] - chunk_off[part] <= 1) return;
    const uint32_t nl = 1u << g.L;
    const uint64_t gb = uint64_t(part) << g.L;
    for (uint32_t i = threadIdx.x; i < nl; i += blockDim.x) {
        gcnt[gb + i]   = 0;
        gbloom[gb + i] = 0;
    }
}

// 4. Per-chunk bucket counts and Bloom tags.
__global__ void __launch_bounds__(kThreads)
    k_bucket_count(Geo g, const uint32_t* __restrict__ chunk_off, const uint32_t* __restrict__ chunk_part,
                   const uint32_t* __restrict__ part_off,
                   const int32_t* __restrict__ tkey, uint32_t* __restrict__ gcnt,
                   uint32_t* __restrict__ gbloom) {
    extern __shared__ uint32_t sh[];
    const uint32_t nl = 1u << g.L;
    uint32_t*      cnt = sh;
    uint32_t*      blm = sh + nl;
    uint32_t       part, s, e;
    bool           single;
    if (!chunk_range(blockIdx.x, chunk_off, chunk_part, part_off, 1u << g.R, part, s, e, single)) return;
    if (fused_part(part_off, part)) return;  // k_bucket_local
    for (uint32_t i = threadIdx.x; i < 2 * nl; i += blockDim.x) sh[i] = 0;
    __syncthreads();
    const uint32_t lmask = nl - 1;
    constexpr int  kU    = 8;  // keys per thread loaded before any of them is counted
    for (uint32_t b0 = s; b0 < e; b0 += kU * blockDim.x) {
        int32_t key[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const uint32_t j = b0 + uint32_t(u) * blockDim.x + threadIdx.x;
            key[u]           = j < e ? __ldg(tkey + j) : 0;
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const uint32_t j   = b0 + uint32_t(u) * blockDim.x + threadIdx.x;
            const bool     ok  = j < e;
            const unsigned act = __ballot_sync(0xffffffffu, ok);
            if (ok) {
                const uint64_t h      = fib_hash(key[u]);
                const uint32_t local  = uint32_t(bucket_of(h, g.b)) & lmask;
                const int      leader = __ffs(act) - 1;
                bucket_add(cnt, local, act);
                // a warp of one heavy key ORs its tags once, not 32 times on one word
                if (__all_sync(act, local == __shfl_sync(act, local, leader))) {
                    const uint32_t all = __reduce_or_sync(act, bloom_mask(h));
                    if (int(threadIdx.x & 31) == leader) atomicOr(blm + local, all);
                } else {
                    atomicOr(blm + local, bloom_mask(h));
                }
            }
        }
    }
    __syncthreads();
    const uint64_t gb = uint64_t(part) << g.L;
    for (uint32_t i = threadIdx.x; i < nl; i += blockDim.x) {
        if (single) {
            gcnt[gb + i]   = cnt[i];
            gbloom[gb + i] = blm[i];
        } else if (cnt[i]) {
            atomicAdd(gcnt + gb + i, cnt[i]);
            atomicOr(gbloom + gb + i, blm[i]);
        }
    }
}

// 5. Directory words.  One block per partition; gcnt becomes the scatter cursor.
__global__ void __launch_bounds__(1024)
    k_bucket_dir(Geo g, const uint32_t* __restrict__ part_off, uint32_t* __restrict__ gcnt,
                 const uint32_t* __restrict__ gbloom, uint64_t* __restrict__ dir) {
    __shared__ uint32_t sm[33];
    const uint32_t part = blockIdx.x;
    const uint32_t nl   = 1u << g.L;
    const uint64_t gb   = uint64_t(part) << g.L;
    uint32_t       run  = part_off[part];
    if (fused_part(part_off, part)) return;  // k_bucket_local (also writes the sentinel word)
    if (part_off[part + 1] == run) {  // empty partition: all buckets empty
        for (uint32_t i = threadIdx.x; i < nl; i += blockDim.x) {
            dir[gb + i]  = uint64_t(run) << 16;
            gcnt[gb + i] = run;
        }
    } else {
        for (uint32_t base = 0; base < nl; base += blockDim.x) {
            const uint32_t i = base + threadIdx.x;
            const uint32_t c = i < nl ? gcnt[gb + i] : 0;
            uint32_t       tot;
            const uint32_t ex = block_exclusive_scan<uint32_t>(c, sm, &tot);
            if (i < nl) {
                const uint32_t start = run + ex;
                dir[gb + i]          = (uint64_t(start) << 16) | (gbloom[gb + i] & 0xffffu);
                gcnt[gb + i]         = start;
            }
            run += tot;
        }
    }
}

// 6. Final scatter into bucket order.
__global__ void __launch_bounds__(kThreads, 2)
    k_bucket_scatter(Geo g, const uint32_t* __restrict__ chunk_off, const uint32_t* __restrict__ chunk_part,
                     const uint32_t* __restrict__ part_off,
                     const int32_t* __restrict__ tkey, const uint32_t* __restrict__ trow,
                     uint32_t* __restrict__ cursor, int32_t* __restrict__ okey,
                     uint32_t* __restrict__ orow) {
    extern __shared__ uint32_t sh[];
    const uint32_t nl = 1u << g.L;
    uint32_t       part, s, e;
    bool           single;
    if (!chunk_range(blockIdx.x, chunk_off, chunk_part, part_off, 1u << g.R, part, s, e, single)) return;
    if (fused_part(part_off, part)) return;  // k_bucket_local
    for (uint32_t i = threadIdx.x; i < nl; i += blockDim.x) sh[i] = 0;
    __syncthreads();
    const uint32_t lmask = nl - 1;
    // a chunk is kSub tiles of kTile tuples: all are counted, then placed
    // (a one-tile chunk keeps its keys in registers between the two)
    constexpr int kSub = kChunk / kTile;
    int32_t       keys[kItems];
    for (uint32_t b0 = s; b0 < e; b0 += kTile) {
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const uint32_t j = b0 + uint32_t(k) * kThreads + threadIdx.x;
            keys[k]          = j < e ? __ldg(tkey + j) : 0;
            // the rows are stored after the counts: bring their lines into L1 now
            if (kSub == 1 && j < e) asm volatile("prefetch.global.L1 [%0];" ::"l"(trow + j));
        }
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const uint32_t j  = b0 + uint32_t(k) * kThreads + threadIdx.x;
            const bool     ok = j < e;
            const unsigned act = __ballot_sync(0xffffffffu, ok);
            if (ok) bucket_add(sh, uint32_t(bucket_of(fib_hash(keys[k]), g.b)) & lmask, act);
        }
    }
    __syncthreads();
    const uint64_t gb = uint64_t(part) << g.L;
    {
        // the thread's buckets (at most 2^kLocalBits / kThreads): every cursor
        // load or atomic issued before any result is stored
        constexpr int kPer = (1 << kLocalBits) / kThreads;
        uint32_t      c[kPer];
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            const uint32_t i = threadIdx.x + uint32_t(q) * kThreads;
            const uint32_t n = i < nl ? sh[i] : 0u;
            c[q]             = n == 0 ? 0u : (single ? cursor[gb + i] : atomicAdd(cursor + gb + i, n));
        }
#pragma unroll
        for (int q = 0; q < kPer; ++q) {
            const uint32_t i = threadIdx.x + uint32_t(q) * kThreads;
            if (i < nl && sh[i]) sh[i] = c[q];
        }
    }
    __syncthreads();
    for (uint32_t b0 = s; b0 < e; b0 += kTile) {
        uint32_t rows[kItems];
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const uint32_t j = b0 + uint32_t(k) * kThreads + threadIdx.x;
            if (kSub > 1) keys[k] = j < e ? __ldg(tkey + j) : 0;
            rows[k] = j < e ? __ldg(trow + j) : 0u;
        }
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const uint32_t j   = b0 + uint32_t(k) * kThreads + threadIdx.x;
            const bool     ok  = j < e;
            const unsigned act = __ballot_sync(0xffffffffu, ok);
            if (ok) {
                const uint32_t pos = bucket_add(sh, uint32_t(bucket_of(fib_hash(keys[k]), g.b)) & lmask, act);
                okey[pos]          = keys[k];
                orow[pos]          = rows[k];
            }
        }
    }
}

// 4-7 in one block for a partition of at most kFuseMax tuples: bucket counts
// and Bloom tags in shared memory, the directory words from one scan of the
// counts, then the tuples placed in bucket order in shared memory and stored
// with coalesced writes (scattered 4-byte stores would cost one L2 request
// each); the mixed bits come from neighbouring keys of the placed order.
// Larger partitions (Zipf-heavy keys) take the chunked kernels, which skip the
// partitions handled here.
constexpr int kLT = 1024;            // threads of k_bucket_local
constexpr int kLU = kFuseMax / kLT;  // tuples per thread of a partition it takes, at most
static_assert(kLU * kLT == int(kFuseMax), "a partition is one pass of the block");

__global__ void __launch_bounds__(kLT, 1)
    k_bucket_local(Geo g, const uint32_t* __restrict__ part_off, const int32_t* __restrict__ tkey,
                   const uint32_t* __restrict__ trow, uint64_t* __restrict__ dir, int32_t* __restrict__ okey,
                   uint32_t* __restrict__ orow, uint32_t* __restrict__ mixed, uint64_t* __restrict__ summary) {
    extern __shared__ uint32_t sh[];
    __shared__ uint32_t wsum[kLT / 32];
    const uint32_t nl    = 1u << g.L;
    const uint32_t lmask = nl - 1;
    const uint32_t P     = 1u << g.R;
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t nbw = (nl + 1) / 2, nmw = (nl + 31) / 32;
    uint32_t* cnt = sh;                 // nl: counts, then cursors
    uint32_t* blm = sh + nl;            // nbw words: two 16-bit Bloom tags each
    uint32_t* mix = sh + nl + nbw;      // nmw words of mixed bits
    int32_t*  sk  = reinterpret_cast<int32_t*>(mix + nmw);  // kFuseMax staged keys
    uint32_t* sr  = reinterpret_cast<uint32_t*>(sk + kFuseMax);        // and rows
    if (blockIdx.x == 0 && threadIdx.x == 0) dir[uint64_t(P) << g.L] = uint64_t(part_off[P]) << 16;
    for (uint32_t part = blockIdx.x; part < P; part += gridDim.x) {
        if (!fused_part(part_off, part)) continue;
        const uint32_t s = part_off[part], e = part_off[part + 1];
        const uint64_t gb = uint64_t(part) << g.L;
        for (uint32_t i = threadIdx.x; i < nl + nbw + nmw; i += blockDim.x) sh[i] = 0;
        __syncthreads();
        // the partition's keys, all loaded before any is counted (kLU per thread)
        int32_t key[kLU];
#pragma unroll
        for (int u = 0; u < kLU; ++u) {
            const uint32_t j = s + uint32_t(u) * kLT + threadIdx.x;
            key[u]           = j < e ? __ldg(tkey + j) : 0;
        }
        const int nu = int((e - s + kLT - 1) / kLT);  // passes of the block that hold tuples
        // counts and Bloom tags
#pragma unroll
        for (int u = 0; u < kLU; ++u) {
            if (u >= nu) break;
            const uint32_t j   = s + uint32_t(u) * kLT + threadIdx.x;
            const bool     ok  = j < e;
            const unsigned act = __ballot_sync(0xffffffffu, ok);
            if (ok) {
                const uint64_t h     = fib_hash(key[u]);
                const uint32_t local = uint32_t(bucket_of(h, g.b)) & lmask;
                bucket_add(cnt, local, act);
                atomicOr(blm + (local >> 1), bloom_mask(h) << (16 * (local & 1)));
            }
        }
        // the rows are placed after the scan: their loads overlap it
        uint32_t row[kLU];
#pragma unroll
        for (int u = 0; u < kLU; ++u) {
            const uint32_t j = s + uint32_t(u) * kLT + threadIdx.x;
            row[u]           = j < e ? __ldg(trow + j) : 0u;
        }
        __syncthreads();
        // exclusive scan of the counts: warp w scans segments of 32 counts
        // (lane i reads count 32 q + i: no bank conflicts), then the warps' totals
        const uint32_t nseg = (nl + 31) / 32, per_w = (nseg + kLT / 32 - 1) / (kLT / 32);
        uint32_t       wrun = 0;
        for (uint32_t q = warp * per_w; q < min(nseg, (warp + 1) * per_w); ++q) {
            const uint32_t i = 32 * q + lane;
            const uint32_t c = i < nl ? cnt[i] : 0u;
            wrun += warp_sum(c);
        }
        if (lane == 0) wsum[warp] = wrun;
        __syncthreads();
        uint32_t base = s;
        for (uint32_t w = 0; w < warp; ++w) base += wsum[w];
        for (uint32_t q = warp * per_w; q < min(nseg, (warp + 1) * per_w); ++q) {
            const uint32_t i   = 32 * q + lane;
            const uint32_t c   = i < nl ? cnt[i] : 0u;
            const uint32_t inc = warp_inclusive_scan(c);
            if (i < nl) {
                const uint32_t start = base + inc - c;
                cnt[i]               = start;
                dir[gb + i]          = (uint64_t(start) << 16) | ((blm[i >> 1] >> (16 * (i & 1))) & 0xffffu);
            }
            base += __shfl_sync(0xffffffffu, inc, 31);
        }
        __syncthreads();
        // place the tuples in bucket order
#pragma unroll
        for (int u = 0; u < kLU; ++u) {
            if (u >= nu) break;
            const uint32_t j   = s + uint32_t(u) * kLT + threadIdx.x;
            const bool     ok  = j < e;
            const unsigned act = __ballot_sync(0xffffffffu, ok);
            if (ok) {
                const uint32_t local = uint32_t(bucket_of(fib_hash(key[u]), g.b)) & lmask;
                const uint32_t q     = bucket_add(cnt, local, act) - s;
                sk[q]                = key[u];
                sr[q]                = row[u];
            }
        }
        __syncthreads();
        // coalesced stores; a bucket is mixed when two neighbours in it differ
        for (uint32_t q = threadIdx.x; q < e - s; q += blockDim.x) {
            const int32_t k = sk[q];
            okey[s + q]     = k;
            orow[s + q]     = sr[q];
            if (q > 0 && sk[q - 1] != k) {
                const uint32_t local = uint32_t(bucket_of(fib_hash(k), g.b)) & lmask;
                if ((uint32_t(bucket_of(fib_hash(sk[q - 1]), g.b)) & lmask) == local)
                    atomicOr(mix + (local >> 5), 1u << (local & 31));
            }
        }
        __syncthreads();
        // the partition's buckets are whole mixed words (2^L >= 32) or share one
        if (nl >= 32) {
            for (uint32_t i = threadIdx.x; i < nl / 32; i += blockDim.x) mixed[(gb >> 5) + i] = mix[i];
        } else if (threadIdx.x == 0 && mix[0]) {
            atomicOr(mixed + (gb >> 5), mix[0] << (gb & 31));
        }
        // bucket summaries: cnt[i] is now the end of bucket i, so bucket i
        // spans [end of bucket i - 1, cnt[i]); its first key is staged in sk
        for (uint32_t i = threadIdx.x; i < nl; i += blockDim.x) {
            const uint32_t b0  = i == 0 ? s : cnt[i - 1];
            const uint32_t len = cnt[i] - b0;
            summary[gb + i]    = len == 0 ? 0ull
                                          : make_summary(sk[b0 - s], (blm[i >> 1] >> (16 * (i & 1))) & 0xffffu, len,
                                                         (mix[i >> 5] >> (i & 31)) & 1u);
        }
        __syncthreads();
    }
}

// Bucket summaries of the partitions the chunked kernels built (the others
// come from k_bucket_local): one block per partition.
__global__ void __launch_bounds__(256)
    k_bucket_summary(Geo g, const uint32_t* __restrict__ part_off, const uint64_t* __restrict__ dir,
                     const int32_t* __restrict__ key, const uint32_t* __restrict__ mixed,
                     uint64_t* __restrict__ summary) {
    const uint32_t part = blockIdx.x;
    if (fused_part(part_off, part)) return;
    const uint32_t nl = 1u << g.L;
    const uint64_t gb = uint64_t(part) << g.L;
    for (uint32_t i = threadIdx.x; i < nl; i += blockDim.x) {
        const uint64_t p   = gb + i;
        const uint64_t d0  = __ldg(dir + p);
        const uint32_t b0  = uint32_t(d0 >> 16);
        const uint32_t len = uint32_t(__ldg(dir + p + 1) >> 16) - b0;
        summary[p] = len == 0 ? 0ull
                              : make_summary(__ldg(key + b0), uint32_t(d0) & 0xffffu, len,
                                             (__ldg(mixed + (p >> 5)) >> (p & 31)) & 1u);
    }
}

// 7. mixed[p] bit set when bucket p holds two different keys (chunks of the
//    partitions k_bucket_local does not take).
__global__ void __launch_bounds__(kThreads)
    k_bucket_mixed(Geo g, const uint32_t* __restrict__ chunk_off, const uint32_t* __restrict__ chunk_part,
                   const uint32_t* __restrict__ part_off,
                   const uint64_t* __restrict__ dir, const int32_t* __restrict__ key, uint32_t* __restrict__ mixed) {
    uint32_t part, s, e;
    bool     single;
    if (!chunk_range(blockIdx.x, chunk_off, chunk_part, part_off, 1u << g.R, part, s, e, single)) return;
    if (fused_part(part_off, part)) return;  // set by k_bucket_local
    // kMU tuples per thread at a time: keys, then directory words, then first keys
    constexpr int kMU = 8;
    for (uint32_t j0 = s + threadIdx.x; j0 < e; j0 += kMU * blockDim.x) {
        int32_t  k[kMU];
        uint32_t p[kMU], first[kMU];
#pragma unroll
        for (int u = 0; u < kMU; ++u) {
            const uint32_t j = j0 + u * blockDim.x;
            k[u]             = j < e ? key[j] : 0;
        }
#pragma unroll
        for (int u = 0; u < kMU; ++u) {
            p[u]     = uint32_t(bucket_of(fib_hash(k[u]), g.b));
            first[u] = j0 + u * blockDim.x < e ? uint32_t(__ldg(dir + p[u]) >> 16) : 0u;
        }
#pragma unroll
        for (int u = 0; u < kMU; ++u)
            if (j0 + u * blockDim.x < e && key[first[u]] != k[u]) atomicOr(mixed + (p[u] >> 5), 1u << (p[u] & 31));
    }
}

template <class K>
void prefer_shared(K kernel) {
    HJ_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 int(cudaSharedmemCarveoutMaxShared)));
}

uint32_t ceil_log2(uint64_t n) {
    uint32_t b = 0;
    while ((1ull << b) < n) ++b;
    return b;
}

int grid_for(uint64_t work, int threads, int per_sm = 4) {
    const uint64_t want = (work + threads - 1) / threads;
    return int(std::min<uint64_t>(std::max<uint64_t>(want, 1), uint64_t(num_sms()) * per_sm));
}

}  // namespace

void build_table(const KeyCol& kc, int dir_bits, int radix_bits, Table& t, uint64_t* scratch_host,
                 cudaStream_t st, int64_t n_valid, int dir_cap_bits) {
    t = Table{};
    const uint64_t n_upper = n_valid >= 0 ? uint64_t(n_valid) : kc.n;
    const uint32_t cap     = uint32_t(std::max(0, dir_cap_bits));
    const uint32_t b_upper = dir_bits >= 0 ? uint32_t(dir_bits)
                                           : std::min(cap, ceil_log2(std::max<uint64_t>(n_upper, 1)));
    // partition fan-out: the requested one, raised to what keeps a partition's
    // buckets within one shared-memory histogram (2^13) and capped at b
    const uint32_t R_min   = b_upper > kLocalBits ? b_upper - kLocalBits : 0;
    uint32_t       R       = radix_bits >= 0 ? std::max<uint32_t>(uint32_t(radix_bits), R_min) : R_min;
    R                      = std::min(R, b_upper);
    if (R > kMaxRadix) throw Error(HJ_ERR_INVALID, "build side too large for the radix partition");

    prefer_shared(k_part_hist);
    prefer_shared(k_part_scatter<1024>);
    prefer_shared(k_part_scatter<kThreads>);
    prefer_shared(k_bucket_count);
    prefer_shared(k_bucket_scatter);
    prefer_shared(k_bucket_local);
    unsigned long long* d_nvalid = dalloc_n<unsigned long long>(1, st);
    uint32_t*           part_cnt = nullptr;
    auto run_hist = [&](uint32_t r) {
        const uint32_t P = 1u << r;
        part_cnt         = dalloc_n<uint32_t>(P, st);
        HJ_CUDA(cudaMemsetAsync(part_cnt, 0, P * sizeof(uint32_t), st));
        HJ_CUDA(cudaMemsetAsync(d_nvalid, 0, sizeof(unsigned long long), st));
        const size_t smem = P * sizeof(uint32_t);
        if (smem > 48 * 1024)
            HJ_CUDA(cudaFuncSetAttribute(k_part_hist, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         int(smem)));
        k_part_hist<<<grid_for(kc.n, kThreads), kThreads, smem, st>>>(kc, r, part_cnt, d_nvalid);
        HJ_LAUNCH_CHECK();
        if (n_valid < 0) {
            readback(scratch_host, d_nvalid, sizeof(uint64_t), true, st);  // page-locked scratch
            HJ_CUDA(cudaStreamSynchronize(st));
        }
    };
    run_hist(R);
    const uint64_t nv = n_valid >= 0 ? uint64_t(n_valid) : scratch_host[0];
    if (nv == 0) {  // UnchainedHash with no tuples: no directory, every probe misses
        dfree(part_cnt, st);
        dfree(d_nvalid, st);
        return;
    }
    if (nv > 0xffffffffull) throw Error(HJ_ERR_INVALID, "more than 2^32 build tuples");
    const uint32_t b = dir_bits >= 0 ? uint32_t(dir_bits) : std::min(cap, ceil_log2(nv));
    if (R > b) {  // NULLs shrank the directory below the partition fan-out
        dfree(part_cnt, st);
        R = b;
        run_hist(R);
    }
    if (b - R > kLocalBits) throw Error(HJ_ERR_INVALID, "radix_bits too small for the directory");
    const Geo      g{b, R, b - R};
    const uint32_t P = 1u << R;

    uint32_t* part_off    = dalloc_n<uint32_t>(P + 1, st);
    uint32_t* part_cursor = dalloc_n<uint32_t>(P, st);
    uint32_t* chunk_off   = dalloc_n<uint32_t>(P + 1, st);
    // chunks of the partitions above kFuseMax tuples, at most
    const unsigned chunks_upper = unsigned((nv + kChunk - 1) / kChunk + nv / kFuseMax + 1);
    uint32_t*      chunk_part   = dalloc_n<uint32_t>(chunks_upper, st);
    k_part_offsets<<<1, 1024, 0, st>>>(part_cnt, P, part_off, part_cursor, chunk_off, chunk_part);
    HJ_LAUNCH_CHECK();

    int32_t*  tkey = dalloc_n<int32_t>(nv, st);
    uint32_t* trow = dalloc_n<uint32_t>(nv, st);
    {
        // 16384-row tiles (runs of about 8 items per partition at 2048
        // partitions) when the shared memory allows, else 8192-row tiles
        auto smem_for = [&](size_t tile) { return (2 * size_t(P) + 2 * tile) * sizeof(uint32_t) + tile * sizeof(uint16_t); };
        const size_t big = smem_for(size_t(1024) * kItems);
        if (big <= 200 * 1024) {
            HJ_CUDA(cudaFuncSetAttribute(k_part_scatter<1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(big)));
            k_part_scatter<1024><<<div_up(kc.n, 1024 * kItems), 1024, big, st>>>(kc, R, part_cursor, tkey, trow);
        } else {
            const size_t smem = smem_for(kTile);
            HJ_CUDA(cudaFuncSetAttribute(k_part_scatter<kThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         int(smem)));
            k_part_scatter<kThreads><<<div_up(kc.n, kTile), kThreads, smem, st>>>(kc, R, part_cursor, tkey, trow);
        }
        HJ_LAUNCH_CHECK();
    }

    const uint64_t nb     = 1ull << b;
    t.dir_bits            = b;
    t.n_tuples            = nv;
    t.dir                 = dalloc_n<uint64_t>(nb + 1, st);
    t.keys                = dalloc_n<int32_t>(nv, st);
    t.rows                = dalloc_n<uint32_t>(nv, st);
    t.mixed               = dalloc_n<uint32_t>((nb + 31) / 32, st);
    t.summary             = dalloc_n<uint64_t>(nb, st);
    uint32_t* gcnt        = dalloc_n<uint32_t>(nb, st);
    uint32_t* gbloom      = dalloc_n<uint32_t>(nb, st);
    HJ_CUDA(cudaMemsetAsync(t.mixed, 0, ((nb + 31) / 32) * sizeof(uint32_t), st));
    k_bucket_zero<<<P, 256, 0, st>>>(g, chunk_off, part_off, gcnt, gbloom);
    HJ_LAUNCH_CHECK();

    {
        const size_t smem = 2 * (size_t(1) << g.L) * sizeof(uint32_t);
        HJ_CUDA(cudaFuncSetAttribute(k_bucket_count, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(smem)));
        k_bucket_count<<<chunks_upper, kThreads, smem, st>>>(g, chunk_off, chunk_part, part_off, tkey, gcnt, gbloom);
        HJ_LAUNCH_CHECK();
    }
    k_bucket_dir<<<P, 1024, 0, st>>>(g, part_off, gcnt, gbloom, t.dir);
    HJ_LAUNCH_CHECK();
    {
        const size_t nl   = size_t(1) << g.L;
        const size_t smem = (nl + (nl + 1) / 2 + (nl + 31) / 32 + 2 * size_t(kFuseMax)) * sizeof(uint32_t);
        HJ_CUDA(cudaFuncSetAttribute(k_bucket_local, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        k_bucket_local<<<std::min<uint32_t>(P, uint32_t(num_sms())), kLT, smem, st>>>(g, part_off, tkey, trow, t.dir,
                                                                                t.keys, t.rows, t.mixed,
                                                                                t.summary);
        HJ_LAUNCH_CHECK();
    }
    {
        const size_t smem = (size_t(1) << g.L) * sizeof(uint32_t);
        HJ_CUDA(cudaFuncSetAttribute(k_bucket_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(smem)));
        k_bucket_scatter<<<chunks_upper, kThreads, smem, st>>>(g, chunk_off, chunk_part, part_off, tkey, trow, gcnt,
                                                              t.keys, t.rows);
        HJ_LAUNCH_CHECK();
    }
    k_bucket_mixed<<<chunks_upper, kThreads, 0, st>>>(g, chunk_off, chunk_part, part_off, t.dir, t.keys, t.mixed);
    HJ_LAUNCH_CHECK();
    k_bucket_summary<<<P, 256, 0, st>>>(g, part_off, t.dir, t.keys, t.mixed, t.summary);
    HJ_LAUNCH_CHECK();

    for (void* p : {(void*)d_nvalid, (void*)part_cnt, (void*)part_off, (void*)part_cursor,
                    (void*)chunk_off, (void*)chunk_part, (void*)tkey, (void*)trow, (void*)gcnt, (void*)gbloom})
        dfree(p, st);
}

void free_table(Table& t, cudaStream_t st) {
    for (void* p : {(void*)t.dir, (void*)t.keys, (void*)t.rows, (void*)t.mixed, (void*)t.summary})
        if (p) dfree(p, st);
    t = Table{};
}

}  // namespace hj
