// Probe of the unchained table on the GPU.
//
// Semantics of UnchainedHash::probe (include/unchained.h:220-246 of the
// reference) applied to a column of probe keys, as the reference's probe
// workers do (src/execute.cpp:111-165): NULL keys never match (:127-129),
// Bloom early-reject on the bucket's tag, then every tuple of the bucket with
// an equal key is a match.
//
// Count pass (k_probe_count).  A block walks tiles of 1984 probe rows (one
// dense INT32 page).  The tile's keys are staged in shared memory by bulk
// asynchronous copies (TMA) while the previous tile is probed: whole pages
// for a dense column read in place, else the decoded int32 / value_t array.
// Per key the probe issues ONE global load, the bucket's 8-byte summary
// (first key, Bloom tag, length, mixed flag; hj_common.cuh), eight keys per
// thread in flight:
//   miss     empty bucket, or the Bloom tag rejects the key;
//   uniform  bucket of one key (mixed flag clear): the key matches every tuple
//            of the bucket or none, decided by the first key; the hit is
//            (probe row, bucket, length from the summary) -- no further load;
//   mixed    bucket of several keys: a bucket of at most min(light_max, 32)
//            tuples is compared by the probing thread itself, which records
//            the matching tuples as a 32-bit mask over the bucket and stages
//            the hit with the uniform ones; larger buckets go to a list
//            counted by a warp or block per hit (k_mixed_count*).
// A hit stays in the registers of the thread that found it.  Within a warp,
// hits are ordered round by round (the eight keys of a thread are eight
// rounds), so a ballot ranks a round's hits into consecutive list slots
// (coalesced stores) and a warp scan of their match counts gives their first
// output rows.  The kernel keeps its shared memory small (the two key
// stages): the rest of the SM's 256 KB stays L1, where the summaries of
// frequently probed buckets are cached.  Per tile,
// ONE global 64-bit atomic reserves both the block's list slots (high word)
// and its output rows (low word), so list order and output order agree and no
// device-wide prefix sum is needed (the reference's per-thread work-stealing
// counter becomes this per-block reservation).
//
// Write pass.  k_write_uniform walks the OUTPUT positions in chunks of
// 32 x G per warp (G outputs per thread, option probe_group): a chunk's hits
// are located by the chunk map (k_chunk_first) and staged in the warp's own
// shared memory, a uniform hit's bucket start is read from its directory
// word, each thread finds its hit by binary search and reads build rows
// rows[start + k] consecutively, and writes its G row ids of every output
// stream as one 16-byte store (a warp covers 512 contiguous bytes).  Warps
// synchronise only with themselves.  Work is balanced by output rows, so one
// Zipf-heavy key with millions of tuples spreads over all SMs.
// Mixed hits follow the uniform ones.  Every match writes one row id per
// requested output stream, composed through the sides' row-id vectors (late
// materialisation).
#include <algorithm>

#include "hj_block.cuh"
#include "hj_common.cuh"
#include "hj_kernels.h"
#include "hj_tma.cuh"

namespace hj {

namespace {

constexpr int      kPT        = 256;                    // threads of the count kernel
constexpr int      kStep      = 8;                      // rows per thread in flight
constexpr uint32_t kTileRows  = uint32_t(kDenseRows);   // 1984 rows per staged tile (one page)
static_assert(kTileRows <= uint32_t(kPT) * kStep, "a tile is one pass of the count kernel");
static_assert(kPT * kStep == 2048 && kPT == 256, "the staged-hit scan covers 8 warps x 8 rows of 32");
constexpr uint32_t kUncounted = 0xffffffffu;            // mixed hit still to be counted
constexpr uint32_t kMixedWarpMax = 4096;                // mixed buckets up to this size: one warp each
constexpr uint32_t kWaitPolls    = 1u << 20;            // bound of a staging wait (mbarrier polls)

__host__ __device__ __forceinline__ uint64_t umin64(uint64_t a, uint64_t b) { return a < b ? a : b; }

enum KeySrc : int { kSrcPages = 0, kSrcPlain = 1, kSrcTagged = 2, kSrcGather = 3 };

struct ProbeTab {
    const uint64_t* dir;
    const uint64_t* sum;
    const int32_t*  keys;
    const uint32_t* rows;
    uint32_t        b;
};

struct Lists {
    // staged hits, in output order: hit h owns output rows [off[h], off[h + 1])
    // (the last up to the staged total); mask 0: the whole bucket sp matches,
    // else the tuples sp + i for the set bits i of mask
    uint32_t *u_row, *u_sp, *u_off, *u_mask;
    uint32_t *m_row, *m_s, *m_e, *m_cnt;    // mixed hits: tuples [s, e) compared with m_key
    int32_t*  m_key;
    // 0 staged hits << 32 | staged matches mod 2^32, 1 mixed hits, 2 staged
    // matches, 3 mixed matches, 4 staging waits that gave up (an error)
    unsigned long long* ctr;
};

struct Outs {
    int    n;
    RidOut o[kMaxRidOut];
};

__device__ __forceinline__ void emit(const Outs& outs, uint64_t pos, uint32_t prow, uint32_t brow) {
#pragma unroll 4
    for (int i = 0; i < outs.n; ++i) {
        const RidOut& o = outs.o[i];
        const uint32_t x = o.side == 0 ? prow : brow;
        o.dst[pos]       = o.src ? __ldg(o.src + x) : x;
    }
}

// Bytes of one staged tile of each key source (0: no staging).
__host__ __device__ constexpr uint32_t stage_bytes(int src) {
    return src == kSrcPages    ? uint32_t(kPage)
         : src == kSrcPlain    ? kTileRows * 4u
         : src == kSrcTagged   ? kTileRows * 8u
                               : 0u;
}

// Issues the bulk copy of tile `tile` of the key column into `dst`; returns
// the rows of the tile that the copy covers (the rest are read directly).
template <int SRC>
__device__ __forceinline__ uint32_t stage_tile(const KeyCol& pk, uint64_t tile, uint8_t* dst, uint64_t* bar) {
    const uint64_t r0    = tile * kTileRows;
    const uint32_t nrows = uint32_t(umin64(kTileRows, pk.n - r0));
    uint32_t       bytes = 0, covered = 0;
    const void*    src   = nullptr;
    if (SRC == kSrcPages) {
        bytes   = kPage;
        src     = pk.col.pages + tile * kPage;
        covered = nrows;
    } else if (SRC == kSrcPlain) {
        covered = nrows & ~3u;
        bytes   = covered * 4u;
        src     = pk.col.plain + r0;
    } else {
        covered = nrows & ~1u;
        bytes   = covered * 8u;
        src     = pk.col.tagged + r0;
    }
    fence_proxy_async_smem();
    mbar_arrive_expect(bar, bytes);
    if (bytes) bulk_load(dst, src, bytes, bar);
    return covered;
}

// Key of tile row i (row r of the key column); false for NULL.
template <int SRC>
__device__ __forceinline__ bool tile_key(const KeyCol& pk, const uint8_t* stage, uint32_t covered, uint32_t i,
                                         uint64_t r, int32_t& key) {
    if (SRC == kSrcPages) {
        key = reinterpret_cast<const int32_t*>(stage + 4)[i];
        return true;
    } else if (SRC == kSrcPlain) {
        key = i < covered ? reinterpret_cast<const int32_t*>(stage)[i] : __ldg(pk.col.plain + r);
        return bit_valid(pk.col.valid, r);
    } else if (SRC == kSrcTagged) {
        const uint64_t t = i < covered ? reinterpret_cast<const uint64_t*>(stage)[i] : __ldg(pk.col.tagged + r);
        key              = int32_t(uint32_t(t));
        return (t >> 62) == 1;
    } else {
        const uint64_t row = pk.rid ? uint64_t(__ldg(pk.rid + r)) : r;
        bool           ok  = int_get(pk.col, row, key);
        // a filtered scan read raw: rows failing its predicate never match
        if (pk.filt.n && ok) ok = filt_pass(pk.filt, row);
        return ok;
    }
}

template <int SRC>
__global__ void __launch_bounds__(kPT, 4)
    k_probe_count(ProbeTab T, KeyCol pk, int light_max, Lists Ls, uint64_t ntiles) {
    extern __shared__ __align__(128) uint8_t dyn[];
    constexpr uint32_t SB  = stage_bytes(SRC);
    constexpr int      kW  = kPT / 32;
    uint8_t*           stg = dyn;  // 2 stages
    __shared__ uint64_t bar[2];
    __shared__ uint32_t s_cov;
    // per warp: staged hits and their matches (mod 2^32), turned into the
    // warp's bases within the tile by thread 0; exact match counts
    __shared__ uint32_t           s_wh[kW], s_wc[kW];
    __shared__ unsigned long long s_wx[kW];
    __shared__ uint32_t           s_hb, s_ob;
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt   = (1u << lane) - 1;
    uint32_t       cov0 = 0, cov1 = 0;   // thread 0: rows each stage's copy covers
    uint32_t       iss0 = 0, iss1 = 0;   // thread 0: copies issued into each stage
    bool           gave_up = false;  // a staging wait ran out of polls (an error)
    if (SRC != kSrcGather && threadIdx.x == 0) {
        mbar_init(&bar[0]);
        mbar_init(&bar[1]);
    }
    __syncthreads();
    if (SRC != kSrcGather && threadIdx.x == 0 && uint64_t(blockIdx.x) < ntiles) {
        cov0 = stage_tile<SRC>(pk, blockIdx.x, stg, &bar[0]);
        iss0 = 1;
    }
    const uint32_t small = min(uint32_t(light_max), 32u);
    uint32_t       k     = 0;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++k) {
        const uint32_t st = k & 1;
        if (SRC != kSrcGather) {
            // the other stage was last read before the previous iteration's
            // barriers: refill it with the next tile now
            const uint64_t next = tile + gridDim.x;
            if (threadIdx.x == 0 && next < ntiles) {
                const uint32_t c = stage_tile<SRC>(pk, next, stg + (st ^ 1) * SB, &bar[st ^ 1]);
                if (st) { cov0 = c; ++iss0; } else { cov1 = c; ++iss1; }
            }
            gave_up = !mbar_wait_bounded(&bar[st], (k >> 1) & 1, kWaitPolls);
            // thread 0 holds the covered counts; every thread needs this tile's
            if (threadIdx.x == 0) s_cov = st ? cov1 : cov0;
        }
        // one barrier that also tells every thread whether any gave up
        if (__syncthreads_or(gave_up)) {
            gave_up = true;
            break;
        }
        const uint32_t cov   = SRC != kSrcGather ? s_cov : 0u;
        const uint64_t r0    = tile * kTileRows;
        const uint32_t nrows = uint32_t(umin64(kTileRows, pk.n - r0));
        const uint8_t* stage = stg + st * SB;
        int32_t  key[kStep];
        bool     ok[kStep];
        uint64_t w[kStep];
#pragma unroll
        for (int it = 0; it < kStep; ++it) {
            const uint32_t i = uint32_t(it) * kPT + threadIdx.x;
            ok[it]           = false;
            key[it]          = 0;
            w[it]            = 0;
            if (i < nrows) ok[it] = tile_key<SRC>(pk, stage, cov, i, r0 + i, key[it]);
            // through L1: with skewed probe keys the hot buckets' summaries stay there
            if (ok[it]) w[it] = __ldg(T.sum + bucket_of(fib_hash(key[it]), T.b));
        }
        // classify: 0 miss, 1 hit staged here, 2 mixed bucket counted later.
        // Directory words are read only for mixed buckets and for uniform
        // buckets whose length saturated the summary's field.
        uint32_t s[kStep], L[kStep], msk[kStep];
        int      cls[kStep];
#pragma unroll
        for (int it = 0; it < kStep; ++it) {
            const uint64_t h = fib_hash(key[it]);
            L[it]            = sum_len(w[it]);
            msk[it]          = 0;
            cls[it]          = 0;
            if (ok[it] && L[it] != 0) {
                if (!sum_mixed(w[it])) {
                    // a bucket of one key: its first key decides exactly (a matching
                    // key's Bloom bits are always in the bucket's tag)
                    cls[it] = sum_head(w[it]) == key[it] ? 1 : 0;
                } else {
                    const uint32_t m = bloom_mask(h);
                    cls[it]          = (sum_bloom(w[it]) & m) == m ? 2 : 0;
                }
            }
            const uint64_t p = bucket_of(h, T.b);
            s[it]            = uint32_t(p);
            uint32_t e       = 0;
            if (cls[it] == 2 || (cls[it] == 1 && L[it] == kSumLenMax)) {
                const uint32_t b0 = uint32_t(__ldg(T.dir + p) >> 16);
                L[it]             = uint32_t(__ldg(T.dir + p + 1) >> 16) - b0;
                if (cls[it] == 2) s[it] = b0;
                e = b0 + L[it];
            }
            // a small mixed bucket: compared here, its matches as a mask
            if (cls[it] == 2 && L[it] <= small) {
                uint32_t mm = 0;
                for (uint32_t q = 0; q < L[it]; ++q) mm |= uint32_t(__ldg(T.keys + s[it] + q) == key[it]) << q;
                msk[it] = mm;
                L[it]   = __popc(mm);
                cls[it] = mm ? 1 : 0;
            }
            // larger mixed buckets: counted later; rare, so warp-aggregated
            // global atomics
            const unsigned bal = __ballot_sync(0xffffffffu, cls[it] == 2);
            if (bal) {
                unsigned long long q0 = 0;
                if (lane == 0) q0 = atomicAdd(Ls.ctr + 1, (unsigned long long)__popc(bal));
                q0 = __shfl_sync(0xffffffffu, q0, 0);
                if (cls[it] == 2) {
                    const uint64_t q = q0 + __popc(bal & lt);
                    Ls.m_row[q]      = uint32_t(r0 + uint32_t(it) * kPT + threadIdx.x);
                    Ls.m_s[q]        = s[it];
                    Ls.m_e[q]        = e;
                    Ls.m_key[q]      = key[it];
                    Ls.m_cnt[q]      = kUncounted;
                }
            }
        }
        // the warp's hits in (it, lane) order, so the hits of one round are
        // consecutive list slots (coalesced stores): per round a ballot ranks
        // them and a warp scan of their counts gives their first output rows
        // within the warp -- a ballot suffices when no hit has more than one
        // match (32-bit prefix sums; the exact total is summed beside them)
        uint32_t           nh = 0, nc = 0;
        unsigned long long lx = 0;
        uint32_t           slot[kStep], oo[kStep];
        static_assert(kStep % 2 == 0, "rounds are scanned in pairs");
#pragma unroll
        for (int it = 0; it < kStep; it += 2) {
            const bool     h0 = cls[it] == 1, h1 = cls[it + 1] == 1;
            const uint32_t c0 = h0 ? L[it] : 0u, c1 = h1 ? L[it + 1] : 0u;
            const unsigned b0 = __ballot_sync(0xffffffffu, h0), b1 = __ballot_sync(0xffffffffu, h1);
            const uint32_t r0 = __popc(b0 & lt), r1 = __popc(b1 & lt);
            slot[it]          = nh + r0;
            slot[it + 1]      = nh + __popc(b0) + r1;
            nh += __popc(b0) + __popc(b1);
            if (!__any_sync(0xffffffffu, (c0 | c1) > 1)) {  // one match per hit: the ranks
                oo[it]     = nc + r0;
                oo[it + 1] = nc + __popc(b0) + r1;
                nc += __popc(b0) + __popc(b1);
            } else if (__all_sync(0xffffffffu, (c0 | c1) < 2048)) {
                // both rounds in one scan of 16-bit halves (a half sums to < 2^16)
                const uint32_t v   = c0 | (c1 << 16);
                const uint32_t inc = warp_inclusive_scan<uint32_t>(v);
                const uint32_t tot = __shfl_sync(0xffffffffu, inc, 31);
                const uint32_t ex  = inc - v;
                oo[it]             = nc + (ex & 0xffffu);
                oo[it + 1]         = nc + (tot & 0xffffu) + (ex >> 16);
                nc += (tot & 0xffffu) + (tot >> 16);
            } else {
                const uint32_t i0 = warp_inclusive_scan<uint32_t>(c0);
                oo[it]            = nc + i0 - c0;
                nc += __shfl_sync(0xffffffffu, i0, 31);
                const uint32_t i1 = warp_inclusive_scan<uint32_t>(c1);
                oo[it + 1]        = nc + i1 - c1;
                nc += __shfl_sync(0xffffffffu, i1, 31);
            }
            lx += uint64_t(c0) + c1;
        }
        const unsigned long long nx = warp_sum<unsigned long long>(lx);
        if (lane == 0) {
            s_wh[warp] = nh;
            s_wc[warp] = nc;
            s_wx[warp] = nx;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t           hs = 0, cs = 0;
            unsigned long long xs = 0;
#pragma unroll
            for (int q = 0; q < kW; ++q) {
                const uint32_t h = s_wh[q], c = s_wc[q];
                s_wh[q] = hs;
                s_wc[q] = cs;
                hs += h;
                cs += c;
                xs += s_wx[q];
            }
            const unsigned long long base = hs ? atomicAdd(Ls.ctr + 0, (uint64_t(hs) << 32) + cs) : 0ull;
            if (xs) atomicAdd(Ls.ctr + 2, xs);
            s_hb = uint32_t(base >> 32);
            s_ob = uint32_t(base);
        }
        __syncthreads();
        const uint32_t hb = s_hb + s_wh[warp], ob = s_ob + s_wc[warp];
#pragma unroll
        for (int it = 0; it < kStep; ++it) {
            if (cls[it] == 1) {
                const uint32_t q = hb + slot[it];
                Ls.u_row[q]      = uint32_t(r0 + uint32_t(it) * kPT + threadIdx.x);
                Ls.u_sp[q]       = s[it];
                Ls.u_off[q]      = ob + oo[it];
                Ls.u_mask[q]     = msk[it];
            }
        }
    }
    if (SRC != kSrcGather) {
        // a block that gave up waits (bounded) for the copies it issued, so no
        // copy lands in shared memory after the block has exited
        if (gave_up && threadIdx.x == 0) {
            atomicAdd(Ls.ctr + 4, 1ull);
            if (iss0) mbar_wait_bounded(&bar[0], (iss0 - 1) & 1, kWaitPolls);
            if (iss1) mbar_wait_bounded(&bar[1], (iss1 - 1) & 1, kWaitPolls);
        }
    }
}

// Mixed hits still uncounted: a warp each for buckets of up to kMixedWarpMax
// tuples, a block each above.
__global__ void __launch_bounds__(256) k_mixed_count_warp(ProbeTab T, Lists Ls) {
    const uint64_t n    = Ls.ctr[1];
    const unsigned lane = threadIdx.x & 31;
    const uint64_t gw   = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw   = (uint64_t(gridDim.x) * blockDim.x) >> 5;
    unsigned long long acc = 0;
    for (uint64_t q = gw; q < n; q += nw) {
        if (Ls.m_cnt[q] != kUncounted) continue;
        const uint32_t s = Ls.m_s[q], e = Ls.m_e[q];
        if (e - s > kMixedWarpMax) continue;
        const int32_t key = Ls.m_key[q];
        uint32_t      c   = 0;
        for (uint32_t i = s + lane; i < e; i += 32) c += __ldg(T.keys + i) == key;
        c = warp_sum(c);
        if (lane == 0) {
            Ls.m_cnt[q] = c;
            acc += c;
        }
    }
    if (lane == 0 && acc) atomicAdd(Ls.ctr + 3, acc);
}

__global__ void __launch_bounds__(512) k_mixed_count(ProbeTab T, Lists Ls) {
    __shared__ unsigned long long s_red[33];
    const uint64_t n   = Ls.ctr[1];
    uint64_t       acc = 0;
    for (uint64_t q = blockIdx.x; q < n; q += gridDim.x) {
        const uint32_t s = Ls.m_s[q], e = Ls.m_e[q];
        if (e - s <= kMixedWarpMax || Ls.m_cnt[q] != kUncounted) continue;
        const int32_t  key = Ls.m_key[q];
        unsigned long long c = 0;
        for (uint32_t k = s + threadIdx.x; k < e; k += blockDim.x) c += __ldg(T.keys + k) == key;
        unsigned long long tot;
        block_exclusive_scan<unsigned long long>(c, s_red, &tot);
        if (threadIdx.x == 0) {
            Ls.m_cnt[q] = uint32_t(tot);
            acc += tot;
        }
    }
    if (threadIdx.x == 0 && acc) atomicAdd(Ls.ctr + 3, (unsigned long long)acc);
}

// Largest h < n with off[h] <= x (off non-decreasing, off[0] = 0).
__device__ __forceinline__ uint64_t hit_of(const uint32_t* __restrict__ off, uint64_t n, uint64_t x) {
    uint64_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint64_t mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= x) lo = mid;
        else                       hi = mid;
    }
    return lo;
}

// chunk_first[c] = the uniform hit holding output position c * chunk.
__global__ void k_chunk_first(const uint32_t* __restrict__ off, uint64_t n_u, uint64_t nchunks, uint32_t chunk,
                              uint32_t* __restrict__ chunk_first) {
    const uint64_t c = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c < nchunks) chunk_first[c] = uint32_t(hit_of(off, n_u, c * chunk));
}

// Outputs of one warp's chunk in k_write_uniform<G>, and the per-warp
// shared memory: the chunk's hits (at most chunk + 1: every hit holds at least
// one output, plus the hit that starts at the next chunk's first position):
// relative starts (chunk + 2), probe rows, tuple starts, unclamped relative
// starts and masks.
constexpr uint32_t warp_chunk(int G) { return 32u * uint32_t(G); }
constexpr size_t   write_uniform_smem(int G) { return 8 * 5 * (size_t(warp_chunk(G)) + 2) * sizeof(uint32_t); }

// Index of the k-th set bit of m (k < popcount(m)).
__device__ __forceinline__ uint32_t nth_bit(uint32_t m, uint32_t k) {
    for (uint32_t i = 0; i < k; ++i) m &= m - 1;
    return uint32_t(__ffs(m) - 1);
}

// G consecutive values to dst (16-byte aligned runs of 4 as vector stores).
template <int G>
__device__ __forceinline__ void store_run(uint32_t* dst, const uint32_t (&v)[G], bool vec, uint64_t pol) {
    if (G >= 4 && vec) {
#pragma unroll
        for (int i = 0; i < G; i += 4)
            st_hint(reinterpret_cast<uint4*>(dst + i), make_uint4(v[i], v[i + 1], v[i + 2], v[i + 3]), pol);
    } else if (G == 2 && vec) {
        *reinterpret_cast<uint2*>(dst) = make_uint2(v[0], v[G > 1 ? 1 : 0]);
    } else {
#pragma unroll
        for (int i = 0; i < G; ++i) dst[i] = v[i];
    }
}

template <int G>
__global__ void __launch_bounds__(256, G <= 4 ? 6 : (G <= 8 ? 4 : 2))
    k_write_uniform(ProbeTab T, Lists Ls, uint64_t n_u, const uint32_t* __restrict__ chunk_first, uint64_t total,
                    Outs outs) {
    const uint32_t* __restrict__ off = Ls.u_off;
    constexpr uint32_t CH = warp_chunk(G);
    constexpr uint32_t NW = CH + 2;
    extern __shared__ __align__(16) uint32_t wsh[];
    const unsigned lane  = threadIdx.x & 31;
    uint32_t*      s_rel  = wsh + (threadIdx.x >> 5) * 5 * NW;  // hit starts relative to the chunk, clamped to [0, len]
    uint32_t*      s_pr   = s_rel + NW;                         // probe row of each hit
    uint32_t*      s_s    = s_pr + NW;                          // first tuple of each hit's bucket
    uint32_t*      s_orel = s_s + NW;                           // hit start - chunk start, mod 2^32
    uint32_t*      s_msk  = s_orel + NW;                        // match mask (0: every tuple)
    // vector stores need every stream 16-byte aligned (engine buffers are)
    bool vec = true;
    for (int oi = 0; oi < outs.n; ++oi) vec &= (reinterpret_cast<uintptr_t>(outs.o[oi].dst) & 15) == 0;
    const uint64_t nchunks = (total + CH - 1) / CH;
    const uint64_t nw      = (uint64_t(gridDim.x) * blockDim.x) >> 5;
    const uint64_t stream  = l2_evict_first();  // row ids are written once, read later in order
    for (uint64_t c = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; c < nchunks; c += nw) {
        const uint64_t o0  = c * CH;
        const uint32_t len = uint32_t(umin64(CH, total - o0));
        const uint64_t h0  = chunk_first ? __ldg(chunk_first + c) : hit_of(off, n_u, o0);
        const uint64_t h1  = c + 1 < nchunks ? (chunk_first ? __ldg(chunk_first + c + 1) : hit_of(off, n_u, o0 + CH))
                                             : n_u - 1;
        const uint32_t nh  = uint32_t(h1 - h0) + 1;  // hits h0 .. h0 + nh - 1 cover the chunk
        if (nh == 1) {
            // the whole chunk inside one hit (the usual case for a Zipf-heavy
            // key): lane 0 reads the hit, every lane takes consecutive matches
            uint32_t orel = 0, m = 0, t0 = 0, prow = 0;
            if (lane == 0) {
                orel           = uint32_t(uint64_t(__ldg(off + h0)) - o0);  // mod 2^32: the hit may start earlier
                m              = __ldg(Ls.u_mask + h0);
                const uint32_t sp = __ldg(Ls.u_sp + h0);
                prow           = __ldg(Ls.u_row + h0);
                t0             = m ? sp : uint32_t(__ldg(T.dir + sp) >> 16);
            }
            orel = __shfl_sync(0xffffffffu, orel, 0);
            m    = __shfl_sync(0xffffffffu, m, 0);
            t0   = __shfl_sync(0xffffffffu, t0, 0);
            prow = __shfl_sync(0xffffffffu, prow, 0);
            const uint32_t q0 = lane * G;
            if (q0 < len) {
                uint32_t brow[G];
#pragma unroll
                for (int i = 0; i < G; ++i) {
                    const uint32_t idx = q0 + i - orel;  // match number within the hit
                    brow[i]            = q0 + i < len ? __ldg(T.rows + t0 + (m ? nth_bit(m, idx) : idx)) : 0u;
                }
                const bool full = q0 + G <= len;
                for (int oi = 0; oi < outs.n; ++oi) {
                    const RidOut o = outs.o[oi];
                    uint32_t     v[G];
                    const uint32_t pv = o.side == 0 ? (o.src ? __ldg(o.src + prow) : prow) : 0u;
#pragma unroll
                    for (int i = 0; i < G; ++i)
                        v[i] = o.side == 0 ? pv : ((o.src && q0 + i < len) ? __ldg(o.src + brow[i]) : brow[i]);
                    uint32_t* dst = o.dst + o0 + q0;
                    if (full) {
                        store_run<G>(dst, v, vec, stream);
                    } else {
#pragma unroll
                        for (int i = 0; i < G; ++i)
                            if (q0 + i < len) dst[i] = v[i];
                    }
                }
            }
            continue;
        }
        for (uint32_t q = lane; q <= nh; q += 32) {
            const uint64_t hq  = h0 + q;
            const uint64_t o   = hq < n_u ? uint64_t(__ldg(off + hq)) : total;
            const uint64_t rel = o > o0 ? o - o0 : 0;
            s_rel[q]           = uint32_t(umin64(rel, len));
            if (q < nh) {
                const uint32_t m  = __ldg(Ls.u_mask + hq);
                const uint32_t sp = __ldg(Ls.u_sp + hq);
                s_pr[q]   = __ldg(Ls.u_row + hq);
                // a uniform hit names its bucket: the start is its directory word's
                s_s[q]    = m ? sp : uint32_t(__ldg(T.dir + sp) >> 16);
                s_orel[q] = uint32_t(o - o0);
                s_msk[q]  = m;
            }
        }
        __syncwarp();
        const uint32_t q0 = lane * G;
        if (q0 < len) {
            uint32_t prow[G], brow[G];
            uint32_t lo = 0, hi = nh;  // largest k with s_rel[k] <= q0
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (s_rel[mid] <= q0) lo = mid;
                else                  hi = mid;
            }
            uint32_t k = lo;
#pragma unroll
            for (int i = 0; i < G; ++i) {
                const uint32_t q = q0 + i;
                prow[i] = brow[i] = 0;
                if (q < len) {
                    while (s_rel[k + 1] <= q) ++k;
                    const uint32_t idx = q - s_orel[k];  // match number within the hit
                    const uint32_t m   = s_msk[k];
                    prow[i]            = s_pr[k];
                    brow[i]            = __ldg(T.rows + s_s[k] + (m ? nth_bit(m, idx) : idx));
                }
            }
            const bool full = q0 + G <= len;
            for (int oi = 0; oi < outs.n; ++oi) {
                const RidOut o = outs.o[oi];
                uint32_t     v[G];
#pragma unroll
                for (int i = 0; i < G; ++i) {
                    const uint32_t x = o.side == 0 ? prow[i] : brow[i];
                    v[i]             = (o.src && q0 + i < len) ? __ldg(o.src + x) : x;
                }
                uint32_t* dst = o.dst + o0 + q0;
                if (full) {
                    store_run<G>(dst, v, vec, stream);
                } else {
#pragma unroll
                    for (int i = 0; i < G; ++i)
                        if (q0 + i < len) dst[i] = v[i];
                }
            }
        }
        __syncwarp();  // the next chunk's hits overwrite this warp's shared memory
    }
}

__global__ void __launch_bounds__(256)
    k_write_mixed_warp(ProbeTab T, Lists Ls, const uint64_t* __restrict__ mixed_off, uint64_t base_pos,
                       Outs outs) {
    const uint64_t n    = Ls.ctr[1];
    const unsigned lane = threadIdx.x & 31;
    const uint64_t gw   = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw   = (uint64_t(gridDim.x) * blockDim.x) >> 5;
    for (uint64_t q = gw; q < n; q += nw) {
        const uint32_t s = Ls.m_s[q], e = Ls.m_e[q];
        if (e - s > kMixedWarpMax) continue;
        const uint32_t prow = Ls.m_row[q];
        const int32_t  key  = Ls.m_key[q];
        uint64_t       pos  = base_pos + mixed_off[q];
        for (uint32_t b = s; b < e; b += 32) {
            const uint32_t k   = b + lane;
            const bool     m   = k < e && __ldg(T.keys + k) == key;
            const unsigned bal = __ballot_sync(0xffffffffu, m);
            if (m) emit(outs, pos + __popc(bal & ((1u << lane) - 1)), prow, __ldg(T.rows + k));
            pos += __popc(bal);
        }
    }
}

__global__ void __launch_bounds__(512)
    k_write_mixed(ProbeTab T, Lists Ls, const uint64_t* __restrict__ mixed_off, uint64_t base_pos,
                  Outs outs) {
    __shared__ uint32_t sm[33];
    const uint64_t n = Ls.ctr[1];
    for (uint64_t q = blockIdx.x; q < n; q += gridDim.x) {
        const uint32_t s = Ls.m_s[q], e = Ls.m_e[q], prow = Ls.m_row[q];
        if (e - s <= kMixedWarpMax) continue;  // done by k_write_mixed_warp
        const int32_t  key = Ls.m_key[q];
        uint64_t       pos = base_pos + mixed_off[q];
        for (uint32_t b = s; b < e; b += blockDim.x) {
            const uint32_t k = b + threadIdx.x;
            const bool     m = k < e && __ldg(T.keys + k) == key;
            uint32_t       tot;
            const uint32_t r = block_exclusive_scan<uint32_t>(m ? 1u : 0u, sm, &tot);
            if (m) emit(outs, pos + r, prow, __ldg(T.rows + k));
            pos += tot;
        }
    }
}

ProbeTab tab_of(const Table& t) { return ProbeTab{t.dir, t.summary, t.keys, t.rows, t.dir_bits}; }

// How the count kernel reads a probe column's keys.  A bulk copy needs a
// 16-byte aligned source; tiles start at multiples of 3968 rows (of 16-byte
// multiples for every form), so the column's base address decides.  Columns
// at other addresses (a caller's array at an arbitrary 4-byte offset) are
// read by direct loads.
int key_source(const KeyCol& pk) {
    auto aligned = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
    if (pk.rid || pk.filt.n) return kSrcGather;
    if (pk.col.tagged) return aligned(pk.col.tagged) ? kSrcTagged : kSrcGather;
    if (pk.col.plain) return aligned(pk.col.plain) ? kSrcPlain : kSrcGather;
    return aligned(pk.col.pages) ? kSrcPages : kSrcGather;
}

template <int SRC>
void launch_count_src(const ProbeTab& T, const KeyCol& pk, int light_max, const Lists& L, cudaStream_t st) {
    const uint64_t ntiles = (pk.n + kTileRows - 1) / kTileRows;
    const size_t   smem   = std::max<size_t>(16, 2 * size_t(stage_bytes(SRC)));
    HJ_CUDA(cudaFuncSetAttribute(k_probe_count<SRC>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    // shared memory for the resident blocks only; the rest of the unified
    // L1 / shared memory caches bucket summaries
    HJ_CUDA(cudaFuncSetAttribute(k_probe_count<SRC>, cudaFuncAttributePreferredSharedMemoryCarveout, 30));
    // resident blocks walk the tiles (each prefetching its next tile)
    int per_sm = 0;
    HJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_probe_count<SRC>, kPT, smem));
    const uint64_t grid = std::max<uint64_t>(1, std::min<uint64_t>(ntiles, uint64_t(num_sms()) * std::max(1, per_sm)));
    k_probe_count<SRC><<<unsigned(grid), kPT, smem, st>>>(T, pk, light_max, L, ntiles);
    HJ_LAUNCH_CHECK();
}

// Count kernels over a probe column: uniform and mixed lists, counters in L.ctr.
void launch_count(const ProbeTab& T, const KeyCol& pk, int light_max, const Lists& L, cudaStream_t st) {
    switch (key_source(pk)) {
    case kSrcPages: launch_count_src<kSrcPages>(T, pk, light_max, L, st); break;
    case kSrcPlain: launch_count_src<kSrcPlain>(T, pk, light_max, L, st); break;
    case kSrcTagged: launch_count_src<kSrcTagged>(T, pk, light_max, L, st); break;
    default: launch_count_src<kSrcGather>(T, pk, light_max, L, st); break;
    }
}

// After the counters were read back into host[0..4]: when the count pass
// listed large mixed buckets (host[1] > 0), counts their matches and reads
// their total back into host[3] (one more host wait; most tables have none).
void count_mixed(const ProbeTab& T, const Lists& L, uint64_t* host, cudaStream_t st) {
    if (host[1] == 0) return;
    k_mixed_count_warp<<<num_sms() * 4, 256, 0, st>>>(T, L);
    HJ_LAUNCH_CHECK();
    k_mixed_count<<<num_sms() * 2, 512, 0, st>>>(T, L);
    HJ_LAUNCH_CHECK();
    readback(host + 3, L.ctr + 3, sizeof(uint64_t), true, st);  // page-locked scratch
    HJ_CUDA(cudaStreamSynchronize(st));
}

// Outputs per thread of the uniform writer from option probe_group.
int writer_items(int group) {
    switch (group) {
    case 1: return 1;
    case 2: return 2;
    case 4: return 4;
    case 16:
    case 32: return 16;  // 32 would take 196 KB of shared memory per block
    default: return 8;
    }
}

template <int G>
void launch_uniform_g(const ProbeTab& T, const Lists& L, uint64_t n_u, const uint32_t* chunk_first, uint64_t total,
                      const Outs& outs, cudaStream_t st) {
    const size_t smem = write_uniform_smem(G);
    HJ_CUDA(cudaFuncSetAttribute(k_write_uniform<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int per_sm = 0;
    HJ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_write_uniform<G>, 256, smem));
    const uint64_t nchunks = (total + warp_chunk(G) - 1) / warp_chunk(G);
    const uint64_t grid    = std::max<uint64_t>(1, std::min<uint64_t>((nchunks + 7) / 8, uint64_t(num_sms()) * std::max(1, per_sm)));
    k_write_uniform<G><<<unsigned(grid), 256, smem, st>>>(T, L, n_u, chunk_first, total, outs);
    HJ_LAUNCH_CHECK();
}

// The staged hits' matches (total of them, < 2^32) into the output streams.
void launch_uniform(int G, const ProbeTab& T, const Lists& L, uint64_t n_u, const uint32_t* chunk_first,
                    uint64_t total, const Outs& outs, cudaStream_t st) {
    if (total > 0xffffffffull) throw Error(HJ_ERR_INVALID, "join result exceeds 2^32 rows");
    switch (G) {
    case 1: launch_uniform_g<1>(T, L, n_u, chunk_first, total, outs, st); break;
    case 2: launch_uniform_g<2>(T, L, n_u, chunk_first, total, outs, st); break;
    case 4: launch_uniform_g<4>(T, L, n_u, chunk_first, total, outs, st); break;
    case 16: launch_uniform_g<16>(T, L, n_u, chunk_first, total, outs, st); break;
    default: launch_uniform_g<8>(T, L, n_u, chunk_first, total, outs, st); break;
    }
}

void launch_mixed_writers(const ProbeTab& T, const Lists& L, const uint64_t* mixed_off, uint64_t base_pos,
                          const Outs& outs, cudaStream_t st) {
    k_write_mixed_warp<<<num_sms() * 8, 256, 0, st>>>(T, L, mixed_off, base_pos, outs);
    HJ_LAUNCH_CHECK();
    k_write_mixed<<<num_sms() * 2, 512, 0, st>>>(T, L, mixed_off, base_pos, outs);
    HJ_LAUNCH_CHECK();
}

void check_staging(const uint64_t* host_ctr) {
    if (host_ctr[4])
        throw Error(HJ_ERR_DEVICE_STATUS, "probe: " + std::to_string(host_ctr[4])
                                              + " blocks gave up waiting for their staged key tiles");
}

}  // namespace

struct ProbePlan {
    Lists     ls{};
    uint64_t  cap     = 0;
    uint64_t  n_u = 0, n_m = 0, tot_u = 0, tot_m = 0;
    uint64_t* host    = nullptr;  // pinned readback of the counters (owned by the caller)
    int       group   = 8;
};

uint64_t probe_count(const Table& t, const KeyCol& pk, const ProbeParams& prm, ProbePlan** out,
                     cudaStream_t st) {
    auto* pp  = new ProbePlan();
    *out      = pp;
    pp->group = prm.group;
    if (t.n_tuples == 0 || pk.n == 0) return 0;
    if (pk.n > 0xffffffffull) throw Error(HJ_ERR_INVALID, "more than 2^32 probe rows");
    const uint64_t n = pk.n;
    pp->cap          = n;
    Lists& L         = pp->ls;
    L.u_row = dalloc_n<uint32_t>(n, st);
    L.u_sp  = dalloc_n<uint32_t>(n, st);
    L.u_off = dalloc_n<uint32_t>(n, st);
    L.u_mask = dalloc_n<uint32_t>(n, st);
    L.m_row = dalloc_n<uint32_t>(n, st);
    L.m_s   = dalloc_n<uint32_t>(n, st);
    L.m_e   = dalloc_n<uint32_t>(n, st);
    L.m_cnt = dalloc_n<uint32_t>(n, st);
    L.m_key = dalloc_n<int32_t>(n, st);
    L.ctr   = dalloc_n<unsigned long long>(8, st);
    HJ_CUDA(cudaMemsetAsync(L.ctr, 0, 8 * sizeof(unsigned long long), st));
    launch_count(tab_of(t), pk, prm.light_max, L, st);
    if (prm.after_count) prm.after_count();
    pp->host = prm.pinned;
    readback(pp->host, L.ctr, 5 * sizeof(uint64_t), true, st);  // page-locked scratch
    HJ_CUDA(cudaStreamSynchronize(st));
    check_staging(pp->host);
    count_mixed(tab_of(t), L, pp->host, st);
    pp->n_u   = pp->host[0] >> 32;
    pp->n_m   = pp->host[1];
    pp->tot_u = pp->host[2];
    pp->tot_m = pp->host[3];
    return pp->tot_u + pp->tot_m;
}

void probe_write(const Table& t, const KeyCol& pk, ProbePlan* pp, const RidOut* ro, int nout,
                 cudaStream_t st) {
    (void)pk;
    if (nout > kMaxRidOut) throw Error(HJ_ERR_INVALID, "too many output row-id streams");
    Outs outs{};
    outs.n = nout;
    for (int i = 0; i < nout; ++i) outs.o[i] = ro[i];
    if (pp->cap == 0 || nout == 0) return;
    const ProbeTab T = tab_of(t);
    Lists&         L = pp->ls;
    if (pp->n_u) {
        const int      G       = writer_items(pp->group);
        const uint64_t chunk   = warp_chunk(G);
        const uint64_t nchunks = (pp->tot_u + chunk - 1) / chunk;
        uint32_t*      cfirst  = dalloc_n<uint32_t>(nchunks + 1, st);
        k_chunk_first<<<div_up(nchunks, 256), 256, 0, st>>>(L.u_off, pp->n_u, nchunks, uint32_t(chunk), cfirst);
        HJ_LAUNCH_CHECK();
        launch_uniform(G, T, L, pp->n_u, cfirst, pp->tot_u, outs, st);
        dfree(cfirst, st);
    }
    if (pp->n_m) {
        uint64_t* off = dalloc_n<uint64_t>(pp->n_m + 1, st);
        scan_exclusive_u32_to_u64(L.m_cnt, off, pp->n_m, st);
        launch_mixed_writers(T, L, off, pp->tot_u, outs, st);
        dfree(off, st);
    }
}

namespace {

// Bump carve-out of 256-byte-aligned pieces from a caller-owned buffer.
struct Carve {
    uint8_t* p;
    size_t   used = 0;
    template <class T>
    T* take(uint64_t n) {
        T* r = reinterpret_cast<T*>(p + used);
        used += (n * sizeof(T) + 255) & ~size_t(255);
        return r;
    }
};

}  // namespace

size_t probe_scratch_bytes(uint64_t n) {
    const uint64_t tmp = scan_tmp_words(n) + 1;
    return 256 + 9 * ((4 * n + 255) & ~uint64_t(255)) + ((8 * (n + 1) + 255) & ~uint64_t(255))
         + ((8 * tmp + 255) & ~uint64_t(255));
}

int probe_into_scratch(const Table& t, const KeyCol& pk, const ProbeParams& prm, uint8_t* scratch,
                       size_t scratch_bytes, uint32_t* out_probe, uint32_t* out_build, uint64_t capacity,
                       uint64_t* num_matches, cudaStream_t st) {
    *num_matches = 0;
    if (t.n_tuples == 0 || pk.n == 0) return HJ_OK;
    const uint64_t n = pk.n;
    if (probe_scratch_bytes(n) > scratch_bytes) throw Error(HJ_ERR_INVALID, "probe scratch too small");
    Lists     L{};
    uint64_t *m_off, *tmp;
    Carve     c{scratch};
    L.ctr   = c.take<unsigned long long>(8);
    L.u_row = c.take<uint32_t>(n);
    L.u_sp  = c.take<uint32_t>(n);
    L.u_off = c.take<uint32_t>(n);
    L.u_mask = c.take<uint32_t>(n);
    L.m_row = c.take<uint32_t>(n);
    L.m_s   = c.take<uint32_t>(n);
    L.m_e   = c.take<uint32_t>(n);
    L.m_cnt = c.take<uint32_t>(n);
    L.m_key = c.take<int32_t>(n);
    m_off   = c.take<uint64_t>(n + 1);
    tmp     = c.take<uint64_t>(scan_tmp_words(n) + 1);
    // the scratch keeps the previous call's contents: the counters restart at zero
    HJ_CUDA(cudaMemsetAsync(L.ctr, 0, 8 * sizeof(unsigned long long), st));
    const ProbeTab T = tab_of(t);
    launch_count(T, pk, prm.light_max, L, st);
    uint64_t* h = prm.pinned;
    readback(h, L.ctr, 5 * sizeof(uint64_t), true, st);  // page-locked scratch
    HJ_CUDA(cudaStreamSynchronize(st));
    check_staging(h);
    count_mixed(T, L, h, st);
    const uint64_t n_u = h[0] >> 32, n_m = h[1], tot_u = h[2], total = h[2] + h[3];
    *num_matches = total;
    if (total > capacity) return HJ_ERR_CAPACITY;
    if (total == 0) return HJ_OK;
    Outs outs{};
    outs.n    = 2;
    outs.o[0] = RidOut{0, nullptr, out_probe};
    outs.o[1] = RidOut{1, nullptr, out_build};
    if (n_u) {
        // no chunk map (its size would follow the match count): each chunk
        // finds its first hit by binary search
        launch_uniform(writer_items(prm.group), T, L, n_u, nullptr, tot_u, outs, st);
    }
    if (n_m) {
        scan_exclusive_u32_to_u64_into(L.m_cnt, m_off, n_m, tmp, st);
        launch_mixed_writers(T, L, m_off, tot_u, outs, st);
    }
    return HJ_OK;
}

void probe_free(ProbePlan* pp, cudaStream_t st) {
    if (!pp) return;
    Lists& L = pp->ls;
    for (void* p : {(void*)L.u_row, (void*)L.u_sp, (void*)L.u_off, (void*)L.u_mask, (void*)L.m_row, (void*)L.m_s, (void*)L.m_e,
                    (void*)L.m_cnt, (void*)L.m_key, (void*)L.ctr})
        if (p) dfree(p, st);
    delete pp;
}

}  // namespace hj
