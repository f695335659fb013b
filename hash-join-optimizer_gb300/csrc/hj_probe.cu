// Probe of the unchained table on the GPU.
//
// Semantics of UnchainedHash::probe (include/unchained.h:220-246 of the
// reference) applied to a column of probe keys, as the reference's probe
// workers do (src/execute.cpp:111-165): NULL keys never match (:127-129),
// Bloom early-reject on the directory word, then every tuple of the bucket
// with an equal key is a match.
//
// Count pass (k_probe_count): each block walks 2048-row tiles.  A probe key
// reads its directory word, rejects on the Bloom tag, and classifies the hit:
//   light  bucket of <= light_max tuples (or a single tuple): counted by key
//          compare; staged in shared memory via warp ballot/popc and flushed
//          with ONE global atomic per tile (the reference's per-thread
//          work-stealing counter becomes this per-block reservation);
//   big    larger bucket whose tuples all carry one key (the per-bucket
//          "mixed" bit is clear): the whole bucket matches or nothing does,
//          so the count is the bucket size without reading it;
//   mixed  larger bucket with several keys: counted by a whole block
//          (k_mixed_count).
// Write pass: prefix sums of the counts give each hit its output slot; light
// hits are expanded by groups of `group` threads, big hits in 16K-tuple units
// spread over all SMs (one Zipf-heavy key can own millions of tuples), mixed
// hits by a block each.  Every match writes one row id per requested output
// stream, composed through the sides' row-id vectors (late materialisation).
#include <algorithm>

#include "hj_block.cuh"
#include "hj_common.cuh"
#include "hj_kernels.h"

namespace hj {

namespace {

constexpr int      kPT      = 256;
constexpr int      kPI      = 8;
constexpr int      kPTile   = kPT * kPI;
constexpr uint32_t kSplit   = 2048;   // tuples per big-hit work unit (one warp each)

struct ProbeTab {
    const uint64_t* dir;
    const int32_t*  keys;
    const uint32_t* rows;
    const uint32_t* mixed;
    uint32_t        b;
};

struct Lists {
    uint32_t *l_row, *l_s, *l_cnt;
    int32_t*  l_key;
    uint32_t *b_row, *b_s, *b_e;
    uint32_t *m_row, *m_s, *m_e, *m_cnt;
    int32_t*  m_key;
    unsigned long long* ctr;  // 0 n_light, 1 n_big, 2 n_mixed, 3 tot_light, 4 tot_big, 5 tot_mixed
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

__global__ void __launch_bounds__(kPT)
    k_probe_count(ProbeTab T, KeyCol pk, int light_max, Lists Ls, uint64_t ntiles) {
    __shared__ uint32_t s_row[kPTile], s_s[kPTile], s_cnt[kPTile];
    __shared__ int32_t  s_key[kPTile];
    __shared__ uint32_t s_n, s_base;
    __shared__ unsigned long long s_red[33];
    const unsigned lane = threadIdx.x & 31;
    uint64_t       tot_light = 0, tot_big = 0;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        if (threadIdx.x == 0) s_n = 0;
        __syncthreads();
        // The lookups of a thread's kPI keys are issued phase by phase (keys,
        // then directory words, then bucket heads) so that up to kPI
        // independent memory accesses per thread are in flight.
        int32_t  key[kPI];
        bool     ok[kPI];
        uint64_t w[kPI];
#pragma unroll
        for (int it = 0; it < kPI; ++it) {
            const uint64_t j = tile * kPTile + uint64_t(it) * kPT + threadIdx.x;
            ok[it]           = false;
            key[it]          = 0;
            if (j < pk.n) {
                const uint64_t row = pk.rid ? uint64_t(__ldg(pk.rid + j)) : j;
                ok[it]             = int_get(pk.col, row, key[it]);
                // a filtered scan read raw: rows failing its predicate never match
                if (pk.filt.n && ok[it]) ok[it] = filt_pass(pk.filt, row);
            }
        }
#pragma unroll
        for (int it = 0; it < kPI; ++it) {
            w[it] = 0;
            if (ok[it]) {
                const uint64_t h = fib_hash(key[it]);
                const uint64_t wd = __ldg(T.dir + bucket_of(h, T.b));
                const uint32_t m  = bloom_mask(h);
                w[it]             = (uint32_t(wd) & m) == m ? wd : 0;  // 0: rejected by the Bloom tag
                ok[it]            = w[it] != 0;
            }
        }
        uint32_t ends[kPI], heads[kPI], mixw[kPI];
#pragma unroll
        for (int it = 0; it < kPI; ++it) {
            ends[it] = heads[it] = mixw[it] = 0;
            if (ok[it]) {
                const uint64_t p = bucket_of(fib_hash(key[it]), T.b);
                ends[it]         = uint32_t(__ldg(T.dir + p + 1) >> 16);
                heads[it]        = uint32_t(__ldg(T.keys + uint32_t(w[it] >> 16)));
                mixw[it]         = __ldg(T.mixed + (p >> 5)) >> (p & 31);
            }
        }
#pragma unroll
        for (int it = 0; it < kPI; ++it) {
            const uint64_t j   = tile * kPTile + uint64_t(it) * kPT + threadIdx.x;
            int            cls = 0;  // 0 miss, 1 light, 2 big, 3 mixed
            uint32_t       c = 0, s = 0, e = 0;
            const int32_t  k = key[it];
            if (ok[it]) {
                s                 = uint32_t(w[it] >> 16);
                e                 = ends[it];
                const uint32_t L  = e - s;
                const int32_t  k0 = int32_t(heads[it]);
                if (L == 1) {
                    c   = k0 == k;
                    cls = c ? 1 : 0;
                } else if (!(mixw[it] & 1u)) {
                    c   = k0 == k ? L : 0;
                    cls = c ? (L <= uint32_t(light_max) ? 1 : 2) : 0;
                } else if (L <= uint32_t(light_max)) {
                    for (uint32_t q = s; q < e; ++q) c += __ldg(T.keys + q) == k;
                    cls = c ? 1 : 0;
                } else {
                    cls = 3;
                }
            }
            const int32_t key = k;
            // light: stage in shared memory
            {
                const unsigned bal = __ballot_sync(0xffffffffu, cls == 1);
                uint32_t       base = 0;
                if (lane == 0 && bal) base = atomicAdd(&s_n, uint32_t(__popc(bal)));
                base = __shfl_sync(0xffffffffu, base, 0);
                if (cls == 1) {
                    const uint32_t q = base + __popc(bal & ((1u << lane) - 1));
                    s_row[q]         = uint32_t(j);
                    s_s[q]           = s;
                    s_cnt[q]         = c;
                    s_key[q]         = key;
                    tot_light += c;
                }
            }
            // big / mixed: rare, warp-aggregated global atomics
            {
                const unsigned bal = __ballot_sync(0xffffffffu, cls == 2);
                if (bal) {
                    unsigned long long base = 0;
                    if (lane == 0) base = atomicAdd(Ls.ctr + 1, (unsigned long long)__popc(bal));
                    base = __shfl_sync(0xffffffffu, base, 0);
                    if (cls == 2) {
                        const uint64_t q = base + __popc(bal & ((1u << lane) - 1));
                        Ls.b_row[q]      = uint32_t(j);
                        Ls.b_s[q]        = s;
                        Ls.b_e[q]        = e;
                        tot_big += c;
                    }
                }
            }
            {
                const unsigned bal = __ballot_sync(0xffffffffu, cls == 3);
                if (bal) {
                    unsigned long long base = 0;
                    if (lane == 0) base = atomicAdd(Ls.ctr + 2, (unsigned long long)__popc(bal));
                    base = __shfl_sync(0xffffffffu, base, 0);
                    if (cls == 3) {
                        const uint64_t q = base + __popc(bal & ((1u << lane) - 1));
                        Ls.m_row[q]      = uint32_t(j);
                        Ls.m_s[q]        = s;
                        Ls.m_e[q]        = e;
                        Ls.m_key[q]      = key;
                    }
                }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) s_base = uint32_t(atomicAdd(Ls.ctr + 0, (unsigned long long)s_n));
        __syncthreads();
        const uint32_t nst = s_n, gb = s_base;
        for (uint32_t q = threadIdx.x; q < nst; q += blockDim.x) {
            Ls.l_row[gb + q] = s_row[q];
            Ls.l_s[gb + q]   = s_s[q];
            Ls.l_cnt[gb + q] = s_cnt[q];
            Ls.l_key[gb + q] = s_key[q];
        }
        __syncthreads();
    }
    unsigned long long t1, t2;
    block_exclusive_scan<unsigned long long>(tot_light, s_red, &t1);
    block_exclusive_scan<unsigned long long>(tot_big, s_red, &t2);
    if (threadIdx.x == 0) {
        if (t1) atomicAdd(Ls.ctr + 3, t1);
        if (t2) atomicAdd(Ls.ctr + 4, t2);
    }
}

// Grid of the count pass: up to 8 blocks of 256 threads per SM, looping over
// the tiles (measured faster than a register-capped single resident wave).
int probe_count_grid(uint64_t ntiles) {
    return int(std::max<uint64_t>(1, std::min<uint64_t>(ntiles, uint64_t(num_sms()) * 8)));
}

__global__ void __launch_bounds__(512) k_mixed_count(ProbeTab T, Lists Ls) {
    __shared__ unsigned long long s_red[33];
    const uint64_t n   = Ls.ctr[2];
    uint64_t       acc = 0;
    for (uint64_t q = blockIdx.x; q < n; q += gridDim.x) {
        const uint32_t s = Ls.m_s[q], e = Ls.m_e[q];
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
    if (threadIdx.x == 0 && acc) atomicAdd(Ls.ctr + 5, (unsigned long long)acc);
}

__global__ void k_big_units(const uint32_t* __restrict__ b_s, const uint32_t* __restrict__ b_e,
                            uint64_t n, uint32_t* __restrict__ units, uint32_t* __restrict__ lens) {
    const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t L = b_e[i] - b_s[i];
    lens[i]          = L;
    units[i]         = (L + kSplit - 1) / kSplit;
}

template <int G>
__global__ void __launch_bounds__(256)
    k_write_light(ProbeTab T, Lists Ls, uint64_t n_light, const uint64_t* __restrict__ off, Outs outs) {
    const unsigned lane = threadIdx.x & 31;
    const unsigned grp  = lane / G, gl = lane % G;
    const unsigned gmask = G == 32 ? 0xffffffffu : ((1u << G) - 1) << (grp * G);
    const uint64_t warp   = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = (uint64_t(gridDim.x) * blockDim.x) >> 5;
    constexpr int  HPW    = 32 / G;  // hits per warp step
    for (uint64_t hb = warp * HPW; hb < n_light; hb += nwarps * HPW) {
        const uint64_t h    = hb + grp;
        const bool     have = h < n_light;
        uint32_t       s = 0, L = 0, prow = 0;
        int32_t        key = 0;
        uint64_t       pos = 0;
        bool mixed = false;
        if (have) {
            s    = Ls.l_s[h];
            prow = Ls.l_row[h];
            key  = Ls.l_key[h];
            pos  = off[h];
            // a bucket of one key matches whole: its length is the count (the
            // mixed bitmap, 1 bit per bucket, stays in L2); a mixed bucket's end
            // is the next directory word's start
            const uint64_t p = bucket_of(fib_hash(key), T.b);
            mixed            = (__ldg(T.mixed + (p >> 5)) >> (p & 31)) & 1u;
            L                = mixed ? uint32_t(__ldg(T.dir + p + 1) >> 16) - s : Ls.l_cnt[h];
        }
        for (uint32_t k0 = 0; __any_sync(0xffffffffu, have && k0 < L); k0 += G) {
            const uint32_t k   = s + k0 + gl;
            const bool     in  = have && k0 + gl < L;
            const uint32_t row = in ? __ldg(T.rows + k) : 0u;  // loaded beside the key
            const bool     m   = in && (!mixed || __ldg(T.keys + k) == key);
            const unsigned bl  = __ballot_sync(0xffffffffu, m) & gmask;
            if (m) emit(outs, pos + __popc(bl & ((1u << lane) - 1)), prow, row);
            pos += __popc(bl);
        }
    }
}

// unit_hit[u] = the big hit that work unit u belongs to.
__global__ void k_unit_map(const uint64_t* __restrict__ unit_off, uint64_t n_big, uint32_t* __restrict__ unit_hit) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t h = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; h < n_big; h += stride)
        for (uint64_t u = unit_off[h]; u < unit_off[h + 1]; ++u) unit_hit[u] = uint32_t(h);
}

__global__ void __launch_bounds__(256)
    k_write_big(ProbeTab T, Lists Ls, uint64_t n_big, const uint64_t* __restrict__ unit_off,
                const uint32_t* __restrict__ unit_hit, const uint64_t* __restrict__ big_off, uint64_t base_pos,
                Outs outs) {
    // one warp per unit: most big hits are a few hundred tuples, so a whole
    // block per unit would leave most of its lanes idle
    const uint64_t nunits = unit_off[n_big];
    const unsigned lane   = threadIdx.x & 31;
    const uint64_t gw     = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw     = (uint64_t(gridDim.x) * blockDim.x) >> 5;
    for (uint64_t u = gw; u < nunits; u += nw) {
        uint64_t h;
        if (unit_hit) {
            h = unit_hit[u];
        } else {  // no map: largest h with unit_off[h] <= u
            uint64_t lo = 0, hi = n_big;
            while (hi - lo > 1) {
                const uint64_t mid = (lo + hi) >> 1;
                if (unit_off[mid] <= u) lo = mid;
                else                    hi = mid;
            }
            h = lo;
        }
        const uint64_t sub  = u - unit_off[h];
        const uint32_t s0   = Ls.b_s[h] + uint32_t(sub) * kSplit;
        const uint32_t e0   = min(Ls.b_e[h], s0 + kSplit);
        const uint32_t prow = Ls.b_row[h];
        const uint64_t pos0 = base_pos + big_off[h] + sub * kSplit;
        // four loads per lane in flight, then their outputs
        for (uint32_t k0 = s0; k0 < e0; k0 += 128) {
            uint32_t r[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t k = k0 + 32u * q + lane;
                r[q]             = k < e0 ? __ldg(T.rows + k) : 0u;
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t k = k0 + 32u * q + lane;
                if (k < e0) emit(outs, pos0 + (k - s0), prow, r[q]);
            }
        }
    }
}

constexpr uint32_t kMixedWarpMax = 4096;  // mixed buckets up to this size: one warp each

__global__ void __launch_bounds__(256)
    k_write_mixed_warp(ProbeTab T, Lists Ls, const uint64_t* __restrict__ mixed_off, uint64_t base_pos,
                       Outs outs) {
    const uint64_t n    = Ls.ctr[2];
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
    const uint64_t n = Ls.ctr[2];
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

ProbeTab tab_of(const Table& t) { return ProbeTab{t.dir, t.keys, t.rows, t.mixed, t.dir_bits}; }

}  // namespace

struct ProbePlan {
    Lists     ls{};
    uint64_t  cap     = 0;
    uint64_t  n_light = 0, n_big = 0, n_mixed = 0;
    uint64_t  tot_light = 0, tot_big = 0, tot_mixed = 0;
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
    L.l_row = dalloc_n<uint32_t>(n, st);
    L.l_s   = dalloc_n<uint32_t>(n, st);
    L.l_cnt = dalloc_n<uint32_t>(n, st);
    L.l_key = dalloc_n<int32_t>(n, st);
    L.b_row = dalloc_n<uint32_t>(n, st);
    L.b_s   = dalloc_n<uint32_t>(n, st);
    L.b_e   = dalloc_n<uint32_t>(n, st);
    L.m_row = dalloc_n<uint32_t>(n, st);
    L.m_s   = dalloc_n<uint32_t>(n, st);
    L.m_e   = dalloc_n<uint32_t>(n, st);
    L.m_cnt = dalloc_n<uint32_t>(n, st);
    L.m_key = dalloc_n<int32_t>(n, st);
    L.ctr   = dalloc_n<unsigned long long>(8, st);
    HJ_CUDA(cudaMemsetAsync(L.ctr, 0, 8 * sizeof(unsigned long long), st));
    const ProbeTab T      = tab_of(t);
    const uint64_t ntiles = (n + kPTile - 1) / kPTile;
    const int      grid   = probe_count_grid(ntiles);
    k_probe_count<<<grid, kPT, 0, st>>>(T, pk, prm.light_max, L, ntiles);
    HJ_LAUNCH_CHECK();
    k_mixed_count<<<num_sms() * 2, 512, 0, st>>>(T, L);
    HJ_LAUNCH_CHECK();
    if (prm.after_count) prm.after_count();
    pp->host = prm.pinned;
    readback(pp->host, L.ctr, 6 * sizeof(uint64_t), true, st);  // page-locked scratch
    HJ_CUDA(cudaStreamSynchronize(st));
    pp->n_light   = pp->host[0];
    pp->n_big     = pp->host[1];
    pp->n_mixed   = pp->host[2];
    pp->tot_light = pp->host[3];
    pp->tot_big   = pp->host[4];
    pp->tot_mixed = pp->host[5];
    return pp->tot_light + pp->tot_big + pp->tot_mixed;
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
    if (pp->n_light) {
        uint64_t* off = dalloc_n<uint64_t>(pp->n_light + 1, st);
        scan_exclusive_u32_to_u64(L.l_cnt, off, pp->n_light, st);
        const int grid = int(std::min<uint64_t>(div_up(pp->n_light, 256), uint64_t(num_sms()) * 16));
        switch (pp->group) {
        case 1: k_write_light<1><<<grid, 256, 0, st>>>(T, L, pp->n_light, off, outs); break;
        case 4: k_write_light<4><<<grid, 256, 0, st>>>(T, L, pp->n_light, off, outs); break;
        case 32: k_write_light<32><<<grid, 256, 0, st>>>(T, L, pp->n_light, off, outs); break;
        default: k_write_light<8><<<grid, 256, 0, st>>>(T, L, pp->n_light, off, outs); break;
        }
        HJ_LAUNCH_CHECK();
        dfree(off, st);
    }
    if (pp->n_big) {
        uint32_t* units    = dalloc_n<uint32_t>(pp->n_big, st);
        uint32_t* lens     = dalloc_n<uint32_t>(pp->n_big, st);
        uint64_t* unit_off = dalloc_n<uint64_t>(pp->n_big + 1, st);
        uint64_t* big_off  = dalloc_n<uint64_t>(pp->n_big + 1, st);
        k_big_units<<<div_up(pp->n_big, 256), 256, 0, st>>>(L.b_s, L.b_e, pp->n_big, units, lens);
        HJ_LAUNCH_CHECK();
        scan_exclusive_u32_to_u64(units, unit_off, pp->n_big, st);
        scan_exclusive_u32_to_u64(lens, big_off, pp->n_big, st);
        // every big hit has >= 1 unit and units = ceil(len / kSplit) <= 1 + len / kSplit
        const uint64_t max_units = pp->n_big + pp->tot_big / kSplit + 1;
        uint32_t*      unit_hit  = dalloc_n<uint32_t>(max_units, st);
        k_unit_map<<<div_up(pp->n_big, 256), 256, 0, st>>>(unit_off, pp->n_big, unit_hit);
        HJ_LAUNCH_CHECK();
        k_write_big<<<num_sms() * 8, 256, 0, st>>>(T, L, pp->n_big, unit_off, unit_hit, big_off, pp->tot_light, outs);
        HJ_LAUNCH_CHECK();
        for (void* p : {(void*)units, (void*)lens, (void*)unit_off, (void*)big_off, (void*)unit_hit}) dfree(p, st);
    }
    if (pp->n_mixed) {
        uint64_t* off = dalloc_n<uint64_t>(pp->n_mixed + 1, st);
        scan_exclusive_u32_to_u64(L.m_cnt, off, pp->n_mixed, st);
        k_write_mixed_warp<<<num_sms() * 8, 256, 0, st>>>(T, L, off, pp->tot_light + pp->tot_big, outs);
        HJ_LAUNCH_CHECK();
        k_write_mixed<<<num_sms() * 2, 512, 0, st>>>(T, L, off, pp->tot_light + pp->tot_big, outs);
        HJ_LAUNCH_CHECK();
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
    return 14 * ((4 * n + 255) & ~uint64_t(255)) + 4 * ((8 * (n + 1) + 255) & ~uint64_t(255))
         + ((8 * tmp + 255) & ~uint64_t(255)) + 256;
}

int probe_into_scratch(const Table& t, const KeyCol& pk, const ProbeParams& prm, uint8_t* scratch,
                       size_t scratch_bytes, uint32_t* out_probe, uint32_t* out_build, uint64_t capacity,
                       uint64_t* num_matches, cudaStream_t st) {
    *num_matches = 0;
    if (t.n_tuples == 0 || pk.n == 0) return HJ_OK;
    const uint64_t n = pk.n;
    if (probe_scratch_bytes(n) > scratch_bytes) throw Error(HJ_ERR_INVALID, "probe scratch too small");
    Lists     L{};
    uint64_t *light_off, *unit_off, *big_off, *mixed_off, *tmp;
    uint32_t *units, *lens;
    Carve     c{scratch};
    L.ctr     = c.take<unsigned long long>(8);
    L.l_row   = c.take<uint32_t>(n);
    L.l_s     = c.take<uint32_t>(n);
    L.l_cnt   = c.take<uint32_t>(n);
    L.l_key   = c.take<int32_t>(n);
    L.b_row   = c.take<uint32_t>(n);
    L.b_s     = c.take<uint32_t>(n);
    L.b_e     = c.take<uint32_t>(n);
    L.m_row   = c.take<uint32_t>(n);
    L.m_s     = c.take<uint32_t>(n);
    L.m_e     = c.take<uint32_t>(n);
    L.m_cnt   = c.take<uint32_t>(n);
    L.m_key   = c.take<int32_t>(n);
    units     = c.take<uint32_t>(n);
    lens      = c.take<uint32_t>(n);
    light_off = c.take<uint64_t>(n + 1);
    unit_off  = c.take<uint64_t>(n + 1);
    big_off   = c.take<uint64_t>(n + 1);
    mixed_off = c.take<uint64_t>(n + 1);
    tmp       = c.take<uint64_t>(scan_tmp_words(n) + 1);
    // the scratch keeps the previous call's contents: the counters restart at zero
    HJ_CUDA(cudaMemsetAsync(L.ctr, 0, 8 * sizeof(unsigned long long), st));
    const ProbeTab T      = tab_of(t);
    const uint64_t ntiles = (n + kPTile - 1) / kPTile;
    const int      grid   = probe_count_grid(ntiles);
    k_probe_count<<<grid, kPT, 0, st>>>(T, pk, prm.light_max, L, ntiles);
    HJ_LAUNCH_CHECK();
    k_mixed_count<<<num_sms() * 2, 512, 0, st>>>(T, L);
    HJ_LAUNCH_CHECK();
    uint64_t* h = prm.pinned;
    readback(h, L.ctr, 6 * sizeof(uint64_t), true, st);  // page-locked scratch
    HJ_CUDA(cudaStreamSynchronize(st));
    const uint64_t n_light = h[0], n_big = h[1], n_mixed = h[2];
    const uint64_t tot_light = h[3], tot_big = h[4], total = h[3] + h[4] + h[5];
    *num_matches = total;
    if (total > capacity) return HJ_ERR_CAPACITY;
    if (total == 0) return HJ_OK;
    Outs outs{};
    outs.n    = 2;
    outs.o[0] = RidOut{0, nullptr, out_probe};
    outs.o[1] = RidOut{1, nullptr, out_build};
    if (n_light) {
        scan_exclusive_u32_to_u64_into(L.l_cnt, light_off, n_light, tmp, st);
        const int g = int(std::min<uint64_t>(div_up(n_light, 256), uint64_t(num_sms()) * 16));
        switch (prm.group) {
        case 1: k_write_light<1><<<g, 256, 0, st>>>(T, L, n_light, light_off, outs); break;
        case 4: k_write_light<4><<<g, 256, 0, st>>>(T, L, n_light, light_off, outs); break;
        case 32: k_write_light<32><<<g, 256, 0, st>>>(T, L, n_light, light_off, outs); break;
        default: k_write_light<8><<<g, 256, 0, st>>>(T, L, n_light, light_off, outs); break;
        }
        HJ_LAUNCH_CHECK();
    }
    if (n_big) {
        k_big_units<<<div_up(n_big, 256), 256, 0, st>>>(L.b_s, L.b_e, n_big, units, lens);
        HJ_LAUNCH_CHECK();
        scan_exclusive_u32_to_u64_into(units, unit_off, n_big, tmp, st);
        scan_exclusive_u32_to_u64_into(lens, big_off, n_big, tmp, st);
        // the per-hit unit counts were consumed by the scan above, so their
        // n-entry array holds the unit map when it fits; otherwise the write
        // kernel finds each unit's hit by binary search
        const uint64_t max_units = n_big + h[4] / kSplit + 1;
        uint32_t*      unit_hit  = max_units <= n ? units : nullptr;
        if (unit_hit) {
            k_unit_map<<<div_up(n_big, 256), 256, 0, st>>>(unit_off, n_big, unit_hit);
            HJ_LAUNCH_CHECK();
        }
        k_write_big<<<num_sms() * 8, 256, 0, st>>>(T, L, n_big, unit_off, unit_hit, big_off, tot_light, outs);
        HJ_LAUNCH_CHECK();
    }
    if (n_mixed) {
        scan_exclusive_u32_to_u64_into(L.m_cnt, mixed_off, n_mixed, tmp, st);
        k_write_mixed_warp<<<num_sms() * 8, 256, 0, st>>>(T, L, mixed_off, tot_light + tot_big, outs);
        HJ_LAUNCH_CHECK();
        k_write_mixed<<<num_sms() * 2, 512, 0, st>>>(T, L, mixed_off, tot_light + tot_big, outs);
        HJ_LAUNCH_CHECK();
    }
    return HJ_OK;
}

void probe_free(ProbePlan* pp, cudaStream_t st) {
    if (!pp) return;
    Lists& L = pp->ls;
    for (void* p : {(void*)L.l_row, (void*)L.l_s, (void*)L.l_cnt, (void*)L.l_key, (void*)L.b_row,
                    (void*)L.b_s, (void*)L.b_e, (void*)L.m_row, (void*)L.m_s, (void*)L.m_e,
                    (void*)L.m_cnt, (void*)L.m_key, (void*)L.ctr})
        if (p) dfree(p, st);
    delete pp;
}

}  // namespace hj
