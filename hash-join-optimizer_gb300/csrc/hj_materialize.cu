// Final materialisation: join output (row ids into base columns) -> pages in
// the reference's format, assembled in HBM.  Device form of table_to_columnar
// and deref_str_ref (src/execute.cpp:371-573 of the reference).
//
// Page packing.  The reference appends rows to a page while the page,
// including the new row, fits in 8192 bytes (execute.cpp:472-479, 545-556).
// Its readers (copy_scan, Table::from_columnar) accept any packing that fits.
// Row order of a join result is unspecified, so page boundaries cannot be
// compared with the reference's anyway; the GPU writer picks packings that
// parallelise:
//  * INT32: exactly 1984 rows per page (the last page holds the rest).  That is
//    the reference's packing whenever the column has no NULLs, and always
//    fits (1984 values + 248 bitmap bytes + 4 header bytes = 8188 bytes).
//  * VARCHAR: the reference's greedy rule applied independently inside tiles
//    of 4096 consecutive rows (a page never spans two tiles), so tiles are
//    packed in parallel by one warp each; strings longer than 8185 bytes get
//    0xffff/0xfffe long-string pages exactly as the reference writes them.
// Bytes the reference leaves uninitialised (between data and bitmap) are zero.
#include <algorithm>

#include "../../include/value_t.h"
#include "hj_block.cuh"
#include "hj_common.cuh"
#include "hj_kernels.h"

namespace hj {
namespace {

constexpr int      kMT        = 256;
constexpr uint32_t kNullLen   = 0xffffffffu;
constexpr uint32_t kLongLimit = kPage - 7;  // longer strings go to long-string pages
constexpr uint32_t kLongChunk = kPage - 4;  // bytes per long-string page
constexpr int      kStrTile   = 4096;       // rows per packing tile

// ---- INT32 -----------------------------------------------------------------

__global__ void __launch_bounds__(kMT)
    k_write_int32_pages(const int32_t* __restrict__ vals, const uint32_t* __restrict__ valid,
                        const uint32_t* __restrict__ rid, uint64_t n, uint8_t* __restrict__ out) {
    __shared__ __align__(16) uint32_t img[kPage / 4];
    __shared__ uint32_t               sm[33];
    const uint64_t p  = blockIdx.x;
    const uint64_t r0 = p * kDenseRows;
    const uint32_t nr = uint32_t(n - r0 < uint64_t(kDenseRows) ? n - r0 : uint64_t(kDenseRows));
    for (uint32_t i = threadIdx.x; i < kPage / 4; i += blockDim.x) img[i] = 0;
    __syncthreads();
    uint8_t*       bytes   = reinterpret_cast<uint8_t*>(img);
    const uint32_t bm_base = kPage - (nr + 7) / 8;
    uint32_t       nn      = 0;
    for (uint32_t c = 0; c < nr; c += blockDim.x) {
        const uint32_t i  = c + threadIdx.x;
        bool           on = false;
        int32_t        v  = 0;
        if (i < nr) {
            const uint64_t r = rid ? uint64_t(__ldg(rid + r0 + i)) : r0 + i;
            on               = bit_valid(valid, r);
            if (on) v = __ldg(vals + r);
        }
        uint32_t       tot;
        const uint32_t rank = valid ? block_exclusive_scan<uint32_t>(on ? 1u : 0u, sm, &tot)
                                    : threadIdx.x;
        if (!valid) tot = min(nr - c, uint32_t(blockDim.x));
        if (on) img[1 + nn + rank] = uint32_t(v);
        const uint32_t b = __ballot_sync(0xffffffffu, on);
        if ((threadIdx.x & 31) == 0) {
            const uint32_t first = c + (threadIdx.x & ~31u);  // row of bit 0, multiple of 32
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const uint32_t byte = first / 8 + k;
                if (byte < (nr + 7) / 8) bytes[bm_base + byte] = uint8_t(b >> (8 * k));
            }
        }
        nn += tot;
    }
    __syncthreads();
    if (threadIdx.x == 0) img[0] = nr | (nn << 16);
    __syncthreads();
    uint4*       dst = reinterpret_cast<uint4*>(out + p * kPage);
    const uint4* src = reinterpret_cast<const uint4*>(img);
    for (uint32_t i = threadIdx.x; i < kPage / 16; i += blockDim.x) dst[i] = src[i];
}

// ---- VARCHAR -----------------------------------------------------------------

struct StrLoc {
    const uint8_t* bytes;  // first byte (normal strings) or the 0xffff page (long)
    uint32_t       len;
    bool           is_long;
};

// Resolves a StrRef against the base column's pages (deref_str_ref).
__device__ __forceinline__ StrLoc locate(uint64_t v, const uint8_t* base, uint64_t npages) {
    StrRef r;
    r.ref             = v;
    const uint64_t pg = r.get_page();
    const uint8_t* page = base + pg * kPage;
    StrLoc         s;
    if (r.is_long()) {
        uint32_t len = *reinterpret_cast<const uint16_t*>(page + 2);
        for (uint64_t q = pg + 1; q < npages; ++q) {
            const uint8_t* nx = base + q * kPage;
            if (*reinterpret_cast<const uint16_t*>(nx) != 0xfffe) break;
            len += *reinterpret_cast<const uint16_t*>(nx + 2);
        }
        s.bytes   = page;
        s.len     = len;
        s.is_long = true;
        return s;
    }
    const uint32_t  off  = uint32_t(r.get_offset());
    const uint16_t* offs = reinterpret_cast<const uint16_t*>(page + 4);
    const uint32_t  nn   = *reinterpret_cast<const uint16_t*>(page + 2);
    const uint32_t  st   = off == 0 ? 0 : offs[off - 1];
    s.bytes              = page + 4 + 2 * nn + st;
    s.len                = uint32_t(offs[off]) - st;
    s.is_long            = false;
    return s;
}

__global__ void k_str_len(const uint64_t* __restrict__ refs, const uint8_t* __restrict__ base,
                          uint64_t npages, const uint32_t* __restrict__ rid, uint64_t n,
                          uint32_t* __restrict__ lens) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint64_t r = rid ? uint64_t(__ldg(rid + i)) : i;
        const uint64_t v = __ldg(refs + r);
        lens[i]          = (v >> 62) == 2 ? locate(v, base, npages).len : kNullLen;
    }
}

struct PageDesc {
    uint64_t row;    // first row (normal page) or the string's row (long page)
    uint32_t count;  // rows on a normal page; 0 for a long-string page
    uint32_t chunk;  // long-string page number within the string
};

// Greedy packing of one tile by one warp.  With desc == nullptr only counts.
__device__ uint32_t pack_tile(const uint32_t* lens, uint64_t t0, uint64_t t1, PageDesc* desc) {
    const unsigned lane  = threadIdx.x & 31;
    uint32_t       npg   = 0;
    uint64_t       pstart = t0;
    uint32_t       n = 0, m = 0, D = 0;  // rows, non-NULL rows, data bytes of the open page
    auto close_page = [&](uint64_t row_end) {
        if (n > 0) {
            if (desc && lane == 0) desc[npg] = PageDesc{pstart, n, 0};
            ++npg;
        }
        n = m = D = 0;
        pstart    = row_end;
    };
    for (uint64_t b0 = t0; b0 < t1; b0 += 32) {
        const uint64_t r    = b0 + lane;
        const bool     in   = r < t1;
        const uint32_t len  = in ? lens[r] : 0;
        const bool     nn   = in && len != kNullLen;
        const bool     lng  = nn && len > kLongLimit;
        const unsigned inmask = __ballot_sync(0xffffffffu, in);
        const unsigned lmask  = __ballot_sync(0xffffffffu, lng);
        unsigned       sl     = 0;  // first lane not yet placed
        const unsigned nl     = 32 - __clz(inmask);  // lanes in this batch
        while (sl < nl) {
            const unsigned later_long = lmask & (0xffffffffu << sl);
            const unsigned ll         = later_long ? unsigned(__ffs(later_long) - 1) : nl;
            if (ll == sl) {  // long string: own pages
                const uint32_t L = __shfl_sync(0xffffffffu, len, sl);
                close_page(b0 + sl);
                const uint32_t chunks = (L + kLongChunk - 1) / kLongChunk;
                if (desc && lane == 0)
                    for (uint32_t k = 0; k < chunks; ++k) desc[npg + k] = PageDesc{b0 + sl, 0, k};
                npg += chunks;
                pstart = b0 + sl + 1;
                ++sl;
                continue;
            }
            // lanes [sl, ll): prefix of rows / non-NULL / bytes from lane sl
            const bool     seg  = lane >= sl && lane < ll;
            const uint32_t cnn  = warp_inclusive_scan<uint32_t>(seg && nn ? 1u : 0u);
            const uint32_t cby  = warp_inclusive_scan<uint32_t>(seg && nn ? len : 0u);
            const uint32_t crow = seg ? lane - sl + 1 : 0;
            const uint32_t n2 = n + crow, m2 = m + cnn, D2 = D + cby;
            const bool     fits = 4 + 2 * m2 + D2 + (n2 + 7) / 8 <= uint32_t(kPage);
            const unsigned bad  = __ballot_sync(0xffffffffu, seg && !fits);
            unsigned       f    = bad ? unsigned(__ffs(bad) - 1) : ll;
            // a row that fits no empty page cannot occur (strings over 8185 bytes
            // are long strings); place it alone rather than loop
            if (f == sl && n == 0) f = sl + 1;
            if (f > sl) {  // lanes [sl, f) join the open page
                const unsigned src = f - 1;
                n = __shfl_sync(0xffffffffu, n2, src);
                m = __shfl_sync(0xffffffffu, m2, src);
                D = __shfl_sync(0xffffffffu, D2, src);
            }
            if (f < ll) close_page(b0 + f);  // row f opens a new page
            sl = f;
        }
    }
    close_page(t1);
    return npg;
}

__global__ void k_pack_count(const uint32_t* __restrict__ lens, uint64_t n, uint64_t ntiles,
                             uint32_t* __restrict__ tile_pages) {
    const uint64_t t = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (t >= ntiles) return;
    const uint64_t t0 = t * kStrTile, t1 = (n < t0 + kStrTile ? n : t0 + kStrTile);
    const uint32_t c  = pack_tile(lens, t0, t1, nullptr);
    if ((threadIdx.x & 31) == 0) tile_pages[t] = c;
}

__global__ void k_pack_emit(const uint32_t* __restrict__ lens, uint64_t n, uint64_t ntiles,
                            const uint64_t* __restrict__ tile_off, PageDesc* __restrict__ desc) {
    const uint64_t t = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (t >= ntiles) return;
    const uint64_t t0 = t * kStrTile, t1 = (n < t0 + kStrTile ? n : t0 + kStrTile);
    pack_tile(lens, t0, t1, desc + tile_off[t]);
}

__global__ void __launch_bounds__(kMT)
    k_write_varchar_pages(const PageDesc* __restrict__ desc, const uint32_t* __restrict__ lens,
                          const uint64_t* __restrict__ refs, const uint8_t* __restrict__ base,
                          uint64_t npages, const uint32_t* __restrict__ rid, uint8_t* __restrict__ out) {
    __shared__ __align__(16) uint8_t img[kPage];
    __shared__ uint32_t              sm[33];
    __shared__ uint32_t              s_m;
    const PageDesc d = desc[blockIdx.x];
    for (uint32_t i = threadIdx.x; i < kPage / 4; i += blockDim.x) reinterpret_cast<uint32_t*>(img)[i] = 0;
    __syncthreads();
    if (d.count == 0) {  // long-string page `chunk` of the string in row d.row
        const uint64_t r   = rid ? uint64_t(rid[d.row]) : d.row;
        const StrLoc   s   = locate(refs[r], base, npages);
        const uint32_t beg = d.chunk * kLongChunk;
        const uint32_t len = min(kLongChunk, s.len - beg);
        if (threadIdx.x == 0) {
            *reinterpret_cast<uint16_t*>(img)     = d.chunk == 0 ? 0xffff : 0xfffe;
            *reinterpret_cast<uint16_t*>(img + 2) = uint16_t(len);
        }
        // source: the 0xffff page and its 0xfffe continuations, in order
        uint64_t q = (s.bytes - base) / kPage;
        uint32_t so = 0;  // string offset of page q's first byte
        for (; q < npages && so < beg + len; ++q) {
            const uint8_t* pg = base + q * kPage;
            const uint32_t pl = *reinterpret_cast<const uint16_t*>(pg + 2);
            const uint32_t lo = max(so, beg), hi = min(so + pl, beg + len);
            for (uint32_t x = lo + threadIdx.x; x < hi; x += blockDim.x) img[4 + x - beg] = pg[4 + x - so];
            so += pl;
        }
    } else {
        // pass 1: number of non-NULL rows -> offsets start at +4, data after them
        uint32_t mcount = 0;
        for (uint32_t c = 0; c < d.count; c += blockDim.x) {
            const uint32_t i = c + threadIdx.x;
            const bool     on = i < d.count && lens[d.row + i] != kNullLen;
            uint32_t       tot;
            block_exclusive_scan<uint32_t>(on ? 1u : 0u, sm, &tot);
            mcount += tot;
        }
        const uint32_t data0 = 4 + 2 * mcount;
        const uint32_t bm0   = kPage - (d.count + 7) / 8;
        uint32_t       rank0 = 0, byte0 = 0;
        for (uint32_t c = 0; c < d.count; c += blockDim.x) {
            const uint32_t i   = c + threadIdx.x;
            const uint32_t len = i < d.count ? lens[d.row + i] : kNullLen;
            const bool     on  = len != kNullLen;
            uint32_t       tr, tb;
            const uint32_t rank = rank0 + block_exclusive_scan<uint32_t>(on ? 1u : 0u, sm, &tr);
            const uint32_t boff = byte0 + block_exclusive_scan<uint32_t>(on ? len : 0u, sm, &tb);
            if (on) {
                const uint64_t r = rid ? uint64_t(__ldg(rid + d.row + i)) : d.row + i;
                const StrLoc   s = locate(__ldg(refs + r), base, npages);
                *reinterpret_cast<uint16_t*>(img + 4 + 2 * rank) = uint16_t(boff + len);
                for (uint32_t x = 0; x < len; ++x) img[data0 + boff + x] = s.bytes[x];
            }
            const uint32_t b = __ballot_sync(0xffffffffu, on && i < d.count);
            if ((threadIdx.x & 31) == 0) {
                const uint32_t first = c + (threadIdx.x & ~31u);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const uint32_t byte = first / 8 + k;
                    if (byte < (d.count + 7) / 8) img[bm0 + byte] = uint8_t(b >> (8 * k));
                }
            }
            rank0 += tr;
            byte0 += tb;
        }
        if (threadIdx.x == 0) {
            *reinterpret_cast<uint16_t*>(img)     = uint16_t(d.count);
            *reinterpret_cast<uint16_t*>(img + 2) = uint16_t(mcount);
        }
    }
    __syncthreads();
    uint4*       dst = reinterpret_cast<uint4*>(out + uint64_t(blockIdx.x) * kPage);
    const uint4* src = reinterpret_cast<const uint4*>(img);
    for (uint32_t i = threadIdx.x; i < kPage / 16; i += blockDim.x) dst[i] = src[i];
}

}  // namespace

void launch_write_int32_pages(const int32_t* vals, const uint32_t* valid, const uint32_t* rid,
                              uint64_t n, uint8_t* out_pages, cudaStream_t st) {
    if (n == 0) return;
    const uint64_t pages = (n + kDenseRows - 1) / kDenseRows;
    k_write_int32_pages<<<unsigned(pages), kMT, 0, st>>>(vals, valid, rid, n, out_pages);
    HJ_LAUNCH_CHECK();
}

uint64_t write_varchar_pages(const uint64_t* refs, const uint8_t* base_pages, uint64_t base_num_pages,
                             const uint32_t* rid, uint64_t n, uint8_t** out_pages, uint64_t* pinned,
                             cudaStream_t st) {
    *out_pages = nullptr;
    if (n == 0) return 0;
    uint32_t* lens = dalloc_n<uint32_t>(n, st);
    k_str_len<<<std::min<uint64_t>(div_up(n, 256), uint64_t(kSMs) * 8), 256, 0, st>>>(
        refs, base_pages, base_num_pages, rid, n, lens);
    HJ_LAUNCH_CHECK();
    const uint64_t ntiles     = (n + kStrTile - 1) / kStrTile;
    uint32_t*      tile_pages = dalloc_n<uint32_t>(ntiles, st);
    uint64_t*      tile_off   = dalloc_n<uint64_t>(ntiles + 1, st);
    const unsigned grid       = div_up(ntiles * 32, 256);
    k_pack_count<<<grid, 256, 0, st>>>(lens, n, ntiles, tile_pages);
    HJ_LAUNCH_CHECK();
    scan_exclusive_u32_to_u64(tile_pages, tile_off, ntiles, st);
    HJ_CUDA(cudaMemcpyAsync(pinned, tile_off + ntiles, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    HJ_CUDA(cudaStreamSynchronize(st));
    const uint64_t npages = pinned[0];
    PageDesc*      desc   = static_cast<PageDesc*>(dalloc(npages * sizeof(PageDesc) + 16, st));
    k_pack_emit<<<grid, 256, 0, st>>>(lens, n, ntiles, tile_off, desc);
    HJ_LAUNCH_CHECK();
    uint8_t* out = static_cast<uint8_t*>(dalloc(npages * kPage, st));
    k_write_varchar_pages<<<unsigned(npages), kMT, 0, st>>>(desc, lens, refs, base_pages,
                                                            base_num_pages, rid, out);
    HJ_LAUNCH_CHECK();
    for (void* p : {(void*)lens, (void*)tile_pages, (void*)tile_off, (void*)desc}) dfree(p, st);
    *out_pages = out;
    return npages;
}

}  // namespace hj
