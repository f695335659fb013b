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
// Every page is assembled in shared memory and stored with 16-byte writes;
// bytes the reference leaves uninitialised (between data and bitmap) are zero.
#include <algorithm>

#include "hj_block.cuh"
#include "hj_common.cuh"
#include "hj_kernels.h"

namespace hj {

// One output page of a VARCHAR column (declared in hj_kernels.h).
struct PageDesc {
    uint64_t row;    // first row (normal page) or the string's row (long page)
    uint32_t count;  // rows on a normal page; 0 for a long-string page
    uint32_t nn;     // non-NULL rows (normal page)
    uint32_t bytes;  // string bytes (normal page)
    uint32_t chunk;  // long-string page number within the string
};

namespace {

constexpr int      kMT        = 256;
constexpr uint32_t kLongLimit = kPage - 7;  // longer strings go to long-string pages
constexpr uint32_t kLongChunk = kPage - 4;  // bytes per long-string page
constexpr int      kStrTile   = 4096;       // rows per packing tile

__device__ __forceinline__ void store_page(uint8_t* out, const uint8_t* img) {
    uint4*       dst = reinterpret_cast<uint4*>(out);
    const uint4* src = reinterpret_cast<const uint4*>(img);
    for (uint32_t i = threadIdx.x; i < kPage / 16; i += blockDim.x) dst[i] = src[i];
}

__device__ __forceinline__ void zero_img(uint8_t* img) {
    uint4* w = reinterpret_cast<uint4*>(img);
    for (uint32_t i = threadIdx.x; i < kPage / 16; i += blockDim.x) w[i] = make_uint4(0, 0, 0, 0);
}

// Bitmap bytes of 32 rows starting at row `first` (a multiple of 32).
__device__ __forceinline__ void put_bits(uint8_t* img, uint32_t bm0, uint32_t nbytes, uint32_t first,
                                         uint32_t ballot) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t byte = first / 8 + k;
        if (byte < nbytes) img[bm0 + byte] = uint8_t(ballot >> (8 * k));
    }
}

// ---- INT32 -----------------------------------------------------------------

// Block per output page of 1984 rows: thread t takes rows 8t .. 8t+7, issues
// their 8 gathers together, and owns bitmap byte t; one block scan of the
// non-NULL counts places the values.
constexpr int kIntRows = 8;
static_assert(kMT * kIntRows >= kDenseRows, "one pass per page");

__global__ void __launch_bounds__(kMT)
    k_write_int32_pages(IntCol col, const uint32_t* __restrict__ rid, uint64_t n, uint8_t* __restrict__ out) {
    __shared__ __align__(16) uint8_t img[kPage];
    __shared__ uint32_t              sm[33];
    const bool     nullable = col.tagged != nullptr || col.valid != nullptr;
    uint32_t*      words    = reinterpret_cast<uint32_t*>(img);
    const uint64_t npg      = (n + kDenseRows - 1) / kDenseRows;
    for (uint64_t p = blockIdx.x; p < npg; p += gridDim.x) {
        const uint64_t r0 = p * kDenseRows;
        const uint32_t nr = uint32_t(n - r0 < uint64_t(kDenseRows) ? n - r0 : uint64_t(kDenseRows));
        zero_img(img);
        const uint32_t i0 = threadIdx.x * kIntRows;
        uint32_t       row[kIntRows];
#pragma unroll
        for (int k = 0; k < kIntRows; ++k) {
            const uint32_t i = i0 + k;
            row[k]           = i < nr ? (rid ? __ldg(rid + r0 + i) : uint32_t(r0 + i)) : 0u;
        }
        int32_t  v[kIntRows];
        uint32_t on = 0;
#pragma unroll
        for (int k = 0; k < kIntRows; ++k) {
            v[k] = 0;
            if (i0 + k < nr && int_get(col, row[k], v[k])) on |= 1u << k;
        }
        uint32_t tot;
        const uint32_t rank = nullable ? block_exclusive_scan<uint32_t>(__popc(on), sm, &tot)
                                       : (i0 < nr ? i0 : nr);
        if (!nullable) {
            tot = nr;
            __syncthreads();  // the image is zeroed
        }
        uint32_t q = rank;
#pragma unroll
        for (int k = 0; k < kIntRows; ++k)
            if ((on >> k) & 1u) words[1 + q++] = uint32_t(v[k]);
        const uint32_t nbytes = (nr + 7) / 8;
        if (i0 < nr) img[kPage - nbytes + threadIdx.x] = uint8_t(on);
        if (threadIdx.x == 0) words[0] = nr | (tot << 16);
        __syncthreads();
        store_page(out + p * kPage, img);
        __syncthreads();
    }
}

// ---- VARCHAR -----------------------------------------------------------------

__device__ __forceinline__ uint32_t loc_len(uint64_t loc, const uint8_t* base, uint64_t npages) {
    const uint64_t f = loc_len_field(loc);
    if ((loc & kLocLong) && f == kLocLenMax) return long_len(base, loc_off(loc) / kPage, npages);
    return uint32_t(f);
}


// Greedy packing of one tile by one warp.  With desc == nullptr only counts.
__device__ uint32_t pack_tile(const uint64_t* ol, const uint8_t* base, uint64_t npages, uint64_t t0,
                              uint64_t t1, PageDesc* desc) {
    const unsigned lane   = threadIdx.x & 31;
    uint32_t       npg    = 0;
    uint64_t       pstart = t0;
    uint32_t       n = 0, m = 0, D = 0;  // rows, non-NULL rows, data bytes of the open page
    auto close_page = [&](uint64_t row_end) {
        if (n > 0) {
            if (desc && lane == 0) desc[npg] = PageDesc{pstart, n, m, D, 0};
            ++npg;
        }
        n = m = D = 0;
        pstart    = row_end;
    };
    // the next batch's locators are loaded while the current one is packed
    uint64_t next = t0 + lane < t1 ? ol[t0 + lane] : 0;
    for (uint64_t b0 = t0; b0 < t1; b0 += 32) {
        const uint64_t r      = b0 + lane;
        const bool     in     = r < t1;
        const uint64_t loc    = next;
        next                  = b0 + 32 + lane < t1 ? ol[b0 + 32 + lane] : 0;
        const bool     nn     = loc != 0;
        const uint32_t len    = nn ? loc_len(loc, base, npages) : 0;
        const bool     lng    = nn && len > kLongLimit;
        const unsigned inmask = __ballot_sync(0xffffffffu, in);
        const unsigned lmask  = __ballot_sync(0xffffffffu, lng);
        unsigned       sl     = 0;                   // first lane not yet placed
        const unsigned nl     = 32 - __clz(inmask);  // lanes in this batch
        while (sl < nl) {
            const unsigned later_long = lmask & (0xffffffffu << sl);
            const unsigned ll         = later_long ? unsigned(__ffs(later_long) - 1) : nl;
            if (ll == sl) {  // long string: its own pages
                const uint32_t L = __shfl_sync(0xffffffffu, len, sl);
                close_page(b0 + sl);
                const uint32_t chunks = (L + kLongChunk - 1) / kLongChunk;
                if (desc && lane == 0)
                    for (uint32_t k = 0; k < chunks; ++k) desc[npg + k] = PageDesc{b0 + sl, 0, 0, 0, k};
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

// The VARCHAR output columns of one materialisation are packed together:
// warp w of a launch takes tile w of the concatenated tile lists, so short
// columns share the GPU instead of each filling a fraction of it.
constexpr int kMaxPackCols = 8;
struct PackCol {
    const uint64_t* locs;
    const uint32_t* rid;
    uint64_t*       ol;
    const uint8_t*  base;
    uint64_t        npages, n, ntiles, tile_base;
    uint32_t*       tile_pages;
    const uint64_t* tile_off;
    PageDesc*       desc;
    uint64_t*       recs;  // kRec page-start records per tile
};
struct PackCols {
    int     n;
    PackCol c[kMaxPackCols];
};

__device__ __forceinline__ int pack_col_of(const PackCols& P, uint64_t t) {
    int c = 0;
    while (c + 1 < P.n && P.c[c + 1].tile_base <= t) ++c;
    return c;
}

// Packing by prefix sums.  A row costs 8 * (2 + length) + 1 eighths of a
// byte when non-NULL (offset, string bytes, bitmap bit) and 1 when NULL; a
// page of rows [a, b) fits when 32 + sum(cost) + 7 <= 65536 eighths (header,
// bitmap rounded up to whole bytes), i.e. sum(cost) <= kCap.  With S_i the
// tile's exclusive prefix of costs and T = kCap - (largest cost in the tile),
// row i goes to page floor(S_i / T): a page then holds less than T + max cost
// <= kCap, and no page is empty because no row costs more than T.  Tiles with
// a long string or a row costing more than kCap / 8 (strings over ~1 KB) are
// packed by the greedy rule instead (pack_tile, one warp).
constexpr uint32_t kCap     = 65536 - 32 - 7;
constexpr int      kPackT   = 512;                 // threads per tile block
constexpr int      kPackRow = kStrTile / kPackT;   // consecutive rows per thread
static_assert(kPackRow * kPackT == kStrTile, "tile split");

struct TileCosts {
    uint32_t cost[kPackRow];
    uint32_t nn, len;  // this thread's non-NULL rows and string bytes
    uint32_t maxc;
    bool     greedy;   // a long string or a costly row in this thread's rows
};

__device__ __forceinline__ TileCosts row_costs(const uint64_t (&loc)[kPackRow], uint32_t rows) {
    TileCosts c{};
#pragma unroll
    for (int k = 0; k < kPackRow; ++k) {
        const bool     on  = uint32_t(k) < rows && loc[k] != 0;
        const bool     lng = on && (loc[k] & kLocLong);
        const uint32_t len = on ? uint32_t(loc_len_field(loc[k])) : 0u;
        c.cost[k]          = uint32_t(k) >= rows ? 0u : (on ? 8u * (2u + min(len, kPage)) + 1u : 1u);
        c.nn += on;
        c.len += len;
        c.maxc = max(c.maxc, c.cost[k]);
        c.greedy |= lng || c.cost[k] > kCap / 8;
    }
    return c;
}

// Block reduction of (max, any) over the tile; every thread gets the result.
__device__ __forceinline__ void tile_max_any(uint32_t& maxc, bool& any, uint32_t* sm) {
    uint32_t m = maxc, a = any;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        m = max(m, __shfl_xor_sync(0xffffffffu, m, d));
        a |= __shfl_xor_sync(0xffffffffu, a, d);
    }
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        sm[warp]      = m;
        sm[16 + warp] = a;
    }
    __syncthreads();
    m = 0;
    a = 0;
    for (int w = 0; w < kPackT / 32; ++w) {
        m = max(m, sm[w]);
        a |= sm[16 + w];
    }
    maxc = m;
    any  = a != 0;
    __syncthreads();
}

// Cost of one row from its locator (as row_costs).
__device__ __forceinline__ uint32_t loc_cost(uint64_t loc) {
    return loc != 0 ? 8u * (2u + min(uint32_t(loc_len_field(loc)), kPage)) + 1u : 1u;
}

// Page starts of a prefix-summed tile, kRec records per tile: record p is
// (first row | non-NULL rows before it << 16 | string bytes before it << 32),
// tile-relative; record np closes the last page.  Rows cost at most kCap / 8,
// so a page holds at least 7 rows.  Record 0 of a greedy tile is kGreedyRec.
constexpr int      kMaxTilePages = kStrTile / 7 + 1;
constexpr int      kRec          = kMaxTilePages + 1;
constexpr uint64_t kGreedyRec    = 0xffffull;

__device__ __forceinline__ uint64_t page_rec(uint32_t row, uint32_t nn, uint32_t len) {
    return uint64_t(row) | (uint64_t(nn) << 16) | (uint64_t(len) << 32);
}

// Gathers the tile's locators through the row ids into `ol` (read back by the
// later passes in output order), and packs the tile: its page count, and for
// a prefix-summed tile its page starts.  Thread t takes the tile's rows
// 8t .. 8t+7 from the start: its row ids as two 16-byte loads, its eight
// locator gathers in flight together, its locators kept in registers for the
// packing and stored to `ol` as 16-byte writes (no shared-memory staging).
__global__ void __launch_bounds__(kPackT) k_pack_count(PackCols P, uint64_t ntiles) {
    __shared__ uint32_t sm[33];
    __shared__ uint64_t s_scan[33];
    __shared__ uint64_t s_last[kPackT / 32];  // each warp's last locator
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint64_t g = blockIdx.x; g < ntiles; g += gridDim.x) {
        const PackCol& v  = P.c[pack_col_of(P, g)];
        const uint64_t t  = g - v.tile_base;
        const uint64_t t0 = t * kStrTile, t1 = (v.n < t0 + kStrTile ? v.n : t0 + kStrTile);
        const uint32_t nt = uint32_t(t1 - t0);
        const uint32_t li0  = threadIdx.x * kPackRow;  // this thread's first row in the tile
        const uint64_t r0   = t0 + li0;
        const uint32_t rows = li0 >= nt ? 0u : (nt - li0 < kPackRow ? nt - li0 : uint32_t(kPackRow));
        const bool     full = rows == kPackRow;
        uint64_t       loc[kPackRow];
        {
            uint32_t src[kPackRow];
            if (v.rid && full && (reinterpret_cast<uintptr_t>(v.rid + r0) & 15) == 0) {
                const uint4 x = __ldg(reinterpret_cast<const uint4*>(v.rid + r0));
                const uint4 y = __ldg(reinterpret_cast<const uint4*>(v.rid + r0) + 1);
                src[0] = x.x; src[1] = x.y; src[2] = x.z; src[3] = x.w;
                src[4] = y.x; src[5] = y.y; src[6] = y.z; src[7] = y.w;
            } else {
#pragma unroll
                for (int k = 0; k < kPackRow; ++k) src[k] = v.rid && uint32_t(k) < rows ? __ldg(v.rid + r0 + k) : 0u;
            }
#pragma unroll
            for (int k = 0; k < kPackRow; ++k)
                loc[k] = uint32_t(k) < rows ? __ldg(v.locs + (v.rid ? uint64_t(src[k]) : r0 + k)) : 0ull;
            if (full && (reinterpret_cast<uintptr_t>(v.ol + r0) & 15) == 0) {
                ulonglong2* o = reinterpret_cast<ulonglong2*>(v.ol + r0);
#pragma unroll
                for (int k = 0; k < kPackRow; k += 2) o[k / 2] = make_ulonglong2(loc[k], loc[k + 1]);
            } else {
#pragma unroll
                for (int k = 0; k < kPackRow; ++k)
                    if (uint32_t(k) < rows) v.ol[r0 + k] = loc[k];
            }
        }
        // the locator of the row before this thread's first: the previous
        // lane's last, or across warps through shared memory (read after the
        // barriers of tile_max_any)
        uint64_t prev = __shfl_up_sync(0xffffffffu, loc[kPackRow - 1], 1);
        if (lane == 31) s_last[warp] = loc[kPackRow - 1];
        uint64_t*      rec  = v.recs + t * kRec;
        TileCosts c = row_costs(loc, rows);
        tile_max_any(c.maxc, c.greedy, sm);
        if (lane == 0 && warp > 0) prev = s_last[warp - 1];
        if (c.greedy) {
            if (threadIdx.x < 32) {
                const uint32_t np = pack_tile(v.ol, v.base, v.npages, t0, t1, nullptr);
                if (threadIdx.x == 0) {
                    v.tile_pages[t] = np;
                    rec[0]          = kGreedyRec;
                }
            }
            __syncthreads();
            continue;
        }
        // S stays below 2^32: at most 4096 rows of at most kCap / 8 eighths each
        const uint32_t T = kCap - c.maxc;
        // exclusive prefix of (non-NULL rows << 40 | string bytes) at this thread's first row
        uint64_t       tot;
        const uint64_t pre = block_exclusive_scan<uint64_t>((uint64_t(c.nn) << 40) | c.len, s_scan, &tot);
        uint32_t       NN = uint32_t(pre >> 40), LEN = uint32_t(pre & ((1ull << 40) - 1));
        // S: the row's start in eighths of a byte (offsets, string bytes, one bit per row)
        uint32_t S       = 8u * (2u * NN + LEN) + li0;
        uint32_t pg_prev = li0 > 0 && rows > 0 ? (S - loc_cost(prev)) / T : 0u;
#pragma unroll
        for (int k = 0; k < kPackRow; ++k) {
            if (uint32_t(k) >= rows) break;
            const uint32_t li = li0 + k;
            const uint32_t pg = S / T;
            if ((li == 0 || pg_prev != pg) && pg < uint32_t(kMaxTilePages)) rec[pg] = page_rec(li, NN, LEN);
            if (uint64_t(li) + 1 == t1 - t0) {  // last row: the closing record and the page count
                const uint32_t np = pg + 1 < uint32_t(kMaxTilePages) ? pg + 1 : uint32_t(kMaxTilePages);
                rec[np]           = page_rec(uint32_t(t1 - t0), uint32_t(tot >> 40),
                                             uint32_t(tot & ((1ull << 40) - 1)));
                v.tile_pages[t]   = np;
            }
            NN += loc[k] != 0;
            LEN += loc[k] != 0 ? uint32_t(loc_len_field(loc[k])) : 0u;
            pg_prev = pg;
            S += c.cost[k];
        }
        __syncthreads();
    }
}

// Page descriptors at tile_off[t]: one warp per tile, from the page starts of
// k_pack_count or by the greedy rule.
__global__ void k_pack_emit(PackCols P, uint64_t ntiles) {
    const uint64_t g = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (g >= ntiles) return;
    const PackCol&  v    = P.c[pack_col_of(P, g)];
    const uint64_t  t    = g - v.tile_base;
    const uint64_t  t0   = t * kStrTile, t1 = (v.n < t0 + kStrTile ? v.n : t0 + kStrTile);
    const uint64_t* rec  = v.recs + t * kRec;
    PageDesc*       desc = v.desc + v.tile_off[t];
    if (rec[0] == kGreedyRec) {
        pack_tile(v.ol, v.base, v.npages, t0, t1, desc);
        return;
    }
    const uint32_t np = uint32_t(v.tile_off[t + 1] - v.tile_off[t]);
    for (uint32_t p = threadIdx.x & 31; p < np; p += 32) {
        const uint64_t a = rec[p], b = rec[p + 1];
        const uint32_t rs = uint32_t(a & 0xffff), re = uint32_t(b & 0xffff);
        const uint32_t ns = uint32_t((a >> 16) & 0xffff), ne = uint32_t((b >> 16) & 0xffff);
        const uint32_t ls = uint32_t(a >> 32), le = uint32_t(b >> 32);
        desc[p] = PageDesc{t0 + rs, re - rs, ne - ns, le - ls, 0};
    }
}

// Copies `len` bytes of a normal string from global `src` (inside an input
// page) to shared memory at img + dst.  Strings of up to 64 bytes: all covering
// source words are loaded first (up to 18 independent loads in flight), then
// aligned destination words are formed with funnel shifts and stored as 32-bit
// words; the two boundary words, which neighbouring strings share, are merged
// into the zeroed image with a masked shared-memory OR (one instruction instead
// of up to four byte stores).  Only words that overlap the string are read.
__device__ __forceinline__ void copy_string(uint8_t* img, uint32_t dst, const uint8_t* src, uint32_t len) {
    if (len == 0) return;
    const uintptr_t a  = reinterpret_cast<uintptr_t>(src);
    const uint32_t  sa = uint32_t(a & 3), da = dst & 3;
    if (len > 64) {  // generic path
        for (uint32_t k = 0; k < len; ++k) img[dst + k] = src[k];
        return;
    }
    // start one word early when the source is less offset than the destination,
    // so that destination word j always takes source words j and j + 1
    const uint32_t  pre = sa < da ? 4u : 0u;
    const uintptr_t w0  = (a & ~uintptr_t(3)) - pre;  // source word W[0]
    const uint32_t  so  = sa + pre;                   // string start within the words
    const uint32_t  sh  = 8 * (so - da);              // 0, 8, 16 or 24
    const uint32_t  nsw = (so + len + 3) / 4;         // words W[k] that overlap the string
    // The words are read as 8-byte pairs from the 8-byte boundary at or below
    // W[0]: W[k] = P[k + odd].  Bytes outside the string that come along are
    // masked off below; the reads stay inside the string's input page (its
    // data starts at byte >= 6 and ends before the bitmap) or the buffer slack.
    const uintptr_t q0    = w0 & ~uintptr_t(7);
    const uint32_t  odd   = uint32_t((w0 - q0) >> 2);
    const uint32_t  first = so / 4;  // first W[k] that overlaps the string
    const uint2*    qs    = reinterpret_cast<const uint2*>(q0);
    uint32_t        P[20];
#pragma unroll
    for (int q = 0; q < 10; ++q) {
        const bool  need = uint32_t(2 * q) < odd + nsw && uint32_t(2 * q + 1) >= odd + first;
        const uint2 v    = need ? __ldg(qs + q) : make_uint2(0u, 0u);
        P[2 * q]         = v.x;
        P[2 * q + 1]     = v.y;
    }
    const uint32_t ndw = (da + len + 3) / 4;  // destination words touched
    uint32_t*      wd  = reinterpret_cast<uint32_t*>(img + (dst & ~3u));
#pragma unroll
    for (int j = 0; j < 18; ++j) {
        if (uint32_t(j) >= ndw) break;
        const uint32_t D = __funnelshift_r(odd ? P[j + 1] : P[j], odd ? P[j + 2] : P[j + 1], sh);
        if (j == 0 || uint32_t(j) == ndw - 1) {
            // boundary word: only the bytes of this string, bytes [lo, hi) of the word
            const int      lo   = j == 0 ? int(da) : 0;
            const int      hi   = min(4, int(da) + int(len) - 4 * j);
            const uint32_t mask = (hi >= 4 ? 0xffffffffu : ((1u << (8 * hi)) - 1u)) & ~((1u << (8 * lo)) - 1u);
            atomicOr(wd + j, D & mask);
        } else {
            wd[j] = D;
        }
    }
}

// One output page per kVWP warps, assembled in one 8 KB image in shared
// memory: the page's 32-row chunks are split into kVWP contiguous parts, one
// per warp (a part's first rank and byte come from summing the locators before
// it), each warp runs a warp scan of (non-NULL, bytes) per chunk with one
// string per lane, and the image is stored with 16-byte writes.  The warps of
// a page meet only at two named barriers per page (image zeroed; image
// complete); a page's latency chain of dependent string loads is split
// kVWP ways without more shared memory, which keeps L1 for the string loads.
constexpr int kVWP  = 2;  // warps per page
constexpr int kVPB  = 4;  // pages in flight per block
constexpr int kVMin = 4;  // blocks per SM
constexpr int kVT   = kVWP * kVPB * 32;
static_assert(kVPB <= 15, "one named barrier per page slot");

// Barrier of the kVWP warps of page slot `slot` (named barrier 1 + slot; the
// warp is reconverged first, as bar.sync requires).
__device__ __forceinline__ void page_sync(unsigned slot) {
    __syncwarp();
    if (kVWP > 1) asm volatile("bar.sync %0, %1;" ::"r"(1 + slot), "r"(32 * kVWP) : "memory");
}

__global__ void __launch_bounds__(kVT, kVMin)
    k_write_varchar_pages(const PageDesc* __restrict__ desc, uint64_t ndesc, const uint64_t* __restrict__ ol,
                          const uint8_t* __restrict__ base, uint64_t npages, uint8_t* __restrict__ out) {
    extern __shared__ __align__(16) uint8_t vimg[];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned slot = warp / kVWP, part = warp % kVWP;
    uint8_t*       img  = vimg + size_t(slot) * kPage;
    constexpr int  kQ   = kPage / 16 / (32 * kVWP);  // 16-byte words per lane of a part's share
    uint4*         w4   = reinterpret_cast<uint4*>(img) + part * 32 * kQ;  // this part's share of the image
    for (uint64_t pi = uint64_t(blockIdx.x) * kVPB + slot; pi < ndesc; pi += uint64_t(gridDim.x) * kVPB) {
        const PageDesc d = desc[pi];
#pragma unroll
        for (int k = 0; k < kQ; ++k) w4[lane + 32 * k] = make_uint4(0, 0, 0, 0);
        page_sync(slot);  // strings may cross into the other parts' shares
        if (d.count == 0) {  // long-string page `chunk` of the string in row d.row
            if (part == 0) {
                const uint64_t loc = ol[d.row];
                const uint32_t L   = loc_len(loc, base, npages);
                const uint32_t beg = d.chunk * kLongChunk;
                const uint32_t len = min(kLongChunk, L - beg);
                if (lane == 0) {
                    *reinterpret_cast<uint16_t*>(img)     = d.chunk == 0 ? 0xffff : 0xfffe;
                    *reinterpret_cast<uint16_t*>(img + 2) = uint16_t(len);
                }
                // source: the 0xffff page and its 0xfffe continuations, in order
                uint64_t q  = loc_off(loc) / kPage;
                uint32_t so = 0;  // string offset of page q's first byte
                for (; q < npages && so < beg + len; ++q) {
                    const uint8_t* pg = base + q * kPage;
                    const uint32_t pl = *reinterpret_cast<const uint16_t*>(pg + 2);
                    const uint32_t lo = max(so, beg), hi = min(so + pl, beg + len);
                    for (uint32_t x = lo + lane; x < hi; x += 32) img[4 + x - beg] = pg[4 + x - so];
                    so += pl;
                }
            }
        } else {
            const uint32_t data0  = 4 + 2 * d.nn;
            const uint32_t nbytes = (d.count + 7) / 8, bm0 = kPage - nbytes;
            // this part's rows: whole 32-row chunks, so parts own disjoint bitmap bytes
            const uint32_t nch = (d.count + 31) / 32, per = (nch + kVWP - 1) / kVWP;
            const uint32_t r0  = min(d.count, part * per * 32), r1 = min(d.count, (part + 1) * per * 32);
            // (non-NULL count << 16 | bytes) before the part: a page holds at
            // most 4094 non-NULL rows and 8188 string bytes, so the halves never carry
            uint32_t pre = 0;
            for (uint32_t r = lane; r < r0 && r0 < r1; r += 32) {
                const uint64_t loc = ol[d.row + r];
                pre += loc != 0 ? 0x10000u | uint32_t(loc_len_field(loc)) : 0u;
            }
            pre            = warp_sum(pre);
            uint32_t rank0 = pre >> 16, byte0 = pre & 0xffffu;
            uint64_t next  = r0 + lane < r1 ? ol[d.row + r0 + lane] : 0;
            for (uint32_t c = r0; c < r1; c += 32) {
                const uint64_t loc = next;
                next               = c + 32 + lane < r1 ? ol[d.row + c + 32 + lane] : 0;
                const bool     on  = loc != 0;
                const uint32_t len = on ? uint32_t(loc_len_field(loc)) : 0u;
                const uint32_t v    = (on ? 0x10000u : 0u) | len;
                const uint32_t inc  = warp_inclusive_scan<uint32_t>(v);
                const uint32_t tot  = __shfl_sync(0xffffffffu, inc, 31);
                const uint32_t ex   = inc - v;
                const uint32_t rank = rank0 + (ex >> 16);
                const uint32_t boff = byte0 + (ex & 0xffffu);
                // the packer guarantees both bounds; they are checked so that no
                // inconsistent descriptor can write outside the page image
                if (on && rank < d.nn && data0 + boff + len <= bm0) {
                    *reinterpret_cast<uint16_t*>(img + 4 + 2 * rank) = uint16_t(boff + len);
                    copy_string(img, data0 + boff, base + loc_off(loc), len);
                }
                const uint32_t b = __ballot_sync(0xffffffffu, on);
                if (lane == 0) put_bits(img, bm0, nbytes, c, b);
                rank0 += tot >> 16;
                byte0 += tot & 0xffffu;
            }
            if (part == 0 && lane == 0) {
                *reinterpret_cast<uint16_t*>(img)     = uint16_t(d.count);
                *reinterpret_cast<uint16_t*>(img + 2) = uint16_t(d.nn);
            }
        }
        page_sync(slot);  // image complete
        // each part stores its own share; the next page zeroes only that
        // share, and its first barrier orders the other parts' writes after
        uint4* dst = reinterpret_cast<uint4*>(out + pi * kPage) + part * 32 * kQ;
#pragma unroll
        for (int k = 0; k < kQ; ++k) dst[lane + 32 * k] = w4[lane + 32 * k];
    }
}

unsigned grid_of(uint64_t items, uint64_t per_sm = 16) {
    return unsigned(std::max<uint64_t>(1, std::min<uint64_t>(items, uint64_t(num_sms()) * per_sm)));
}

}  // namespace

void launch_write_int32_pages(const IntCol& col, const uint32_t* rid, uint64_t n, uint8_t* out_pages,
                              cudaStream_t st) {
    if (n == 0) return;
    const uint64_t pages = (n + kDenseRows - 1) / kDenseRows;
    k_write_int32_pages<<<grid_of(pages), kMT, 0, st>>>(col, rid, n, out_pages);
    HJ_LAUNCH_CHECK();
}

namespace {
// The columns of `vs` (n > 0 rows) in groups of kMaxPackCols, as launch parameters.
template <class F>
void for_pack_groups(std::vector<VarcharOut*>& vs, F&& f) {
    std::vector<VarcharOut*> live;
    for (auto* v : vs)
        if (v->n) live.push_back(v);
    for (size_t g0 = 0; g0 < live.size(); g0 += kMaxPackCols) {
        PackCols P{};
        uint64_t tiles = 0;
        for (size_t i = g0; i < std::min(live.size(), g0 + kMaxPackCols); ++i) {
            VarcharOut& v = *live[i];
            P.c[P.n++]    = PackCol{v.locs, v.rid, v.ol, v.base, v.base_pages, v.n, v.ntiles, tiles,
                                 v.tile_pages, v.tile_off, v.desc, v.recs};
            tiles += v.ntiles;
        }
        f(P, tiles);
    }
}
}  // namespace

void varchar_plan(std::vector<VarcharOut*>& vs, cudaStream_t st) {
    for (auto* vp : vs) {
        VarcharOut& v = *vp;
        if (v.n == 0) continue;
        v.ol         = dalloc_n<uint64_t>(v.n, st);
        v.ntiles     = (v.n + kStrTile - 1) / kStrTile;
        v.tile_pages = dalloc_n<uint32_t>(v.ntiles, st);
        v.tile_off   = dalloc_n<uint64_t>(v.ntiles + 1, st);
        v.recs       = dalloc_n<uint64_t>(v.ntiles * kRec, st);
    }
    for_pack_groups(vs, [&](const PackCols& P, uint64_t tiles) {
        k_pack_count<<<grid_of(tiles, 4), kPackT, 0, st>>>(P, tiles);
        HJ_LAUNCH_CHECK();
    });
    for (auto* vp : vs)
        if (vp->n) scan_exclusive_u32_to_u64(vp->tile_pages, vp->tile_off, vp->ntiles, st);
}

std::vector<uint8_t*> varchar_write(std::vector<VarcharOut*>& vs, const std::vector<uint64_t>& pages,
                                    cudaStream_t st) {
    std::vector<uint8_t*> out(vs.size(), nullptr);
    for (size_t i = 0; i < vs.size(); ++i)
        if (vs[i]->n) vs[i]->desc = static_cast<PageDesc*>(dalloc(std::max<uint64_t>(pages[i], 1) * sizeof(PageDesc), st));
    for_pack_groups(vs, [&](const PackCols& P, uint64_t tiles) {
        k_pack_emit<<<div_up(tiles * 32, 256), 256, 0, st>>>(P, tiles);
        HJ_LAUNCH_CHECK();
    });
    for (size_t i = 0; i < vs.size(); ++i) {
        VarcharOut& v = *vs[i];
        if (v.n == 0) continue;
        out[i] = static_cast<uint8_t*>(dalloc(std::max<uint64_t>(pages[i], 1) * kPage, st));
        HJ_CUDA(cudaFuncSetAttribute(k_write_varchar_pages, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     kVPB * kPage));
        k_write_varchar_pages<<<grid_of(div_up(pages[i], kVPB), kVMin), kVT, kVPB * kPage, st>>>(
            v.desc, pages[i], v.ol, v.base, v.base_pages, out[i]);
        HJ_LAUNCH_CHECK();
        for (void* p : {(void*)v.desc, (void*)v.ol, (void*)v.tile_pages, (void*)v.tile_off, (void*)v.recs})
            dfree(p, st);
        v.desc       = nullptr;
        v.ol         = nullptr;
        v.tile_pages = nullptr;
        v.tile_off   = nullptr;
        v.recs       = nullptr;
    }
    return out;
}

}  // namespace hj
