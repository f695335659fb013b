// Host launchers of the engine's CUDA kernels.  Every launcher enqueues on
// `st` and does not synchronise; device pointers only.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <vector>

#include "hj_common.cuh"

namespace hj {

// Stream-ordered device memory (cudaMallocAsync on a pool that keeps freed
// blocks cached for reuse; blocks of 64 MB and more are reused per stream).
void* dalloc(size_t bytes, cudaStream_t st);
void  dfree(void* p, cudaStream_t st);
// Returns the large blocks kept for reuse on `st` (before `st` is destroyed).
void  flush_stream(cudaStream_t st);

template <class T>
T* dalloc_n(size_t n, cudaStream_t st) {
    return static_cast<T*>(dalloc(n * sizeof(T) + 16, st));
}

// ---- host <-> HBM page transfers by the GPU (hj_transfer.cu) ---------------
// Need pageable host memory access (cudaDevAttrPageableMemoryAccess).  gather:
// host pages -> contiguous HBM, page header fields into nr / nn (device arrays).
void launch_gather_host_pages(const void* const* host_pages, uint64_t n, uint8_t* dst, uint16_t* nr,
                              uint16_t* nn, cudaStream_t st);
// scatter: contiguous HBM pages -> host_pages[i] (or host_contig when host_pages is null).
void launch_scatter_host_pages(const uint8_t* src, uint64_t n, void* const* host_pages, void* host_contig,
                               cudaStream_t st);
// Runs of consecutive host pages (page i + 1 at page i + 8192 bytes), when
// every run lies in page-locked memory and there are at most max_runs of
// them; otherwise empty.  Such pages move with one cudaMemcpyAsync per run.
struct PageRun {
    uint64_t first, count;
};
std::vector<PageRun> locked_runs(const void* const* pages, uint64_t n, size_t max_runs);
// Whether [p, p + bytes) starts and ends in page-locked host memory.
bool locked_range(const void* p, uint64_t bytes);
// Device -> host copy of a few bytes (counters, page headers).  kernel: the
// GPU writes `host` itself (page-locked memory, or any host memory with
// pageable host memory access), so the readback never waits behind large
// transfers queued on the copy engines by other streams; otherwise a
// cudaMemcpyAsync.  Stream-ordered; the caller synchronises.
void readback(void* host, const void* dev, uint64_t bytes, bool kernel, cudaStream_t st);
// nr / nn (device arrays) from the headers of n device pages.
void launch_page_headers(const uint8_t* pages, uint64_t n, uint16_t* nr, uint16_t* nn, cudaStream_t st);

// ---- scans (hj_scan.cu) ---------------------------------------------------
// out[i] = sum(in[0..i)), out[n] = total.  out has n + 1 slots.
void scan_exclusive_u32_to_u64(const uint32_t* in, uint64_t* out, uint64_t n, cudaStream_t st);
void scan_exclusive_u64(const uint64_t* in, uint64_t* out, uint64_t n, cudaStream_t st);
// Same as scan_exclusive_u32_to_u64 with caller-provided temporaries of
// scan_tmp_words(n) words; allocates nothing (so it can be graph-captured).
size_t scan_tmp_words(uint64_t n);
void   scan_exclusive_u32_to_u64_into(const uint32_t* in, uint64_t* out, uint64_t n, uint64_t* tmp,
                                      cudaStream_t st);

// ---- page decode (hj_decode.cu) --------------------------------------------
// rows[p] = rows page p contributes to its column (VARCHAR: 0xffff -> 1, 0xfffe -> 0).
void launch_page_rows(const uint8_t* pages, uint64_t num_pages, int32_t type, uint32_t* rows,
                      cudaStream_t st);
// row_start: exclusive scan of page rows.  INT32 -> value_t per row; INT32
// without NULLs -> int32 per row; VARCHAR -> locator per row (hj_common.cuh).
void launch_decode_int32_tagged(const uint8_t* pages, uint64_t num_pages, const uint64_t* row_start,
                                uint64_t* out, cudaStream_t st);
void launch_decode_int32_plain(const uint8_t* pages, uint64_t num_pages, const uint64_t* row_start,
                               int32_t* out, cudaStream_t st);
void launch_decode_varchar_loc(const uint8_t* pages, uint64_t num_pages, const uint64_t* row_start,
                               uint64_t* out, cudaStream_t st);

// ---- unchained table build (hj_build.cu) -----------------------------------
struct KeyCol {
    IntCol          col;    // the base column
    const uint32_t* rid;    // row ids into the base column, or nullptr = identity
    uint64_t        n;      // rows of the (intermediate) column
    Filters         filt;   // probe side only: scan predicates evaluated on base row ids (rid == nullptr)
};

// ---- scan predicates (hj_filter.cu) ----------------------------------------
// Base rows 0..n-1 that pass `f`, in order, into rid_out (n slots); returns their
// number (one host synchronisation through `pinned`).
uint64_t filter_compact(const Filters& f, uint64_t n, uint32_t* rid_out, uint64_t* pinned, cudaStream_t st);

struct Table {
    uint32_t  dir_bits  = 0;
    uint64_t  n_tuples  = 0;
    uint64_t* dir       = nullptr;  // 2^dir_bits + 1 words: start << 16 | bloom
    int32_t*  keys      = nullptr;  // adjacency array: keys
    uint32_t* rows      = nullptr;  // adjacency array: build row ids (index into KeyCol)
    uint32_t* mixed     = nullptr;  // bit p set: bucket p holds more than one distinct key
    uint64_t* summary   = nullptr;  // 2^dir_bits bucket summaries (make_summary, hj_common.cuh)
};

// Builds `t` over the valid keys of `kc`.  dir_bits < 0: next_pow2(#valid).
// radix_bits < 0: automatic.  Allocates t's arrays with dalloc.  n_valid: the
// number of valid keys when the caller knows it (>= 0), else the build reads
// it back from the device (one synchronisation).
// dir_cap_bits bounds the automatic directory size (dir_bits < 0) so the
// directory stays cache resident; 64 = UnchainedHash sizing exactly.
void build_table(const KeyCol& kc, int dir_bits, int radix_bits, Table& t, uint64_t* scratch_host,
                 cudaStream_t st, int64_t n_valid = -1, int dir_cap_bits = 64);
void free_table(Table& t, cudaStream_t st);

// ---- probe (hj_probe.cu) ---------------------------------------------------
// One output row-id stream of a join: out[k] = src ? src[x] : x, where x is the
// probe row (side 0) or the build row (side 1) of match k.
struct RidOut {
    int             side;
    const uint32_t* src;
    uint32_t*       dst;
};
constexpr int kMaxRidOut = 16;

struct ProbeParams {
    int       light_max = 32;       // larger buckets are not scanned by one thread
    int       group     = 8;        // threads per probe key in the write pass (1, 4, 8, 32)
    uint64_t* pinned    = nullptr;  // >= 8 words of pinned host memory for count readback
    std::function<void()> after_count;  // called once the count kernels are enqueued
};

struct ProbePlan;  // opaque match list between the count and write passes

// Count pass: returns the number of matches; keeps the hit list in *pp.
uint64_t probe_count(const Table& t, const KeyCol& pk, const ProbeParams& prm, ProbePlan** pp,
                     cudaStream_t st);
// Write pass: emits the row-id streams for the matches found by probe_count
// (all `nout` streams have probe_count() slots); the caller frees *pp with
// probe_free afterwards.
void probe_write(const Table& t, const KeyCol& pk, ProbePlan* pp, const RidOut* outs, int nout,
                 cudaStream_t st);
void probe_free(ProbePlan* pp, cudaStream_t st);

// Count + write in one call with every temporary carved from `scratch`
// (probe_scratch_bytes(n) bytes, device memory the caller owns); allocates
// nothing.  Returns HJ_ERR_CAPACITY (writing nothing) when the matches exceed
// `capacity`; *num_matches is always set.
size_t probe_scratch_bytes(uint64_t n);
int    probe_into_scratch(const Table& t, const KeyCol& pk, const ProbeParams& prm, uint8_t* scratch,
                          size_t scratch_bytes, uint32_t* out_probe, uint32_t* out_build,
                          uint64_t capacity, uint64_t* num_matches, cudaStream_t st);

// ---- output pages (hj_materialize.cu) --------------------------------------
// INT32 output column of n rows gathered through rid (nullptr = identity) from a
// base column; writes ceil(n / 1984) pages.
void launch_write_int32_pages(const IntCol& col, const uint32_t* rid, uint64_t n, uint8_t* out_pages,
                              cudaStream_t st);

struct PageDesc;  // one output page of a VARCHAR column (hj_materialize.cu)

// VARCHAR output columns in two steps, so that several columns share one
// host synchronisation: plan (gather locators, pack pages, count them into
// *page_count, a device word) then write (after the caller read the counts).
struct VarcharOut {
    const uint64_t* locs;        // locators of the base column
    const uint8_t*  base;        // its pages
    uint64_t        base_pages;
    const uint32_t* rid;         // row ids or nullptr
    uint64_t        n;           // output rows
    // filled by varchar_plan
    uint64_t*       ol         = nullptr;  // gathered locators, n
    uint32_t*       tile_pages = nullptr;
    uint64_t*       tile_off   = nullptr;  // ntiles + 1 (last = page count, on the device)
    uint64_t        ntiles     = 0;
    PageDesc*       desc       = nullptr;  // varchar_write's page descriptors
    uint64_t*       recs       = nullptr;  // page starts per tile (packing scratch)
};
// All VARCHAR columns of a result at once (their packing kernels share launches).
void varchar_plan(std::vector<VarcharOut*>& vs, cudaStream_t st);
// pages[i] = vs[i]->tile_off[ntiles] as read by the caller; returns the page buffers.
std::vector<uint8_t*> varchar_write(std::vector<VarcharOut*>& vs, const std::vector<uint64_t>& pages,
                                    cudaStream_t st);

// ---- batched independent joins (hj_batch.cu) ------------------------------
// One relation of a batch instance: INT32 keys (no NULLs) and one INT32 payload.
struct BatchRelation {
    const int32_t* keys;
    const int32_t* payload;
    uint64_t       rows;
};
// A chain R0 x R1 x ... on one key: R0 probes R1, the result probes R2, ...
// (2 to 8 relations)
struct BatchInstance {
    std::vector<BatchRelation> rels;
};
struct BatchOptions {
    double load       = 0.5;   // build rows per bucket of a partition table (2^ceil(log2(rows / load)) buckets)
    int    part_rows_log2 = 12;  // partitions of ~2^x build rows (x in 8..13); radix bits follow per instance
    bool   graph      = true;  // capture the whole batch in one CUDA graph
};
// Row count and checksum (sum of row fingerprints) per instance.  Returns the
// instances with a partition too large for a shared-memory table (their rows /
// sums are not valid; the caller recomputes them with plain_instance).
std::vector<uint32_t> batch_execute(const std::vector<BatchInstance>& b, const BatchOptions& o,
                                    std::vector<uint64_t>& rows, std::vector<uint64_t>& sums, cudaStream_t st);
// One instance through the regular table build and two-pass probe.
void plain_instance(const BatchInstance& b, const ProbeParams& prm, int dir_bits, int radix_bits, int dir_cap_bits,
                    uint64_t& rows, uint64_t& sum, cudaStream_t st);
// Synthetic instance relations generated on the device from (seed, instance, relation).
void launch_batch_generate(uint64_t seed, uint32_t instance, uint32_t relation, uint64_t build_rows,
                           uint32_t match_q24, uint64_t rows, int32_t* keys, int32_t* payload, cudaStream_t st);

}  // namespace hj

// Read-only views of C-ABI objects for code outside hj_engine.cu.
struct hj_context;
struct hj_hash_table;
struct hj_result;
namespace hj {
int             context_device(const hj_context* c);
cudaStream_t    context_stream(const hj_context* c);
ProbeParams     context_probe_params(const hj_context* c);  // options + pinned readback
void            context_set_error(hj_context* c, const char* msg);
const Table&    hash_table_of(const hj_hash_table* t);
// A context on the same device sharing `p`'s resident tables and options (a
// serving slot: its own stream, pinned buffers and host threads).
hj_context*     context_clone(const hj_context* p);
uint64_t        resident_rows(const hj_context* c, uint64_t handle);  // 0 if unknown
// Frees a result's pages on `st` from now on (the stream it was made on is
// idle and may go away first).
void            result_rebind(hj_result* r, cudaStream_t st);
}  // namespace hj
