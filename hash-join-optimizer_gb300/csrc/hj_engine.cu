// Host runtime of the GB300 join engine and its C ABI (include/hj_api.h).
//
// Device form of Contest::execute (src/execute.cpp:584-608 of the reference):
//   * inputs: each (table, column) a scan touches is uploaded once per call
//     (or found resident in HBM) as its raw 8 KiB pages, then decoded on the
//     GPU (copy_scan, execute.cpp:265-369);
//   * intermediates: a join result is a set of row-id vectors, one per base
//     table instance ("source") that its output columns still reference, plus
//     the (source, input column) of every output column.  This is the device
//     column_t (include/column_t.h): a column_t in "direct" mode over an input
//     column, seen through a selection vector.  Values stay in the input
//     columns; only 4-byte row ids move between joins;
//   * joins: build the unchained table on the build side's key, probe with the
//     probe side's key, write one composed row-id vector per needed source
//     (JoinAlgorithm::run, execute.cpp:26-186);
//   * output: the root's columns are written as pages in HBM
//     (table_to_columnar, execute.cpp:431-573), VARCHAR bytes gathered through
//     their StrRef only there.
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <thread>
#include <vector>

#include "../../include/hj_api.h"
#include "../../include/value_t.h"
#include "hj_common.cuh"
#include "hj_kernels.h"

namespace hj {

std::atomic<uint64_t> g_kernel_launches{0};

int num_sms() {
    constexpr int           kMaxDev = 64;
    static std::atomic<int> cache[kMaxDev];
    int                     dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) dev = 0;
    const int slot = dev < kMaxDev ? dev : kMaxDev - 1;
    int       n    = cache[slot].load(std::memory_order_relaxed);
    if (n > 0) return n;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
        cudaGetLastError();  // leave no sticky status behind
        n = 152;
    }
    if (dev < kMaxDev) cache[slot].store(n, std::memory_order_relaxed);
    return n;
}

// ---------------------------------------------------------------- memory ----

// Blocks are kept per stream when freed on the stream that allocated them,
// and handed back to the next allocation of a similar size on that stream
// without going through the pool: stream order makes the reuse safe, the host
// never waits on the pool's memory mapping between two kernels, and the
// dozens of small temporaries of an execute (counters, offsets, page
// descriptors) cost no driver call.  Large blocks (result pages, decoded
// columns, row-id streams: >= 64 MB) are sized in 16 MB granules and reused
// up to 25% larger; smaller ones in power-of-two classes from 4 KB, reused
// from their own class.  A block freed on another stream (a served result,
// freed through the server's context) goes back to the pool, and a stream
// keeps at most kKeepPerStream bytes.  flush_stream() returns a stream's blocks.
namespace {
constexpr size_t kBig           = size_t(64) << 20;
constexpr size_t kGranule       = size_t(16) << 20;
constexpr size_t kSmallMin      = size_t(4) << 10;
constexpr size_t kKeepPerStream = size_t(48) << 30;
struct BigBlock {
    size_t       bytes;
    cudaStream_t owner;  // the stream that allocated it
};
struct BigBlocks {
    std::mutex                                                     mu;
    std::unordered_map<cudaStream_t, std::multimap<size_t, void*>> free;
    std::unordered_map<cudaStream_t, size_t>                       kept;  // bytes in `free` per stream
    std::unordered_map<void*, BigBlock>                            size;
};
BigBlocks& big_blocks() {
    static BigBlocks* b = new BigBlocks();  // outlives every context
    return *b;
}
void* pool_alloc(size_t bytes, cudaStream_t st) {
    void*             p = nullptr;
    const cudaError_t e = cudaMallocAsync(&p, bytes, st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}
}  // namespace

void flush_stream(cudaStream_t st) {
    BigBlocks&                  b = big_blocks();
    std::lock_guard<std::mutex> g(b.mu);
    auto                        it = b.free.find(st);
    if (it == b.free.end()) return;
    for (auto& kv : it->second) {
        b.size.erase(kv.second);
        cudaFreeAsync(kv.second, st);
    }
    b.free.erase(it);
    b.kept.erase(st);
}

void* dalloc(size_t bytes, cudaStream_t st) {
    if (bytes >= kBig) {
        bytes = (bytes + kGranule - 1) / kGranule * kGranule;
    } else {
        size_t c = kSmallMin;
        while (c < bytes) c <<= 1;
        bytes = c;
    }
    BigBlocks& b = big_blocks();
    {
        std::lock_guard<std::mutex> g(b.mu);
        auto&                       m  = b.free[st];
        auto                        it = m.lower_bound(bytes);
        if (it != m.end() && it->first <= bytes + bytes / 4) {
            void* p = it->second;
            b.kept[st] -= it->first;
            m.erase(it);
            return p;
        }
    }
    void* p = pool_alloc(bytes, st);
    if (!p) {  // give every cached block back and try once more
        std::vector<cudaStream_t> streams;
        {
            std::lock_guard<std::mutex> g(b.mu);
            for (auto& kv : b.free) streams.push_back(kv.first);
        }
        for (auto s2 : streams) flush_stream(s2);
        cudaDeviceSynchronize();
        p = pool_alloc(bytes, st);
    }
    if (!p) throw Error(HJ_ERR_NOMEM, "device allocation of " + std::to_string(bytes) + " bytes failed");
    std::lock_guard<std::mutex> g(b.mu);
    b.size[p] = BigBlock{bytes, st};
    return p;
}

void dfree(void* p, cudaStream_t st) {
    if (!p) return;
    {
        BigBlocks&                  b = big_blocks();
        std::lock_guard<std::mutex> g(b.mu);
        auto                        it = b.size.find(p);
        if (it != b.size.end()) {
            const size_t bytes = it->second.bytes;
            if (it->second.owner == st && b.kept[st] + bytes <= kKeepPerStream) {
                b.free[st].emplace(bytes, p);
                b.kept[st] += bytes;
                return;
            }
            b.size.erase(it);  // back to the pool
        }
    }
    cudaFreeAsync(p, st);
}

namespace {

// Device buffer freed (stream-ordered) when the last reference goes.
struct DevBuf {
    void*        p  = nullptr;
    cudaStream_t st = nullptr;
    DevBuf(size_t bytes, cudaStream_t s) : p(dalloc(bytes, s)), st(s) {}
    DevBuf(void* adopt, cudaStream_t s) : p(adopt), st(s) {}
    ~DevBuf() { dfree(p, st); }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};
using Buf = std::shared_ptr<DevBuf>;

Buf make_buf(size_t bytes, cudaStream_t st) { return std::make_shared<DevBuf>(bytes, st); }

// ------------------------------------------------------------ host threads --

class ThreadPool {
public:
    explicit ThreadPool(unsigned n) {
        for (unsigned i = 0; i < n; ++i) workers_.emplace_back([this] { loop(); });
    }
    ~ThreadPool() {
        {
            std::lock_guard<std::mutex> g(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto& w : workers_) w.join();
    }

    // Runs fn(i) for i in [0, n) on the pool and the calling thread.
    void parallel_for(size_t n, const std::function<void(size_t)>& fn) {
        if (n == 0) return;
        if (n == 1 || workers_.empty()) {
            for (size_t i = 0; i < n; ++i) fn(i);
            return;
        }
        std::atomic<size_t> next{0};
        std::atomic<size_t> done{0};
        const size_t        helpers = std::min<size_t>(workers_.size(), n - 1);
        auto body = [&] {
            for (size_t i; (i = next.fetch_add(1)) < n;) fn(i);
        };
        {
            std::lock_guard<std::mutex> g(mu_);
            for (size_t h = 0; h < helpers; ++h)
                jobs_.push_back([&] {
                    body();
                    done.fetch_add(1);
                });
        }
        cv_.notify_all();
        body();
        while (done.load() < helpers) std::this_thread::yield();
    }

private:
    void loop() {
        for (;;) {
            std::function<void()> job;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [this] { return stop_ || !jobs_.empty(); });
                if (stop_ && jobs_.empty()) return;
                job = std::move(jobs_.back());
                jobs_.pop_back();
            }
            job();
        }
    }
    std::vector<std::thread>           workers_;
    std::vector<std::function<void()>> jobs_;
    std::mutex                         mu_;
    std::condition_variable            cv_;
    bool                               stop_ = false;
};

// ------------------------------------------------------------ input tables --

struct DevColumn {
    int32_t  type      = HJ_INT32;
    uint64_t num_pages = 0;
    Buf      pages;  // raw pages, contiguous
    // page statistics, read from the page headers on the host at upload
    uint64_t rows      = 0;      // rows the reference's copy_scan yields
    uint64_t non_null  = 0;
    bool     dense1984 = false;  // INT32, no NULLs, every page but the last 1984 rows
    int64_t  strref_bad_page = -1;  // first page index > 2^18-1 that carries strings
    // first row of each page (num_pages + 1 words), from the headers at upload,
    // for columns that are decoded (not dense INT32)
    Buf row_start;
    // decoded form (per execute call, or once per resident table: predecoded)
    bool decoded    = false;
    bool predecoded = false;
    Buf  plain;   // INT32 without NULLs on irregular pages
    Buf  tagged;  // INT32 with NULLs: value_t per row
    Buf  locs;    // VARCHAR: locator per row

    IntCol icol() const {
        IntCol c;
        if (tagged) c.tagged = tagged->as<uint64_t>();
        else if (plain) c.plain = plain->as<int32_t>();
        else if (pages) c.pages = pages->as<uint8_t>();
        return c;
    }
};

// Statistics of one column from its page headers (host side).
void page_stats(DevColumn& d, const uint16_t* nr, const uint16_t* nn) {
    d.rows = d.non_null = 0;
    d.dense1984         = d.type == HJ_INT32;
    d.strref_bad_page   = -1;
    for (uint64_t p = 0; p < d.num_pages; ++p) {
        if (d.type == HJ_INT32) {
            d.rows += nr[p];
            d.non_null += nn[p];
            if (nr[p] != nn[p] || (p + 1 < d.num_pages && nr[p] != kDenseRows)) d.dense1984 = false;
        } else if (d.type == HJ_VARCHAR) {
            uint32_t r = nr[p], v = nn[p];
            if (nr[p] == 0xffff) r = v = 1;
            else if (nr[p] == 0xfffe) r = v = 0;
            d.rows += r;
            d.non_null += v;
            if (v > 0 && p > StrRef::PAGE_MASK && d.strref_bad_page < 0) d.strref_bad_page = int64_t(p);
        }
    }
}

struct DevTable {
    uint64_t               num_rows = 0;
    std::vector<DevColumn> cols;
};

// Unchained tables built over a resident base column, kept for reuse by later
// plans (option "table_cache"): keyed by the table handle, the column and the
// options that shape the table.
struct BuiltKey {
    uint64_t handle;
    uint32_t col;
    int64_t  dir_bits, radix_bits, dir_cap_bits;
    bool operator<(const BuiltKey& o) const {
        return std::tie(handle, col, dir_bits, radix_bits, dir_cap_bits)
             < std::tie(o.handle, o.col, o.dir_bits, o.radix_bits, o.dir_cap_bits);
    }
};

// Tables resident in HBM, shared by a context and the serving slots cloned
// from it (hj_server); every access holds `mu`.
struct Store {
    std::mutex                                  mu;
    // Host -> HBM uploads of the contexts that share this store (a server's
    // slots) run one plan at a time: two plans uploading at once only split
    // the host link's upload direction, and they slow the result downloads of
    // finished plans that share the link.
    std::mutex                                  upload_mu;
    std::map<uint64_t, std::shared_ptr<DevTable>> tables;
    std::map<BuiltKey, std::shared_ptr<Table>>    built;
    uint64_t                                    next_handle = 1;
    int                                         device      = 0;
    // built tables may be read by kernels on any stream: free them only after
    // the whole device is idle
    void drop_built(uint64_t handle) {
        std::vector<std::shared_ptr<Table>> gone;
        for (auto it = built.begin(); it != built.end();) {
            if (it->first.handle == handle || handle == 0) {
                gone.push_back(it->second);
                it = built.erase(it);
            } else {
                ++it;
            }
        }
        if (gone.empty()) return;
        cudaSetDevice(device);
        cudaDeviceSynchronize();
        for (auto& t : gone) free_table(*t, nullptr);
        cudaStreamSynchronize(nullptr);
    }
    ~Store() { drop_built(0); }
};

}  // namespace
}  // namespace hj

// ------------------------------------------------------------------ context --

struct hj_context {
    int                 device = 0;
    cudaStream_t        st     = nullptr;
    std::string         err;
    int64_t             dir_bits    = -1;
    int64_t             radix_bits  = -1;
    int64_t             probe_group = 4;
    int64_t             light_max   = 32;
    int64_t             timing      = 0;
    int64_t             dir_cap_bits = 23;  // automatic directories stay <= 64 MB (L2 resident)
    bool                ats_capable  = false;  // GPU reads/writes pageable host memory
    int64_t             host_access  = 1;      // use it for page transfers when capable
    int64_t             batch_load_pct = 50;   // batched joins: build rows per 100 buckets of a partition table
    int64_t             batch_graph    = 1;    // batched joins: launch as one CUDA graph
    int64_t             batch_part_log2 = 12;  // batched joins: ~2^x build rows per partition
    uint64_t*           pinned      = nullptr;  // small readbacks
    uint8_t*            staging     = nullptr;  // pinned transfer ring
    size_t              staging_bytes = 0;
    cudaEvent_t         slot_ev[2]  = {nullptr, nullptr};
    std::unique_ptr<hj::ThreadPool>         pool;
    std::shared_ptr<hj::Store> store;  // resident tables (shared with cloned serving slots)
    int64_t             table_cache = 0;     // reuse tables built over resident base columns
    int64_t             fuse_filters = 0;    // evaluate a probe side's scan predicate inside the probe
};

struct hj_result {
    uint64_t num_rows = 0;
    struct Col {
        int32_t  type;
        uint64_t num_pages;
        hj::Buf  pages;
    };
    std::vector<Col> cols;
    uint64_t         build_tuples = 0, probe_tuples = 0, output_rows = 0;
    uint64_t         dir_words = 0, table_tuples = 0, joins = 0;  // summed over the joins
    uint64_t         kernel_launches = 0;     // kernels this execute launched
    std::map<std::string, double> phase_ms;  // filled when option "timing" is 1
};

struct hj_hash_table {
    hj::Table    t;
    cudaStream_t st;
};

namespace hj {
namespace {

thread_local std::string g_create_error;

constexpr size_t kSlot = 64ull << 20;  // pinned staging slot (two slots)

void ensure_staging(hj_context* c) {
    if (c->staging) return;
    c->staging_bytes = 2 * kSlot;
    HJ_CUDA(cudaMallocHost(&c->staging, c->staging_bytes));
    for (auto& e : c->slot_ev) HJ_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
}

// Copies `n` host pages into the contiguous device buffer `dst`: pages are
// gathered by the host threads into a pinned slot while the previous slot is
// in flight.  The threads also read each page's header (num_rows, second
// field) into nr/nn.
void upload_pages(hj_context* c, const void* const* pages, uint64_t n, uint8_t* dst, uint16_t* nr,
                  uint16_t* nn) {
    if (n == 0) return;
    ensure_staging(c);
    const uint64_t per_slot = kSlot / kPage;
    int            slot     = 0;
    for (uint64_t p0 = 0; p0 < n; p0 += per_slot, slot ^= 1) {
        const uint64_t cnt = std::min(per_slot, n - p0);
        uint8_t*       buf = c->staging + size_t(slot) * kSlot;
        HJ_CUDA(cudaEventSynchronize(c->slot_ev[slot]));
        const uint64_t per_task = 256;
        c->pool->parallel_for((cnt + per_task - 1) / per_task, [&](size_t t) {
            const uint64_t a = t * per_task, b = std::min(cnt, a + per_task);
            for (uint64_t i = a; i < b; ++i) {
                uint8_t* pg = buf + i * kPage;
                std::memcpy(pg, pages[p0 + i], kPage);
                std::memcpy(&nr[p0 + i], pg, 2);
                std::memcpy(&nn[p0 + i], pg + 2, 2);
            }
        });
        HJ_CUDA(cudaMemcpyAsync(dst + p0 * kPage, buf, cnt * kPage, cudaMemcpyHostToDevice, c->st));
        HJ_CUDA(cudaEventRecord(c->slot_ev[slot], c->st));
    }
}

// Copies `n` device pages to host pages dst[i] (or one contiguous buffer).
void download_pages(hj_context* c, const uint8_t* src, uint64_t n, void* const* dst, uint8_t* contig) {
    if (n == 0) return;
    ensure_staging(c);
    const uint64_t per_slot = kSlot / kPage;
    int            slot     = 0;
    uint64_t       pend_p0 = 0, pend_cnt = 0;
    int            pend_slot = -1;
    auto drain = [&]() {
        if (pend_slot < 0) return;
        HJ_CUDA(cudaEventSynchronize(c->slot_ev[pend_slot]));
        uint8_t*       buf      = c->staging + size_t(pend_slot) * kSlot;
        const uint64_t per_task = 256;
        c->pool->parallel_for((pend_cnt + per_task - 1) / per_task, [&](size_t t) {
            const uint64_t a = t * per_task, b = std::min(pend_cnt, a + per_task);
            if (contig) {
                std::memcpy(contig + (pend_p0 + a) * kPage, buf + a * kPage, (b - a) * kPage);
            } else {
                for (uint64_t i = a; i < b; ++i) std::memcpy(dst[pend_p0 + i], buf + i * kPage, kPage);
            }
        });
        pend_slot = -1;
    };
    for (uint64_t p0 = 0; p0 < n; p0 += per_slot, slot ^= 1) {
        const uint64_t cnt = std::min(per_slot, n - p0);
        uint8_t*       buf = c->staging + size_t(slot) * kSlot;
        HJ_CUDA(cudaMemcpyAsync(buf, src + p0 * kPage, cnt * kPage, cudaMemcpyDeviceToHost, c->st));
        HJ_CUDA(cudaEventRecord(c->slot_ev[slot], c->st));
        drain();  // copy out the previous slot while this one transfers
        pend_p0   = p0;
        pend_cnt  = cnt;
        pend_slot = slot;
    }
    drain();
}

// The first row of every page of a column that the decode kernels read (INT32
// that is not dense, VARCHAR), summed on the host from the page headers it
// has already read at upload, and copied to the device once.
void page_row_starts(hj_context* c, DevColumn& d, const uint16_t* nr) {
    if (d.num_pages == 0 || (d.type == HJ_INT32 && d.dense1984) || (d.type != HJ_INT32 && d.type != HJ_VARCHAR))
        return;
    std::vector<uint64_t> rs(d.num_pages + 1);
    uint64_t              run = 0;
    for (uint64_t p = 0; p < d.num_pages; ++p) {
        rs[p]      = run;
        uint32_t r = nr[p];
        if (d.type == HJ_VARCHAR) r = nr[p] == 0xffff ? 1u : (nr[p] == 0xfffe ? 0u : nr[p]);
        run += r;
    }
    rs[d.num_pages] = run;
    d.row_start     = make_buf(rs.size() * sizeof(uint64_t), c->st);
    HJ_CUDA(cudaMemcpyAsync(d.row_start->p, rs.data(), rs.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, c->st));
    // the source is pageable and local: the copy must have read it before return
    HJ_CUDA(cudaStreamSynchronize(c->st));
}

bool direct_host_access(const hj_context* c) { return c->ats_capable && c->host_access; }

// Uploads the listed columns of a host table (others stay empty).  Pages in
// page-locked memory go through the copy engines, one copy per run of
// consecutive pages; otherwise, with direct host access, the GPU gathers the
// pages itself; in both cases the page headers come back in one copy for all
// columns.  Without either, host threads stage the pages.
std::shared_ptr<DevTable> upload_table(hj_context* c, const hj_table_desc& t,
                                       const std::vector<bool>& want) {
    constexpr size_t kMaxRuns = 64;
    auto dt      = std::make_shared<DevTable>();
    dt->num_rows = t.num_rows;
    dt->cols.resize(t.num_columns);
    std::vector<Buf> dhdr(t.num_columns);
    std::vector<uint16_t> nr, nn;
    for (uint32_t i = 0; i < t.num_columns; ++i) {
        DevColumn& d = dt->cols[i];
        d.type       = t.columns[i].type;
        d.num_pages  = t.columns[i].num_pages;
        if (!want.empty() && !want[i]) continue;
        // 256 bytes of slack: no kernel reads past the pages, but word loads near
        // the end of the last page never touch another allocation
        d.pages = make_buf(std::max<uint64_t>(d.num_pages, 1) * kPage + 256, c->st);
        if (d.num_pages == 0) {
            page_stats(d, nullptr, nullptr);
            continue;
        }
        const std::vector<PageRun> runs = locked_runs(t.columns[i].pages, d.num_pages, kMaxRuns);
        if (!runs.empty() || direct_host_access(c)) {
            dhdr[i]       = make_buf(d.num_pages * 4, c->st);
            uint16_t* dnr = dhdr[i]->as<uint16_t>();
            if (!runs.empty()) {
                for (const PageRun& r : runs)
                    HJ_CUDA(cudaMemcpyAsync(d.pages->as<uint8_t>() + r.first * kPage, t.columns[i].pages[r.first],
                                            r.count * kPage, cudaMemcpyHostToDevice, c->st));
                launch_page_headers(d.pages->as<uint8_t>(), d.num_pages, dnr, dnr + d.num_pages, c->st);
            } else {
                launch_gather_host_pages(t.columns[i].pages, d.num_pages, d.pages->as<uint8_t>(), dnr,
                                         dnr + d.num_pages, c->st);
            }
            continue;
        }
        nr.assign(d.num_pages, 0);
        nn.assign(d.num_pages, 0);
        upload_pages(c, t.columns[i].pages, d.num_pages, d.pages->as<uint8_t>(), nr.data(), nn.data());
        page_stats(d, nr.data(), nn.data());
        page_row_starts(c, d, nr.data());
    }
    std::vector<std::vector<uint16_t>> hnr(t.num_columns), hnn(t.num_columns);
    bool                               any = false;
    for (uint32_t i = 0; i < t.num_columns; ++i) {
        if (!dhdr[i]) continue;
        const uint64_t np = dt->cols[i].num_pages;
        hnr[i].resize(np);
        hnn[i].resize(np);
        readback(hnr[i].data(), dhdr[i]->p, np * 2, c->ats_capable, c->st);
        readback(hnn[i].data(), dhdr[i]->as<uint16_t>() + np, np * 2, c->ats_capable, c->st);
        any = true;
    }
    if (any) HJ_CUDA(cudaStreamSynchronize(c->st));
    for (uint32_t i = 0; i < t.num_columns; ++i) {
        if (dhdr[i]) {
            page_stats(dt->cols[i], hnr[i].data(), hnn[i].data());
            page_row_starts(c, dt->cols[i], hnr[i].data());
        }
        const DevColumn& d = dt->cols[i];
        if (d.pages && std::getenv("HJ_TRACE_UPLOAD"))
            std::fprintf(stderr, "[hj upload] column %u type %d pages %llu rows %llu non_null %llu dense1984 %d\n", i,
                         d.type, (unsigned long long)d.num_pages, (unsigned long long)d.rows,
                         (unsigned long long)d.non_null, int(d.dense1984));
    }
    return dt;
}

void decode_kernels(cudaStream_t st, DevColumn& d);

// Decodes a device column (idempotent within one execute call); no host
// synchronisation: sizes come from the page statistics.
void decode_column(hj_context* c, DevColumn& d, uint32_t table_id, uint32_t col_idx) {
    if (d.decoded) return;
    d.decoded = true;
    if (d.type != HJ_INT32 && d.type != HJ_VARCHAR) {  // the reference's copy_scan skips these types
        d.rows = d.non_null = 0;
        return;
    }
    if (d.type == HJ_VARCHAR && d.non_null > 0) {
        // the StrRef the reference builds for each string must fit its fields
        // (include/value_t.h:36-47); same exception class and message
        if (table_id > StrRef::TABLE_MASK)
            throw Error(HJ_ERR_OUT_OF_RANGE, "StrRef table overflow: " + std::to_string(table_id) + " > "
                                                 + std::to_string(StrRef::TABLE_MASK));
        if (col_idx > StrRef::COLUMN_MASK)
            throw Error(HJ_ERR_OUT_OF_RANGE, "StrRef column overflow: " + std::to_string(col_idx) + " > "
                                                 + std::to_string(StrRef::COLUMN_MASK));
        if (d.strref_bad_page >= 0)
            throw Error(HJ_ERR_OUT_OF_RANGE, "StrRef page overflow: " + std::to_string(d.strref_bad_page)
                                                 + " > " + std::to_string(StrRef::PAGE_MASK));
    }
    if (d.predecoded) return;  // decoded once when the resident table was prepared
    decode_kernels(c->st, d);
}

// The decode kernels of one column (no checks): pages -> plain / tagged / locators.
void decode_kernels(cudaStream_t st, DevColumn& d) {
    if (d.num_pages == 0 || d.rows == 0) return;
    if (!d.pages) throw Error(HJ_ERR_INVALID, "column pages were not uploaded");
    if (d.type == HJ_INT32 && d.dense1984) return;  // read in place (direct mode)
    const uint64_t np = d.num_pages;
    uint32_t*      pr = nullptr;
    uint64_t*      rs = d.row_start ? d.row_start->as<uint64_t>() : nullptr;
    if (!rs) {  // a column without host page statistics: row starts on the device
        pr = dalloc_n<uint32_t>(np, st);
        rs = dalloc_n<uint64_t>(np + 1, st);
        launch_page_rows(d.pages->as<uint8_t>(), np, d.type, pr, st);
        scan_exclusive_u32_to_u64(pr, rs, np, st);
    }
    if (d.type == HJ_INT32 && d.non_null == d.rows) {
        d.plain = make_buf(d.rows * 4, st);
        launch_decode_int32_plain(d.pages->as<uint8_t>(), np, rs, d.plain->as<int32_t>(), st);
    } else if (d.type == HJ_INT32) {
        d.tagged = make_buf(d.rows * 8, st);
        launch_decode_int32_tagged(d.pages->as<uint8_t>(), np, rs, d.tagged->as<uint64_t>(), st);
    } else {
        d.locs = make_buf(d.rows * 8, st);
        launch_decode_varchar_loc(d.pages->as<uint8_t>(), np, rs, d.locs->as<uint64_t>(), st);
    }
    if (pr) {
        dfree(pr, st);
        dfree(rs, st);
    }
}

// ------------------------------------------------------------ intermediates --

struct Source {
    uint32_t table;  // input table id
    Buf      rid;    // row ids into the input table's columns; null = identity
};

struct ColRef {
    int      src;    // index into Inter::srcs
    uint32_t table;
    uint32_t col;
};

struct Inter {
    uint64_t               rows = 0;
    std::vector<Source>    srcs;
    std::vector<ColRef>    cols;
    Filters                filt;  // a scan's predicates not yet applied (rows = the table's rows)
};

struct Exec {
    hj_context*                            c;
    const hj_plan_desc&                    plan;
    std::vector<std::shared_ptr<DevTable>> tables;
    uint64_t                               build_tuples = 0, probe_tuples = 0, out_rows = 0;
    uint64_t                               dir_words = 0, table_tuples = 0, joins = 0;
    std::vector<std::pair<std::string, cudaEvent_t>> marks;  // phase boundaries (timing)

    // Starts phase `name` on the stream (no-op unless option "timing" is set).
    void phase(const char* name) {
        if (!c->timing) return;
        cudaEvent_t e;
        HJ_CUDA(cudaEventCreate(&e));
        HJ_CUDA(cudaEventRecord(e, c->st));
        marks.emplace_back(name, e);
    }

    // Closes the last phase and sums device time per phase name (after sync).
    void collect(std::map<std::string, double>& out) {
        if (marks.empty()) return;
        phase("");
        HJ_CUDA(cudaEventSynchronize(marks.back().second));
        for (size_t i = 0; i + 1 < marks.size(); ++i) {
            float ms = 0;
            HJ_CUDA(cudaEventElapsedTime(&ms, marks[i].second, marks[i + 1].second));
            out[marks[i].first] += ms;
        }
        float tot = 0;
        HJ_CUDA(cudaEventElapsedTime(&tot, marks.front().second, marks.back().second));
        out["total"] = tot;
    }

    ~Exec() {
        for (auto& m : marks) cudaEventDestroy(m.second);
    }

    DevColumn& column(uint32_t t, uint32_t col) {
        DevColumn& d = tables[t]->cols[col];
        decode_column(c, d, t, col);
        return d;
    }

    Inter scan(const hj_node_desc& n) {
        Inter in;
        const uint32_t t = uint32_t(n.base_table_id);
        in.srcs.push_back(Source{t, nullptr});
        for (uint32_t a = 0; a < n.num_attrs; ++a) {
            const uint32_t col = uint32_t(n.attrs[a].index);
            in.cols.push_back(ColRef{0, t, col});
        }
        // rows: those of the first output column, as the reference's result
        // columns count them (column_t::rows_num).  Output columns of one scan
        // must agree (the reference indexes them with the same row numbers);
        // INT64/FP64 columns are empty in the reference and are not compared.
        if (n.num_attrs > 0) in.rows = column(t, uint32_t(n.attrs[0].index)).rows;
        int64_t common = -1;
        for (uint32_t a = 0; a < n.num_attrs; ++a) {
            const DevColumn& d = column(t, uint32_t(n.attrs[a].index));
            if (d.type != HJ_INT32 && d.type != HJ_VARCHAR) continue;
            if (common >= 0 && uint64_t(common) != d.rows)
                throw Error(HJ_ERR_INVALID, "columns of input table " + std::to_string(t)
                                                + " have different row counts (" + std::to_string(common)
                                                + " vs " + std::to_string(d.rows) + " in column "
                                                + std::to_string(n.attrs[a].index) + ")");
            common = int64_t(d.rows);
        }
        // scan predicates: applied later, fused into a probe or by compaction
        if (n.num_filters > 0) {
            if (n.num_filters > uint32_t(kMaxFilters) || !n.filters)
                throw Error(HJ_ERR_INVALID, "at most " + std::to_string(kMaxFilters) + " filters per scan");
            for (uint32_t i = 0; i < n.num_filters; ++i) {
                const hj_filter& f = n.filters[i];
                if (f.column >= tables[t]->cols.size()) throw Error(HJ_ERR_INVALID, "filter column out of range");
                const DevColumn& d = column(t, uint32_t(f.column));
                if (d.type != HJ_INT32) throw Error(HJ_ERR_INVALID, "filter column is not INT32");
                if (d.rows != in.rows)
                    throw Error(HJ_ERR_INVALID, "filter column of input table " + std::to_string(t)
                                                    + " has a different row count");
                const bool op_ok = (f.op >= HJ_CMP_EQ && f.op <= HJ_CMP_GEQ) || f.op == HJ_CMP_IS_NULL
                                || f.op == HJ_CMP_IS_NOT_NULL;
                if (!op_ok) throw Error(HJ_ERR_INVALID, "unsupported filter operator " + std::to_string(f.op));
                // the literal is cast as Comparison::eval does (src/statement.cpp:56)
                in.filt.f[in.filt.n++] = Filt{d.icol(), f.op, static_cast<int32_t>(f.value)};
            }
        }
        return in;
    }

    // Applies a scan's pending predicates: its passing rows become row ids, in order.
    void compact(Inter& in) {
        if (in.filt.n == 0) return;
        Buf rid = make_buf(std::max<uint64_t>(in.rows, 1) * 4, c->st);
        in.rows = filter_compact(in.filt, in.rows, rid->as<uint32_t>(), c->pinned, c->st);
        in.srcs[0].rid = rid;
        in.filt.n      = 0;
    }

    // Number of non-NULL rows of a column seen through a source's row ids.
    uint64_t non_null_through(const Inter& in, const ColRef& cr) {
        DevColumn& d = column(cr.table, cr.col);
        if (!in.srcs[cr.src].rid) return d.non_null;
        if (d.non_null == 0 || in.rows == 0) return 0;
        if (d.non_null == d.rows) return in.rows;
        // count through the row ids on the host (rare: VARCHAR join keys and
        // type-mismatched output columns)
        const Buf&            vec = d.type == HJ_VARCHAR ? d.locs : d.tagged;
        std::vector<uint32_t> rid(in.rows);
        std::vector<uint64_t> v(d.rows);
        HJ_CUDA(cudaMemcpyAsync(rid.data(), in.srcs[cr.src].rid->p, in.rows * 4, cudaMemcpyDeviceToHost, c->st));
        HJ_CUDA(cudaMemcpyAsync(v.data(), vec->p, d.rows * 8, cudaMemcpyDeviceToHost, c->st));
        HJ_CUDA(cudaStreamSynchronize(c->st));
        uint64_t k = 0;
        for (uint32_t r : rid) k += v[r] != 0;
        return k;
    }

    KeyCol key_col(const Inter& in, const ColRef& cr) {
        DevColumn& d = column(cr.table, cr.col);
        KeyCol     k{};
        // the reference loops over the key column's own rows (execute.cpp:78,88)
        k.n = in.srcs[cr.src].rid ? in.rows : std::min(in.rows, d.rows);
        if (d.type != HJ_INT32 || d.rows == 0) {  // INT64/FP64 key: the reference's key column is empty
            k.n = 0;
            return k;
        }
        k.col = d.icol();
        k.rid = in.srcs[cr.src].rid ? in.srcs[cr.src].rid->as<uint32_t>() : nullptr;
        return k;
    }

    Inter join(const hj_node_desc& n) {
        Inter left  = run(n.left);
        Inter right = run(n.right);
        const bool bl = n.build_left != 0;
        Inter& B = bl ? left : right;
        Inter& P = bl ? right : left;
        const uint64_t battr = bl ? n.left_attr : n.right_attr;
        const uint64_t pattr = bl ? n.right_attr : n.left_attr;
        if (battr >= B.cols.size() || pattr >= P.cols.size())
            throw Error(HJ_ERR_INVALID, "join attribute out of range");
        const ColRef bk = B.cols[battr], pk = P.cols[pattr];
        // A filtered build side is compacted; a filtered probe side is read raw
        // and its predicate evaluated by the probe's count pass (option
        // "fuse_filters", else compacted too).
        compact(B);
        if (!c->fuse_filters) compact(P);
        // Non-INT32 join keys: the reference throws on the first non-NULL value
        // (execute.cpp:81,130).
        for (auto [in, cr] : {std::pair<Inter*, ColRef>{&B, bk}, std::pair<Inter*, ColRef>{&P, pk}}) {
            DevColumn& d = column(cr.table, cr.col);
            if (d.type == HJ_VARCHAR) compact(*in);
            if (d.type == HJ_VARCHAR && non_null_through(*in, cr) > 0)
                throw Error(HJ_ERR_RUNTIME, "Join key isn't of type int32_t");
        }
        // Output columns: left ++ right (execute.cpp:140-152)
        Inter out;
        std::vector<std::pair<int, int>> need;  // (side 0 probe / 1 build, source index)
        auto src_slot = [&](int side, int s) {
            for (size_t i = 0; i < need.size(); ++i)
                if (need[i] == std::make_pair(side, s)) return int(i);
            need.emplace_back(side, s);
            return int(need.size() - 1);
        };
        for (uint32_t a = 0; a < n.num_attrs; ++a) {
            const uint64_t idx = n.attrs[a].index;
            const bool     from_left = idx < left.cols.size();
            if (!from_left && idx - left.cols.size() >= right.cols.size())
                throw Error(HJ_ERR_INVALID, "output attribute out of range");
            const ColRef cr   = from_left ? left.cols[idx] : right.cols[idx - left.cols.size()];
            const bool   is_b = from_left == bl;
            out.cols.push_back(ColRef{src_slot(is_b ? 1 : 0, cr.src), cr.table, cr.col});
        }
        KeyCol bkc = key_col(B, bk), pkc = key_col(P, pk);
        pkc.filt   = P.filt;  // fused scan predicate (raw rows, no row ids)
        build_tuples += bkc.n;
        probe_tuples += pkc.n;
        Table t;
        phase("build");
        // valid build keys, when known without a device count: all rows if the
        // key column has no NULLs, its non-NULL count when read without row ids
        const DevColumn& bd   = column(bk.table, bk.col);
        int64_t          hint = -1;
        if (bkc.n == 0 || bd.non_null == bd.rows) hint = int64_t(bkc.n);
        else if (!bkc.rid) hint = int64_t(bd.non_null);
        const uint64_t bres = plan.inputs[bk.table].resident;
        std::shared_ptr<Table> cached;
        if (c->table_cache && !bkc.rid && bres) {
            const BuiltKey key{bres, bk.col, c->dir_bits, c->radix_bits, c->dir_cap_bits};
            {
                std::lock_guard<std::mutex> g(c->store->mu);
                auto it = c->store->built.find(key);
                if (it != c->store->built.end()) cached = it->second;
            }
            if (!cached) {
                auto nt = std::make_shared<Table>();
                build_table(bkc, int(c->dir_bits), int(c->radix_bits), *nt, c->pinned, c->st, hint,
                            int(c->dir_cap_bits));
                // other streams read it from now on: the build must be complete
                HJ_CUDA(cudaStreamSynchronize(c->st));
                std::lock_guard<std::mutex> g(c->store->mu);
                auto ins = c->store->built.emplace(key, nt);
                if (!ins.second) free_table(*nt, c->st);  // another slot built it meanwhile
                cached = ins.first->second;
            }
            t = *cached;
        } else {
            build_table(bkc, int(c->dir_bits), int(c->radix_bits), t, c->pinned, c->st, hint,
                        int(c->dir_cap_bits));
        }
        ++joins;
        table_tuples += t.n_tuples;
        if (t.n_tuples) dir_words += (uint64_t(1) << t.dir_bits) + 1;
        phase("probe");
        ProbeParams prm;
        prm.light_max = int(c->light_max);
        prm.group     = int(c->probe_group);
        prm.pinned    = c->pinned;
        prm.after_count = [this] { phase("probe_sync"); };
        ProbePlan* pp = nullptr;
        uint64_t total = 0;
        try {
            total = probe_count(t, pkc, prm, &pp, c->st);
            phase("probe_write");
            if (total > 0xffffffffull) throw Error(HJ_ERR_INVALID, "join result exceeds 2^32 rows");
            out.rows = total;
            std::vector<RidOut> ro;
            for (auto [side, s] : need) {
                Inter& side_in = side == 1 ? B : P;
                Buf    dst     = make_buf(std::max<uint64_t>(total, 1) * 4, c->st);
                ro.push_back(RidOut{side, side_in.srcs[s].rid ? side_in.srcs[s].rid->as<uint32_t>() : nullptr,
                                    dst->as<uint32_t>()});
                out.srcs.push_back(Source{side_in.srcs[s].table, dst});
            }
            if (total > 0) probe_write(t, pkc, pp, ro.data(), int(ro.size()), c->st);
        } catch (...) {
            probe_free(pp, c->st);
            if (!cached) free_table(t, c->st);
            throw;
        }
        probe_free(pp, c->st);
        if (!cached) free_table(t, c->st);
        out_rows += total;
        return out;
    }

    Inter run(uint64_t node) {
        if (node >= plan.num_nodes) throw Error(HJ_ERR_INVALID, "plan node out of range");
        const hj_node_desc& n = plan.nodes[node];
        if (n.kind == HJ_NODE_SCAN) {
            if (n.base_table_id >= plan.num_inputs) throw Error(HJ_ERR_INVALID, "scan table out of range");
            return scan(n);
        }
        if (n.kind != HJ_NODE_JOIN) throw Error(HJ_ERR_INVALID, "unknown node kind");
        return join(n);
    }

    void materialize(const Inter& in, const hj_node_desc& root, hj_result* res) {
        phase("materialize");
        res->cols.assign(root.num_attrs, hj_result::Col{0, 0, nullptr});
        struct IntOut {
            uint32_t        a;
            IntCol          col;
            const uint32_t* rid;
            uint64_t        rows;
        };
        std::vector<IntOut>                          iout;  // written after the VARCHAR page counts are known
        std::vector<std::pair<uint32_t, VarcharOut>> vout;  // (column, plan)
        for (uint32_t a = 0; a < root.num_attrs; ++a) {
            const ColRef&   cr  = in.cols[a];
            const int32_t   ty  = root.attrs[a].type;
            DevColumn&      d   = column(cr.table, cr.col);
            const uint32_t* rid = in.srcs[cr.src].rid ? in.srcs[cr.src].rid->as<uint32_t>() : nullptr;
            hj_result::Col& oc  = res->cols[a];
            oc.type             = ty;
            // rows of this output column: the scan column's own count at a scan root
            const uint64_t rows = in.srcs[cr.src].rid ? in.rows : d.rows;
            if (rows == 0 || (d.type != HJ_INT32 && d.type != HJ_VARCHAR)) continue;
            if (ty == HJ_INT32) {
                // A StrRef in an INT32 output column leaves the reference's bitmap
                // undefined (execute.cpp:467-485); it is rejected here.  All-NULL
                // VARCHAR rows become NULL INT32 rows (their locators read as NULL).
                IntCol col = d.icol();
                if (d.type == HJ_VARCHAR) {
                    if (non_null_through(in, cr) > 0)
                        throw Error(HJ_ERR_RUNTIME, "VARCHAR value in an INT32 output column");
                    col        = IntCol{};
                    col.tagged = d.locs->as<uint64_t>();
                }
                oc.num_pages = (rows + kDenseRows - 1) / kDenseRows;
                oc.pages     = make_buf(oc.num_pages * kPage, c->st);  // allocated while earlier work runs
                iout.push_back({a, col, rid, rows});
            } else if (ty == HJ_VARCHAR) {
                VarcharOut v{};
                if (d.type == HJ_INT32) {
                    // the reference throws on a non-NULL INT32 here (execute.cpp:561-563);
                    // an all-NULL one gives NULL strings (tagged NULL = locator NULL = 0)
                    if (non_null_through(in, cr) > 0) throw Error(HJ_ERR_RUNTIME, "not string or null");
                    v.locs = d.tagged->as<uint64_t>();
                } else {
                    v.locs       = d.locs->as<uint64_t>();
                    v.base       = d.pages->as<uint8_t>();
                    v.base_pages = d.num_pages;
                }
                v.rid = rid;
                v.n   = rows;
                vout.emplace_back(a, v);
            }
        }
        std::vector<VarcharOut*> vptr;
        for (auto& kv : vout) vptr.push_back(&kv.second);
        if (!vout.empty()) {
            phase("mat_varchar_plan");
            varchar_plan(vptr, c->st);
        }
        std::vector<uint64_t> vpages;
        cudaEvent_t           counted = nullptr;
        if (!vout.empty()) {  // one readback for the page counts of every VARCHAR column
            phase("mat_sync");
            for (size_t i = 0; i < vout.size(); ++i)
                readback(c->pinned + i, vout[i].second.tile_off + vout[i].second.ntiles, sizeof(uint64_t), true,
                         c->st);  // page-locked scratch
            HJ_CUDA(cudaEventCreateWithFlags(&counted, cudaEventDisableTiming));
            HJ_CUDA(cudaEventRecord(counted, c->st));
        }
        // the INT32 pages keep the GPU busy while the host waits for the page
        // counts and sizes the VARCHAR buffers
        phase("materialize");
        for (const IntOut& o : iout)
            launch_write_int32_pages(o.col, o.rid, o.rows, res->cols[o.a].pages->as<uint8_t>(), c->st);
        if (counted) {
            const cudaError_t e = cudaEventSynchronize(counted);
            cudaEventDestroy(counted);
            HJ_CUDA(e);
            vpages.assign(c->pinned, c->pinned + vout.size());
        }
        if (!vout.empty()) {
            phase("mat_varchar_write");
            const std::vector<uint8_t*> bufs = varchar_write(vptr, vpages, c->st);
            for (size_t i = 0; i < vout.size(); ++i) {
                hj_result::Col& oc = res->cols[vout[i].first];
                oc.num_pages       = vpages[i];
                oc.pages           = std::make_shared<DevBuf>(static_cast<void*>(bufs[i]), c->st);
            }
        }
        // ColumnarTable::num_rows = rows of the first result column (execute.cpp:437)
        if (root.num_attrs == 0) {
            res->num_rows = 0;
        } else {
            const ColRef& cr = in.cols[0];
            DevColumn&    d  = column(cr.table, cr.col);
            res->num_rows    = in.srcs[cr.src].rid ? in.rows : d.rows;
        }
    }
};

int set_err(hj_context* c, const Error& e) {
    if (c) c->err = e.what();
    return e.status;
}

template <class F>
int guarded(hj_context* c, F&& f) {
    try {
        if (c) HJ_CUDA(cudaSetDevice(c->device));
        f();
        return HJ_OK;
    } catch (const Error& e) {
        return set_err(c, e);
    } catch (const std::bad_alloc&) {
        if (c) c->err = "host allocation failed";
        return HJ_ERR_NOMEM;
    } catch (const std::exception& e) {
        if (c) c->err = e.what();
        return HJ_ERR_INVALID;
    }
}

}  // namespace
}  // namespace hj

namespace hj {

int          context_device(const hj_context* c) { return c->device; }
cudaStream_t context_stream(const hj_context* c) { return c->st; }
ProbeParams  context_probe_params(const hj_context* c) {
    ProbeParams p;
    p.light_max = int(c->light_max);
    p.group     = int(c->probe_group);
    p.pinned    = c->pinned;
    return p;
}
void         context_set_error(hj_context* c, const char* msg) { c->err = msg; }
const Table& hash_table_of(const hj_hash_table* t) { return t->t; }

void result_rebind(hj_result* r, cudaStream_t st) {
    for (auto& col : r->cols)
        if (col.pages) col.pages->st = st;
}

hj_context* context_clone(const hj_context* p) {
    hj_context* c = hj_context_create(p->device);
    if (!c) throw Error(HJ_ERR_CUDA, std::string("context for a serving slot: ") + g_create_error);
    c->store        = p->store;
    c->dir_bits     = p->dir_bits;
    c->radix_bits   = p->radix_bits;
    c->probe_group  = p->probe_group;
    c->light_max    = p->light_max;
    c->timing       = p->timing;
    c->dir_cap_bits = p->dir_cap_bits;
    c->host_access  = p->host_access;
    c->table_cache  = p->table_cache;
    c->fuse_filters = p->fuse_filters;
    return c;
}

uint64_t resident_rows(const hj_context* c, uint64_t handle) {
    std::lock_guard<std::mutex> g(c->store->mu);
    auto it = c->store->tables.find(handle);
    return it == c->store->tables.end() ? 0 : it->second->num_rows;
}

}  // namespace hj

// ===================================================================== C ABI

extern "C" {

const char* hj_version(void) { return "hjgb300 0.1 (sm_103a)"; }

void* hj_context_stream(hj_context* c) { return c ? static_cast<void*>(c->st) : nullptr; }

hj_context* hj_context_create(int device) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        hj::g_create_error = "no CUDA device available";
        return nullptr;
    }
    auto* c = new hj_context();
    try {
        if (device < 0) HJ_CUDA(cudaGetDevice(&device));
        if (device >= n) throw hj::Error(HJ_ERR_NO_DEVICE, "device index out of range");
        c->device = device;
        HJ_CUDA(cudaSetDevice(device));
        HJ_CUDA(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
        cudaMemPool_t mp;
        HJ_CUDA(cudaDeviceGetDefaultMemPool(&mp, device));
        uint64_t keep = ~0ull;  // keep freed blocks for reuse
        HJ_CUDA(cudaMemPoolSetAttribute(mp, cudaMemPoolAttrReleaseThreshold, &keep));
        HJ_CUDA(cudaMallocHost(&c->pinned, 64 * sizeof(uint64_t)));
        int pageable = 0;
        if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess) {
            cudaGetLastError();
            pageable = 0;
        }
        c->ats_capable = pageable != 0;
        c->store         = std::make_shared<hj::Store>();
        c->store->device = device;
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        c->pool           = std::make_unique<hj::ThreadPool>(std::min(hw, 16u) - 1);
    } catch (const hj::Error& e) {
        hj::g_create_error = e.what();
        hj_context_destroy(c);
        return nullptr;
    }
    return c;
}

void hj_context_destroy(hj_context* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->st) cudaStreamSynchronize(c->st);
    c->store.reset();  // the last owner frees the resident tables
    if (c->st) {
        hj::flush_stream(c->st);
        cudaStreamSynchronize(c->st);
    }
    for (auto e : c->slot_ev)
        if (e) cudaEventDestroy(e);
    if (c->staging) cudaFreeHost(c->staging);
    if (c->pinned) cudaFreeHost(c->pinned);
    c->pool.reset();
    if (c->st) cudaStreamDestroy(c->st);
    delete c;
}

const char* hj_last_error(const hj_context* c) {
    return c ? c->err.c_str() : hj::g_create_error.c_str();
}

int hj_set_option(hj_context* c, const char* name, int64_t v) {
    if (!c || !name) return HJ_ERR_INVALID;
    const std::string n = name;
    if (n == "dir_bits") c->dir_bits = v;
    else if (n == "radix_bits") c->radix_bits = v;
    else if (n == "probe_group") {
        if (v != 1 && v != 2 && v != 4 && v != 8 && v != 16 && v != 32) return HJ_ERR_INVALID;
        c->probe_group = v;
    } else if (n == "light_max") {
        if (v < 1) return HJ_ERR_INVALID;
        c->light_max = v;
    } else if (n == "timing") {
        c->timing = v != 0;
    } else if (n == "dir_cap_bits") {
        if (v < 0 || v > 32) return HJ_ERR_INVALID;
        c->dir_cap_bits = v;
    } else if (n == "host_access") {
        c->host_access = v != 0;
    } else if (n == "table_cache") {
        c->table_cache = v != 0;
    } else if (n == "fuse_filters") {
        c->fuse_filters = v != 0;
    } else if (n == "batch_load_pct") {
        if (v < 10 || v > 800) return HJ_ERR_INVALID;
        c->batch_load_pct = v;
    } else if (n == "batch_graph") {
        c->batch_graph = v != 0;
    } else if (n == "batch_part_log2") {
        if (v < 8 || v > 13) return HJ_ERR_INVALID;
        c->batch_part_log2 = v;
    } else {
        c->err = "unknown option " + n;
        return HJ_ERR_INVALID;
    }
    return HJ_OK;
}

int hj_get_option(const hj_context* c, const char* name, int64_t* v) {
    if (!c || !name || !v) return HJ_ERR_INVALID;
    const std::string n = name;
    if (n == "dir_bits") *v = c->dir_bits;
    else if (n == "radix_bits") *v = c->radix_bits;
    else if (n == "probe_group") *v = c->probe_group;
    else if (n == "light_max") *v = c->light_max;
    else if (n == "timing") *v = c->timing;
    else if (n == "dir_cap_bits") *v = c->dir_cap_bits;
    else if (n == "host_access") *v = c->host_access;
    else if (n == "host_access_capable") *v = c->ats_capable;
    else if (n == "table_cache") *v = c->table_cache;
    else if (n == "fuse_filters") *v = c->fuse_filters;
    else if (n == "batch_load_pct") *v = c->batch_load_pct;
    else if (n == "batch_graph") *v = c->batch_graph;
    else if (n == "batch_part_log2") *v = c->batch_part_log2;
    else return HJ_ERR_INVALID;
    return HJ_OK;
}

int hj_table_upload(hj_context* c, const hj_table_desc* t, uint64_t* handle) {
    if (!c || !t || !handle) return HJ_ERR_INVALID;
    return hj::guarded(c, [&] {
        auto dt = hj::upload_table(c, *t, {});
        HJ_CUDA(cudaStreamSynchronize(c->st));
        std::lock_guard<std::mutex> g(c->store->mu);
        const uint64_t              h = c->store->next_handle++;
        c->store->tables[h]           = dt;
        *handle          = h;
    });
}

int hj_table_prepare(hj_context* c, uint64_t handle) {
    if (!c) return HJ_ERR_INVALID;
    return hj::guarded(c, [&] {
        std::shared_ptr<hj::DevTable> dt;
        {
            std::lock_guard<std::mutex> g(c->store->mu);
            auto it = c->store->tables.find(handle);
            if (it == c->store->tables.end()) throw hj::Error(HJ_ERR_INVALID, "unknown table handle");
            dt = it->second;
        }
        // decode into a private copy, then publish it: executions that copied
        // the table meanwhile keep decoding per call
        auto nt = std::make_shared<hj::DevTable>(*dt);
        for (auto& col : nt->cols) {
            if (col.predecoded || (col.type != HJ_INT32 && col.type != HJ_VARCHAR)) continue;
            hj::decode_kernels(c->st, col);
            col.predecoded = true;
        }
        HJ_CUDA(cudaStreamSynchronize(c->st));
        std::lock_guard<std::mutex> g(c->store->mu);
        auto it = c->store->tables.find(handle);
        if (it != c->store->tables.end()) it->second = nt;
    });
}

int hj_table_release(hj_context* c, uint64_t handle) {
    if (!c) return HJ_ERR_INVALID;
    return hj::guarded(c, [&] {
        std::lock_guard<std::mutex> g(c->store->mu);
        if (!c->store->tables.erase(handle)) throw hj::Error(HJ_ERR_INVALID, "unknown table handle");
        c->store->drop_built(handle);
        HJ_CUDA(cudaStreamSynchronize(c->st));
    });
}

int hj_execute(hj_context* c, const hj_plan_desc* plan, hj_result** out) {
    if (!c || !plan || !out) return HJ_ERR_INVALID;
    *out = nullptr;
    auto* res = new hj_result();
    const uint64_t launches0 = hj::g_kernel_launches.load();
    const int rc = hj::guarded(c, [&] {
        if (plan->root >= plan->num_nodes) throw hj::Error(HJ_ERR_INVALID, "plan root out of range");
        hj::Exec ex{c, *plan, {}};
        // which (table, column) pairs do the scans read?
        std::vector<std::vector<bool>> want(plan->num_inputs);
        for (uint32_t i = 0; i < plan->num_inputs; ++i) {
            const hj_table_desc& t = plan->inputs[i];
            want[i].assign(t.resident ? 0 : t.num_columns, false);
        }
        for (uint32_t i = 0; i < plan->num_nodes; ++i) {
            const hj_node_desc& n = plan->nodes[i];
            if (n.kind != HJ_NODE_SCAN) continue;
            if (n.base_table_id >= plan->num_inputs) throw hj::Error(HJ_ERR_INVALID, "scan table out of range");
            const hj_table_desc& t = plan->inputs[n.base_table_id];
            for (uint32_t a = 0; a < n.num_attrs; ++a) {
                const uint64_t col = n.attrs[a].index;
                if (t.resident) continue;
                if (col >= t.num_columns) throw hj::Error(HJ_ERR_INVALID, "scan column out of range");
                want[n.base_table_id][col] = true;
            }
            for (uint32_t f = 0; f < n.num_filters && n.filters && !t.resident; ++f)
                if (n.filters[f].column < t.num_columns) want[n.base_table_id][n.filters[f].column] = true;
        }
        ex.phase("upload");
        // the store's upload turn, held while this plan's host tables are copied
        // (upload_table returns once its copies are complete)
        std::unique_lock<std::mutex> upload_turn(c->store->upload_mu, std::defer_lock);
        bool host_inputs = false;
        for (uint32_t i = 0; i < plan->num_inputs; ++i) host_inputs |= plan->inputs[i].resident == 0;
        if (host_inputs) upload_turn.lock();
        for (uint32_t i = 0; i < plan->num_inputs; ++i) {
            const hj_table_desc& t = plan->inputs[i];
            if (t.resident) {
                std::lock_guard<std::mutex> g(c->store->mu);
                auto it = c->store->tables.find(t.resident);
                if (it == c->store->tables.end()) throw hj::Error(HJ_ERR_INVALID, "unknown resident table");
                // decoded state is per call unless the table was prepared:
                // copy the column records, share the pages (and decoded arrays)
                auto dt = std::make_shared<hj::DevTable>(*it->second);
                for (auto& col : dt->cols) {
                    col.decoded = false;
                    if (!col.predecoded) col.plain = col.tagged = col.locs = nullptr;
                }
                ex.tables.push_back(dt);
            } else {
                ex.tables.push_back(hj::upload_table(c, t, want[i]));
            }
        }
        if (host_inputs) upload_turn.unlock();
        // copy_scan of every scanned column, before any join (execute.cpp:575-582)
        ex.phase("decode");
        for (uint32_t i = 0; i < plan->num_nodes; ++i) {
            const hj_node_desc& n = plan->nodes[i];
            if (n.kind != HJ_NODE_SCAN) continue;
            for (uint32_t a = 0; a < n.num_attrs; ++a) {
                if (n.attrs[a].index >= ex.tables[n.base_table_id]->cols.size())
                    throw hj::Error(HJ_ERR_INVALID, "scan column out of range");
                ex.column(uint32_t(n.base_table_id), uint32_t(n.attrs[a].index));
            }
            for (uint32_t f = 0; f < n.num_filters && n.filters; ++f)
                if (n.filters[f].column < ex.tables[n.base_table_id]->cols.size())
                    ex.column(uint32_t(n.base_table_id), uint32_t(n.filters[f].column));
        }
        hj::Inter root = ex.run(plan->root);
        ex.compact(root);  // a filtered scan as the root
        ex.materialize(root, plan->nodes[plan->root], res);
        ex.collect(res->phase_ms);
        HJ_CUDA(cudaStreamSynchronize(c->st));
        res->build_tuples = ex.build_tuples;
        res->probe_tuples = ex.probe_tuples;
        res->output_rows  = ex.out_rows;
        res->dir_words    = ex.dir_words;
        res->table_tuples = ex.table_tuples;
        res->joins        = ex.joins;
    });
    res->kernel_launches = hj::g_kernel_launches.load() - launches0;
    if (rc != HJ_OK) {
        delete res;
        cudaStreamSynchronize(c->st);
        return rc;
    }
    *out = res;
    return HJ_OK;
}

int hj_result_shape(const hj_result* r, uint64_t* num_rows, uint32_t* num_columns) {
    if (!r) return HJ_ERR_INVALID;
    if (num_rows) *num_rows = r->num_rows;
    if (num_columns) *num_columns = uint32_t(r->cols.size());
    return HJ_OK;
}

int hj_result_column(const hj_result* r, uint32_t col, int32_t* type, uint64_t* num_pages) {
    if (!r || col >= r->cols.size()) return HJ_ERR_INVALID;
    if (type) *type = r->cols[col].type;
    if (num_pages) *num_pages = r->cols[col].num_pages;
    return HJ_OK;
}

int hj_host_register(void* ptr, uint64_t bytes) {
    if (!ptr || !bytes) return HJ_ERR_INVALID;
    const cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return e == cudaErrorHostMemoryAlreadyRegistered ? HJ_ERR_INVALID : HJ_ERR_CUDA;
    }
    return HJ_OK;
}

int hj_host_unregister(void* ptr) {
    if (!ptr) return HJ_ERR_INVALID;
    const cudaError_t e = cudaHostUnregister(ptr);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return e == cudaErrorHostMemoryNotRegistered ? HJ_ERR_INVALID : HJ_ERR_CUDA;
    }
    return HJ_OK;
}

int hj_result_copy_pages(hj_context* c, const hj_result* r, uint32_t col, void* const* dst) {
    if (!c || !r || col >= r->cols.size()) return HJ_ERR_INVALID;
    return hj::guarded(c, [&] {
        const auto& oc = r->cols[col];
        if (!oc.num_pages) return;
        const auto runs = hj::locked_runs(dst, oc.num_pages, 64);
        if (!runs.empty()) {  // page-locked destination: copy engines, one copy per run
            for (const auto& q : runs)
                HJ_CUDA(cudaMemcpyAsync(dst[q.first], oc.pages->as<uint8_t>() + q.first * hj::kPage,
                                        q.count * hj::kPage, cudaMemcpyDeviceToHost, c->st));
            HJ_CUDA(cudaStreamSynchronize(c->st));
        } else if (hj::direct_host_access(c)) {
            hj::launch_scatter_host_pages(oc.pages->as<uint8_t>(), oc.num_pages, dst, nullptr, c->st);
            HJ_CUDA(cudaStreamSynchronize(c->st));
        } else {
            hj::download_pages(c, oc.pages->as<uint8_t>(), oc.num_pages, dst, nullptr);
        }
    });
}

int hj_result_copy_contiguous(hj_context* c, const hj_result* r, uint32_t col, void* dst) {
    if (!c || !r || col >= r->cols.size()) return HJ_ERR_INVALID;
    return hj::guarded(c, [&] {
        const auto& oc = r->cols[col];
        if (!oc.num_pages) return;
        if (hj::locked_range(dst, oc.num_pages * hj::kPage)) {  // page-locked destination: copy engine
            HJ_CUDA(cudaMemcpyAsync(dst, oc.pages->p, oc.num_pages * hj::kPage, cudaMemcpyDeviceToHost, c->st));
            HJ_CUDA(cudaStreamSynchronize(c->st));
        } else if (hj::direct_host_access(c)) {
            hj::launch_scatter_host_pages(oc.pages->as<uint8_t>(), oc.num_pages, nullptr, dst, c->st);
            HJ_CUDA(cudaStreamSynchronize(c->st));
        } else {
            hj::download_pages(c, oc.pages->as<uint8_t>(), oc.num_pages, nullptr, static_cast<uint8_t*>(dst));
        }
    });
}

int hj_result_stats(const hj_result* r, uint64_t* b, uint64_t* p, uint64_t* o) {
    if (!r) return HJ_ERR_INVALID;
    if (b) *b = r->build_tuples;
    if (p) *p = r->probe_tuples;
    if (o) *o = r->output_rows;
    return HJ_OK;
}

int hj_result_phase_ms(const hj_result* r, const char* phase, double* ms) {
    if (!r || !phase || !ms) return HJ_ERR_INVALID;
    if (std::string(phase) == "launches") {
        *ms = double(r->kernel_launches);
        return HJ_OK;
    }
    auto it = r->phase_ms.find(phase);
    *ms     = it == r->phase_ms.end() ? 0.0 : it->second;
    return HJ_OK;
}

int hj_result_counter(const hj_result* r, const char* name, uint64_t* value) {
    if (!r || !name || !value) return HJ_ERR_INVALID;
    const std::string n(name);
    if (n == "dir_words") *value = r->dir_words;
    else if (n == "table_tuples") *value = r->table_tuples;
    else if (n == "joins") *value = r->joins;
    else if (n == "launches") *value = r->kernel_launches;
    else return HJ_ERR_INVALID;
    return HJ_OK;
}

void hj_result_free(hj_result* r) { delete r; }

// ---- hash table on device columns ----------------------------------------

int hj_table_build(hj_context* c, const int32_t* keys, const uint32_t* valid, uint64_t n,
                   int32_t dir_bits, hj_hash_table** out) {
    if (!c || !out || (n > 0 && !keys)) return HJ_ERR_INVALID;
    *out = nullptr;
    auto* ht = new hj_hash_table();
    ht->st   = c->st;
    const int rc = hj::guarded(c, [&] {
        if (n > 0xffffffffull) throw hj::Error(HJ_ERR_INVALID, "more than 2^32 build rows");
        hj::IntCol col;
        col.plain = keys;
        col.valid = valid;
        hj::KeyCol kc{col, nullptr, n};
        hj::build_table(kc, dir_bits, int(c->radix_bits), ht->t, c->pinned, c->st, valid ? -1 : int64_t(n));
        HJ_CUDA(cudaStreamSynchronize(c->st));
    });
    if (rc != HJ_OK) {
        delete ht;
        return rc;
    }
    *out = ht;
    return HJ_OK;
}

int hj_table_info(const hj_hash_table* t, uint32_t* dir_bits, uint64_t* num_tuples, const uint64_t** dir,
                  const int32_t** keys, const uint32_t** rows) {
    if (!t) return HJ_ERR_INVALID;
    if (dir_bits) *dir_bits = t->t.dir_bits;
    if (num_tuples) *num_tuples = t->t.n_tuples;
    if (dir) *dir = t->t.dir;
    if (keys) *keys = t->t.keys;
    if (rows) *rows = t->t.rows;
    return HJ_OK;
}

int hj_table_probe(hj_context* c, const hj_hash_table* t, const int32_t* keys, const uint32_t* valid,
                   uint64_t n, uint32_t* out_probe, uint32_t* out_build, uint64_t capacity,
                   uint64_t* num_matches) {
    if (!c || !t || !num_matches || (n > 0 && !keys)) return HJ_ERR_INVALID;
    int status = HJ_OK;
    const int rc = hj::guarded(c, [&] {
        if (n > 0xffffffffull) throw hj::Error(HJ_ERR_INVALID, "more than 2^32 probe rows");
        hj::IntCol col;
        col.plain = keys;
        col.valid = valid;
        hj::KeyCol      pk{col, nullptr, n};
        hj::ProbeParams prm;
        prm.light_max = int(c->light_max);
        prm.group     = int(c->probe_group);
        prm.pinned    = c->pinned;
        hj::ProbePlan* pp = nullptr;
        try {
            const uint64_t total = hj::probe_count(t->t, pk, prm, &pp, c->st);
            *num_matches         = total;
            if (total > capacity) {
                status = HJ_ERR_CAPACITY;
            } else if (total > 0) {
                if (!out_probe || !out_build) throw hj::Error(HJ_ERR_INVALID, "null output buffer");
                hj::RidOut ro[2] = {{0, nullptr, out_probe}, {1, nullptr, out_build}};
                hj::probe_write(t->t, pk, pp, ro, 2, c->st);
            }
        } catch (...) {
            hj::probe_free(pp, c->st);
            throw;
        }
        hj::probe_free(pp, c->st);
        HJ_CUDA(cudaStreamSynchronize(c->st));
    });
    if (rc != HJ_OK) return rc;
    if (status != HJ_OK) c->err = "output capacity too small";
    return status;
}

int hj_batch_execute(hj_context* c, const hj_batch_instance* inst, uint32_t n, int32_t mode, uint64_t* rows,
                     uint64_t* checksums, uint32_t* recomputed) {
    if (!c || (n > 0 && (!inst || !rows || !checksums))) return HJ_ERR_INVALID;
    if (mode != HJ_BATCH_PERSISTENT && mode != HJ_BATCH_PLAIN) return HJ_ERR_INVALID;
    if (recomputed) *recomputed = 0;
    return hj::guarded(c, [&] {
        std::vector<hj::BatchInstance> B(n);
        for (uint32_t i = 0; i < n; ++i) {
            if (inst[i].num_relations < 2 || !inst[i].relations)
                throw hj::Error(HJ_ERR_INVALID, "batch instance " + std::to_string(i) + " needs >= 2 relations");
            for (uint32_t r = 0; r < inst[i].num_relations; ++r) {
                const hj_batch_relation& x = inst[i].relations[r];
                B[i].rels.push_back({x.keys, x.payload, x.rows});
            }
        }
        const hj::ProbeParams prm = hj::context_probe_params(c);
        auto plain = [&](uint32_t i) {
            hj::plain_instance(B[i], prm, int(c->dir_bits), int(c->radix_bits), int(c->dir_cap_bits), rows[i],
                               checksums[i], c->st);
        };
        if (mode == HJ_BATCH_PLAIN) {
            for (uint32_t i = 0; i < n; ++i) plain(i);
            return;
        }
        hj::BatchOptions o;
        o.load       = double(c->batch_load_pct) / 100.0;
        o.graph      = c->batch_graph != 0;
        o.part_rows_log2 = int(c->batch_part_log2);
        std::vector<uint64_t> r, s;
        const std::vector<uint32_t> redo = hj::batch_execute(B, o, r, s, c->st);
        std::copy(r.begin(), r.end(), rows);
        std::copy(s.begin(), s.end(), checksums);
        for (uint32_t i : redo) plain(i);
        if (recomputed) *recomputed = uint32_t(redo.size());
    });
}

int hj_batch_generate(hj_context* c, uint64_t seed, uint32_t instance, uint32_t relation, uint64_t build_rows,
                      uint32_t match_q24, uint64_t rows, int32_t* keys, int32_t* payload) {
    if (!c) return HJ_ERR_INVALID;
    return hj::guarded(c, [&] {
        hj::launch_batch_generate(seed, instance, relation, build_rows, match_q24, rows, keys, payload, c->st);
    });
}

void hj_table_free(hj_hash_table* t) {
    if (!t) return;
    hj::free_table(t->t, t->st);
    cudaStreamSynchronize(t->st);
    delete t;
}

}  // extern "C"
