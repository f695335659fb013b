// Test infrastructure (oracle only) -- the CPU restatement of the reference's
// join path.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
// leg load it, as the checker or as the timed CPU baseline; the shipped GPU
// library never links, loads or calls it.
//
// It restates Contest::execute of eleanalt/hash-join-optimizer step by step,
// with the same data structures and the same host-thread parallelism, so that
// (a) its results are those of the reference, and (b) timing it measures the
// reference's algorithm on whatever host it runs on (the compiled reference,
// oracle/_ref, cannot be built on a machine without the reference sources).
//
//   execute / execute_impl        src/execute.cpp:584-608
//   execute_hash_join             src/execute.cpp:188-225
//   JoinAlgorithm::run            src/execute.cpp:26-186
//   copy_scan / col_is_dense      src/execute.cpp:251-369
//   deref_str_ref                 src/execute.cpp:371-428
//   table_to_columnar             src/execute.cpp:431-573
//   PartitionedDirectoryHash      include/partitioned_directory_hash.h:15-217
//   column_t                      include/column_t.h:11-82
//   merge_column_pages            include/column_merge.h:7-31
//   value_t / StrRef              include/value_t.h:7-127
//
// Two deliberate differences, both where the reference cannot return:
//  * a non-INT32 join key raises std::runtime_error on the calling thread (the
//    reference throws it inside a std::thread, which ends the process);
//  * with one join thread the reference shifts a 64-bit hash by 64
//    (partitioned_directory_hash.h:100,111, undefined); here partition 0 is used.
#include <algorithm>
#include <chrono>
#include <array>
#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../include/hj_api.h"
#include "oracle_result.h"

namespace oracle {

constexpr size_t PAGE  = 8192;
constexpr size_t DENSE = 1984;  // rows of a dense INT32 page (column_t.h:15)

// ---- value_t / StrRef (value_t.h:7-127) -----------------------------------
constexpr uint64_t TAG_INT = 1ull << 62, TAG_STR = 1ull << 63, LONG_BIT = 1ull << 61;

inline uint64_t v_int(int32_t x) { return uint64_t(uint32_t(x)) | TAG_INT; }
inline bool     v_null(uint64_t v) { return (v >> 62) == 0; }
inline bool     v_isint(uint64_t v) { return (v >> 62) == 1; }
inline bool     v_isstr(uint64_t v) { return (v >> 62) == 2; }

uint64_t strref(bool is_long, uint64_t table, uint64_t col, uint64_t page, uint64_t off) {
    auto chk = [](const char* what, uint64_t v, uint64_t mask) {
        if (v > mask)
            throw std::out_of_range(std::string("StrRef ") + what + " overflow: " + std::to_string(v)
                                    + " > " + std::to_string(mask));
    };
    chk("table", table, 1023);
    chk("column", col, 1023);
    chk("page", page, (1u << 18) - 1);
    chk("offset", off, 65535);
    uint64_t r = is_long ? LONG_BIT : 0;
    r |= table << 51 | col << 41 | page << 23 | off << 7;
    return (r & ~(3ull << 62)) | TAG_STR;
}

inline uint16_t rd16(const uint8_t* p) {
    uint16_t v;
    std::memcpy(&v, p, 2);
    return v;
}
inline int32_t rd32(const uint8_t* p) {
    int32_t v;
    std::memcpy(&v, p, 4);
    return v;
}

// ---- column_t (column_t.h:11-82) ------------------------------------------
struct ColumnT {
    size_t                                                 rows = 0;
    std::vector<std::unique_ptr<std::array<uint64_t, 1024>>> pages;
    const hj_column_desc*                                  direct = nullptr;

    void append(uint64_t v) {
        const size_t off = rows & 1023;
        if (off == 0) pages.push_back(std::make_unique<std::array<uint64_t, 1024>>());
        (*pages.back())[off] = v;
        ++rows;
    }
    uint64_t get(size_t r) const {
        if (direct) {
            const uint8_t* pg = static_cast<const uint8_t*>(direct->pages[r / DENSE]);
            return v_int(rd32(pg + 4 + 4 * (r % DENSE)));
        }
        return (*pages[r >> 10])[r & 1023];
    }
};
using Result = std::vector<ColumnT>;

// merge_column_pages (column_merge.h:7-31): move pages when dst is empty.
void merge(ColumnT& dst, ColumnT& src) {
    if (!src.direct && dst.rows == 0 && dst.pages.empty() && !dst.direct) {
        dst.pages = std::move(src.pages);
        dst.rows  = src.rows;
        src.pages.clear();
        src.rows = 0;
        return;
    }
    for (size_t i = 0; i < src.rows; ++i) dst.append(src.get(i));
}

size_t num_threads_env() {
    if (const char* s = std::getenv("SIGMOD_THREADS")) {
        long v = std::strtol(s, nullptr, 10);
        if (v > 0) return size_t(v);
    }
    return std::max(1u, std::thread::hardware_concurrency());
}

// Runs fn(i) for i in [0, n) on up to `threads` threads, rethrowing the first
// exception on the caller.
template <class F>
void parallel_for(size_t n, size_t threads, F&& fn) {
    std::atomic<size_t>  next{0};
    std::exception_ptr   err;
    std::mutex           mu;
    std::vector<std::thread> pool;
    threads = std::max<size_t>(1, std::min(threads, n));
    for (size_t t = 0; t < threads; ++t)
        pool.emplace_back([&] {
            try {
                for (size_t i; (i = next.fetch_add(1)) < n;) fn(i);
            } catch (...) {
                std::lock_guard<std::mutex> g(mu);
                if (!err) err = std::current_exception();
                next = n;
            }
        });
    for (auto& th : pool) th.join();
    if (err) std::rethrow_exception(err);
}

// ---- copy_scan (execute.cpp:251-369) ----------------------------------------
bool col_is_dense(const hj_column_desc& c) {
    for (uint64_t p = 0; p < c.num_pages; ++p) {
        const uint8_t* pg = static_cast<const uint8_t*>(c.pages[p]);
        if (rd16(pg) != uint16_t(rd16(pg + 2))) return false;
    }
    return true;
}

Result copy_scan(const hj_table_desc& t, size_t table_id, const hj_attr* attrs, uint32_t na) {
    Result res(na);
    // The reference spreads output columns over its 12-thread filter pool
    // (inner_column.h:107, execute.cpp:366).
    parallel_for(na, 12, [&](size_t oc) {
        const size_t          in_col = attrs[oc].index;
        const hj_column_desc& col    = t.columns[in_col];
        ColumnT&              out    = res[oc];
        if (col.type == HJ_INT32 && col_is_dense(col)) {
            out.direct = &col;
            out.rows   = t.num_rows;
            return;
        }
        for (uint64_t p = 0; p < col.num_pages; ++p) {
            const uint8_t* pg = static_cast<const uint8_t*>(col.pages[p]);
            const uint16_t nr = rd16(pg);
            if (col.type == HJ_INT32) {
                const uint8_t* bm = pg + PAGE - (nr + 7) / 8;
                uint16_t       d  = 0;
                for (uint16_t i = 0; i < nr; ++i) {
                    if (bm[i / 8] & (1u << (i % 8))) out.append(v_int(rd32(pg + 4 + 4 * d++)));
                    else                             out.append(0);
                }
            } else if (col.type == HJ_VARCHAR) {
                if (nr == 0xffff) {
                    out.append(strref(true, table_id, in_col, p, 0));
                } else if (nr == 0xfffe) {
                    continue;
                } else {
                    const uint8_t* bm = pg + PAGE - (nr + 7) / 8;
                    uint16_t       d  = 0;
                    for (uint16_t i = 0; i < nr; ++i) {
                        if (bm[i / 8] & (1u << (i % 8)))
                            out.append(strref(false, table_id, in_col, p, d++));
                        else
                            out.append(0);
                    }
                }
            }
            // INT64 / FP64: the reference's switch has no case; column stays empty.
        }
    });
    return res;
}

// ---- PartitionedDirectoryHash (partitioned_directory_hash.h:15-217) -------
inline uint64_t splitmix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

size_t next_pow2(size_t x) {
    size_t p = 1;
    while (p < x) p <<= 1;
    return p;
}

struct DirTuple {
    uint64_t hash;
    uint32_t key;
    size_t   row;
};

struct PDHash {
    std::vector<uint64_t> store;       // directory[-1 .. dir_size)
    uint64_t*             dir = nullptr;
    std::vector<DirTuple> tuples;
    size_t                parts = 0, shift = 0, dir_bits = 0;

    void init(size_t num_parts, size_t bits) {
        parts    = next_pow2(num_parts);
        dir_bits = bits;
        shift    = 64 - bits;
        store.assign((1ull << bits) + 1, 0);
        dir = store.data() + 1;
    }

    // key_of(row) -> -1 for NULL, else the key as uint32.
    template <class KeyOf>
    void build(size_t rows, size_t threads, KeyOf&& key_of) {
        const unsigned lg = unsigned(__builtin_ctzll(parts));
        // Phase 1: each thread splits its row range into per-partition buffers
        // (the reference's SlabAllocator chunks, slab_allocator.h:72-106).
        std::vector<std::vector<std::vector<DirTuple>>> tls(
            threads, std::vector<std::vector<DirTuple>>(parts));
        parallel_for(threads, threads, [&](size_t tid) {
            const size_t chunk = (rows + threads - 1) / threads;
            const size_t b = tid * chunk, e = std::min(rows, b + chunk);
            for (size_t r = b; r < e; ++r) {
                int64_t k = key_of(r);
                if (k < 0) continue;
                const uint64_t h    = splitmix64(uint64_t(uint32_t(k)));
                const size_t   part = lg == 0 ? 0 : size_t(h >> (64 - lg));
                tls[tid][part].push_back(DirTuple{h, uint32_t(k), r});
            }
        });
        // Phase 2: partition counts and offsets.
        std::vector<size_t> off(parts + 1, 0);
        for (size_t p = 0; p < parts; ++p) {
            size_t s = 0;
            for (size_t t = 0; t < threads; ++t) s += tls[t][p].size();
            off[p + 1] = off[p] + s;
        }
        tuples.resize(off[parts]);
        dir[-1] = 0;
        // Phase 3: per partition count -> prefix sum -> scatter.
        parallel_for(parts, threads, [&](size_t p) {
            if (off[p + 1] == off[p]) return;
            const uint64_t k = dir_bits;
            const uint64_t s = (uint64_t(p) << k) / parts, e = (uint64_t(p + 1) << k) / parts;
            for (size_t t = 0; t < threads; ++t)
                for (const auto& tp : tls[t][p]) {
                    const uint64_t slot = tp.hash >> shift;
                    dir[slot] += 1ull << 16;
                    dir[slot] |= uint16_t(tp.hash);
                }
            uint64_t cur = off[p];
            for (uint64_t i = s; i < e; ++i) {
                const uint64_t cnt = dir[i] >> 16;
                dir[i] = (cur << 16) | uint16_t(dir[i]);
                cur += cnt;
            }
            for (size_t t = 0; t < threads; ++t)
                for (const auto& tp : tls[t][p]) {
                    const uint64_t slot = tp.hash >> shift;
                    tuples[dir[slot] >> 16] = tp;
                    dir[slot] += 1ull << 16;
                }
        });
    }

    template <class F>
    void probe(uint32_t key, F&& f) const {
        const uint64_t h = splitmix64(uint64_t(key)), slot = h >> shift;
        const uint64_t end = dir[slot] >> 16;
        const uint64_t beg = (slot == 0 ? dir[-1] : dir[slot - 1]) >> 16;
        for (uint64_t i = beg; i < end; ++i)
            if (tuples[i].key == key) f(tuples[i].row);
    }
};

// Tuples the last execute() built and probed (summed over its joins), and
// its duration without the copy into the oracle_result buffers.
uint64_t g_build_tuples = 0, g_probe_tuples = 0;
double   g_exec_seconds = 0;

// ---- JoinAlgorithm::run (execute.cpp:26-186) ------------------------------
Result hash_join(bool build_left, Result& left, Result& right, size_t left_attr, size_t right_attr,
                 const hj_attr* attrs, uint32_t na) {
    Result&      build = build_left ? left : right;
    Result&      probe = build_left ? right : left;
    const size_t bcol  = build_left ? left_attr : right_attr;
    const size_t pcol  = build_left ? right_attr : left_attr;
    Result       results(na);

    const size_t threads = num_threads_env();
    ColumnT&     bkey    = build[bcol];
    ColumnT&     pkey    = probe[pcol];
    g_build_tuples += bkey.rows;
    g_probe_tuples += pkey.rows;

    PDHash index;
    index.init(threads, 16);
    index.build(bkey.rows, threads, [&](size_t r) -> int64_t {
        const uint64_t v = bkey.get(r);
        if (v_null(v)) return -1;
        if (!v_isint(v)) throw std::runtime_error("Join key isn't of type int32_t");
        return int64_t(uint32_t(v));
    });

    const size_t chunk_rows = 4096, np = pkey.rows, nchunks = (np + chunk_rows - 1) / chunk_rows;
    std::vector<Result> chunk_out(nchunks);
    const size_t        lsize = left.size();
    parallel_for(nchunks, threads, [&](size_t cid) {
        Result out(na);
        const size_t b = cid * chunk_rows, e = std::min(np, b + chunk_rows);
        for (size_t r = b; r < e; ++r) {
            const uint64_t v = pkey.get(r);
            if (v_null(v)) continue;
            if (!v_isint(v)) throw std::runtime_error("Join key isn't of type int32_t");
            index.probe(uint32_t(v), [&](size_t brow) {
                for (uint32_t a = 0; a < na; ++a) {
                    const size_t c = attrs[a].index;
                    uint64_t     val;
                    if (build_left) val = c < lsize ? build[c].get(brow) : probe[c - lsize].get(r);
                    else            val = c < lsize ? probe[c].get(r) : build[c - lsize].get(brow);
                    out[a].append(val);
                }
            });
        }
        chunk_out[cid] = std::move(out);
    });
    // Deterministic merge in chunk order (execute.cpp:167-184).
    for (auto& co : chunk_out)
        for (uint32_t a = 0; a < na; ++a) merge(results[a], co[a]);
    return results;
}

Result execute_impl(const hj_plan_desc& plan, size_t node) {
    const hj_node_desc& n = plan.nodes[node];
    // execute() receives tables already filtered by the loader; scan filters
    // have no counterpart here (tests compare them with pre-filtered plans)
    if (n.num_filters) throw std::invalid_argument("the oracle takes no scan filters");
    if (n.kind == HJ_NODE_SCAN)
        return copy_scan(plan.inputs[n.base_table_id], n.base_table_id, n.attrs, n.num_attrs);
    Result left  = execute_impl(plan, n.left);
    Result right = execute_impl(plan, n.right);
    // The key type drives a template dispatch in the reference (execute.cpp:208-222)
    // whose type parameter is never used; every instance runs the same code.
    return hash_join(n.build_left != 0, left, right, n.left_attr, n.right_attr, n.attrs, n.num_attrs);
}

// ---- deref_str_ref (execute.cpp:371-428) ----------------------------------
void deref(uint64_t v, const hj_plan_desc& plan, std::string& out) {
    const uint64_t ref   = v & ~(3ull << 62);
    const size_t   table = (ref >> 51) & 1023, col = (ref >> 41) & 1023;
    size_t         page  = (ref >> 23) & ((1u << 18) - 1);
    const size_t   off   = (ref >> 7) & 65535;
    const hj_column_desc& c  = plan.inputs[table].columns[col];
    const uint8_t*        pg = static_cast<const uint8_t*>(c.pages[page]);
    if (ref & LONG_BIT) {
        if (rd16(pg) != 0xffff) throw std::runtime_error("Page doesn't refer to long string");
        out.assign(reinterpret_cast<const char*>(pg + 4), rd16(pg + 2));
        while (++page < c.num_pages) {
            pg = static_cast<const uint8_t*>(c.pages[page]);
            if (rd16(pg) != 0xfffe) break;
            out.append(reinterpret_cast<const char*>(pg + 4), rd16(pg + 2));
        }
        return;
    }
    const uint16_t nn    = rd16(pg + 2);
    const uint8_t* data  = pg + 4 + 2 * nn;
    const uint16_t start = off == 0 ? 0 : rd16(pg + 4 + 2 * (off - 1));
    const uint16_t end   = rd16(pg + 4 + 2 * off);
    out.assign(reinterpret_cast<const char*>(data + start), size_t(end) - start);
}

// ---- table_to_columnar (execute.cpp:431-573) ------------------------------
struct PageSink {
    std::vector<std::vector<uint8_t>> pages;
    uint8_t* fresh() {
        pages.emplace_back(PAGE, 0);
        return pages.back().data();
    }
};

void wr16(uint8_t* p, uint16_t v) { std::memcpy(p, &v, 2); }

void int32_to_pages(const ColumnT& col, PageSink& sink) {
    uint16_t             nr = 0;
    std::vector<int32_t> data;
    std::vector<uint8_t> bm;
    auto save = [&] {
        uint8_t* pg = sink.fresh();
        wr16(pg, nr);
        wr16(pg + 2, uint16_t(data.size()));
        std::memcpy(pg + 4, data.data(), data.size() * 4);
        std::memcpy(pg + PAGE - bm.size(), bm.data(), bm.size());
        nr = 0;
        data.clear();
        bm.clear();
    };
    auto bit = [&](uint16_t i, bool on) {
        while (bm.size() < size_t(i) / 8 + 1) bm.push_back(0);
        if (on) bm[i / 8] |= uint8_t(1u << (i % 8));
        else    bm[i / 8] &= uint8_t(~(1u << (i % 8)));
    };
    for (size_t r = 0; r < col.rows; ++r) {
        const uint64_t v = col.get(r);
        if (v_isint(v)) {
            if (4 + (data.size() + 1) * 4 + (nr / 8 + 1) > PAGE) save();
            bit(nr, true);
            data.push_back(int32_t(uint32_t(v)));
        } else if (v_null(v)) {
            if (4 + data.size() * 4 + (nr / 8 + 1) > PAGE) save();
            bit(nr, false);
        }
        ++nr;
    }
    if (nr != 0) save();
}

void varchar_to_pages(const ColumnT& col, const hj_plan_desc& plan, PageSink& sink) {
    uint16_t              nr = 0;
    std::vector<uint8_t>  data;
    std::vector<uint16_t> offs;
    std::vector<uint8_t>  bm;
    std::string           s;
    auto save = [&] {
        uint8_t* pg = sink.fresh();
        wr16(pg, nr);
        wr16(pg + 2, uint16_t(offs.size()));
        std::memcpy(pg + 4, offs.data(), offs.size() * 2);
        std::memcpy(pg + 4 + offs.size() * 2, data.data(), data.size());
        std::memcpy(pg + PAGE - bm.size(), bm.data(), bm.size());
        nr = 0;
        data.clear();
        offs.clear();
        bm.clear();
    };
    auto bit = [&](uint16_t i, bool on) {
        while (bm.size() < size_t(i) / 8 + 1) bm.push_back(0);
        if (on) bm[i / 8] |= uint8_t(1u << (i % 8));
        else    bm[i / 8] &= uint8_t(~(1u << (i % 8)));
    };
    for (size_t r = 0; r < col.rows; ++r) {
        const uint64_t v = col.get(r);
        if (v_isstr(v)) {
            deref(v, plan, s);
            if (s.size() > PAGE - 7) {
                if (nr > 0) save();
                size_t off = 0;
                bool   first = true;
                while (off < s.size()) {
                    uint8_t*     pg  = sink.fresh();
                    const size_t len = std::min(s.size() - off, PAGE - 4);
                    wr16(pg, first ? 0xffff : 0xfffe);
                    wr16(pg + 2, uint16_t(len));
                    std::memcpy(pg + 4, s.data() + off, len);
                    first = false;
                    off += len;
                }
            } else {
                if (4 + (offs.size() + 1) * 2 + (data.size() + s.size()) + (nr / 8 + 1) > PAGE) save();
                bit(nr, true);
                data.insert(data.end(), s.begin(), s.end());
                offs.push_back(uint16_t(data.size()));
                ++nr;
            }
        } else if (v_null(v)) {
            if (4 + offs.size() * 2 + data.size() + (nr / 8 + 1) > PAGE) save();
            bit(nr, false);
            ++nr;
        } else {
            throw std::runtime_error("not string or null");
        }
    }
    if (nr != 0) save();
}

}  // namespace oracle

extern "C" {

// Runs the restated Contest::execute on a flat plan; pages of the result are
// returned per column (see oracle_result.h).
int oracle_execute(const hj_plan_desc* plan, oracle_result* out) {
    using namespace oracle;
    std::memset(out, 0, sizeof(*out));
    g_build_tuples = g_probe_tuples = 0;
    const auto t0 = std::chrono::steady_clock::now();
    try {
        Result res = execute_impl(*plan, plan->root);
        const hj_node_desc& root = plan->nodes[plan->root];
        std::vector<PageSink> sinks(root.num_attrs);
        for (uint32_t c = 0; c < root.num_attrs; ++c) {
            if (root.attrs[c].type == HJ_INT32)        int32_to_pages(res[c], sinks[c]);
            else if (root.attrs[c].type == HJ_VARCHAR) varchar_to_pages(res[c], *plan, sinks[c]);
        }
        g_exec_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        out->num_rows    = res.empty() ? 0 : res[0].rows;
        out->num_columns = root.num_attrs;
        out->types       = new int32_t[root.num_attrs + 1];
        out->num_pages   = new uint64_t[root.num_attrs + 1];
        out->pages       = new uint8_t*[root.num_attrs + 1];
        for (uint32_t c = 0; c < root.num_attrs; ++c) {
            out->types[c]     = root.attrs[c].type;
            out->num_pages[c] = sinks[c].pages.size();
            out->pages[c]     = new uint8_t[sinks[c].pages.size() * PAGE + 1];
            for (size_t p = 0; p < sinks[c].pages.size(); ++p)
                std::memcpy(out->pages[c] + p * PAGE, sinks[c].pages[p].data(), PAGE);
        }
        return HJ_OK;
    } catch (const std::out_of_range& e) {
        out->status = HJ_ERR_OUT_OF_RANGE;
        std::snprintf(out->error, sizeof(out->error), "%s", e.what());
    } catch (const std::runtime_error& e) {
        out->status = HJ_ERR_RUNTIME;
        std::snprintf(out->error, sizeof(out->error), "%s", e.what());
    } catch (const std::exception& e) {
        out->status = HJ_ERR_INVALID;
        std::snprintf(out->error, sizeof(out->error), "%s", e.what());
    }
    return out->status;
}

// Build and probe tuples of the last oracle_execute (all joins) and its
// duration up to the finished result pages.
void oracle_last_stats(uint64_t* build, uint64_t* probe, double* seconds) {
    *build   = oracle::g_build_tuples;
    *probe   = oracle::g_probe_tuples;
    *seconds = oracle::g_exec_seconds;
}

}  // extern "C"
