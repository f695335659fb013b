// Serving: a request loop over join plans (hj_server_*).
//
// Clients submit plans from any thread; each gets a ticket and later waits on
// it.  The server runs `slots` plans at once, each in its own slot -- a host
// thread with a context cloned from the server's (own CUDA stream, pinned
// readback buffers and staging threads) that shares the resident base tables
// and the cache of tables built over them -- so the kernels of concurrent
// plans overlap on the GPU.  Admission is first come, first served against an
// HBM budget: a plan is admitted when a slot is free and its estimated working
// memory (hash tables, probe lists, intermediate row ids, output pages, from
// the row counts of its inputs) fits beside the plans already running; the
// head of the queue waits, so a large plan is never starved by small ones, and
// a plan larger than the whole budget runs alone.  Requests that arrive while
// others run are admitted as slots and memory free up (continuous batching),
// and every request's queueing, service and total latency is recorded.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "hj_common.cuh"
#include "hj_kernels.h"

namespace hj {
namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// A request's own copy of its plan descriptor (the caller's may go away after
// submit).  Host pages of non-resident inputs stay the caller's.
struct PlanCopy {
    std::vector<hj_node_desc>                nodes;
    std::vector<std::vector<hj_attr>>        attrs;
    std::vector<hj_table_desc>               inputs;
    std::vector<std::vector<hj_column_desc>> cols;
    hj_plan_desc                             desc{};

    explicit PlanCopy(const hj_plan_desc& p) {
        if (p.num_nodes && !p.nodes) throw Error(HJ_ERR_INVALID, "plan without nodes");
        if (p.num_inputs && !p.inputs) throw Error(HJ_ERR_INVALID, "plan without inputs");
        nodes.assign(p.nodes, p.nodes + p.num_nodes);
        attrs.resize(nodes.size());
        for (size_t i = 0; i < nodes.size(); ++i) {
            if (nodes[i].num_attrs && !nodes[i].attrs) throw Error(HJ_ERR_INVALID, "node without attributes");
            attrs[i].assign(nodes[i].attrs, nodes[i].attrs + nodes[i].num_attrs);
            nodes[i].attrs = attrs[i].data();
        }
        inputs.assign(p.inputs, p.inputs + p.num_inputs);
        cols.resize(inputs.size());
        for (size_t i = 0; i < inputs.size(); ++i) {
            if (inputs[i].num_columns && inputs[i].columns)
                cols[i].assign(inputs[i].columns, inputs[i].columns + inputs[i].num_columns);
            inputs[i].columns = cols[i].empty() ? nullptr : cols[i].data();
        }
        desc            = p;
        desc.nodes      = nodes.data();
        desc.inputs     = inputs.data();
    }
};

uint64_t next_pow2(uint64_t x) {
    uint64_t p = 1;
    while (p < x) p <<= 1;
    return p;
}

// Working memory of a plan in HBM, from the row counts of its inputs: per
// join its table (adjacency array, directory, partition temporaries), its
// probe lists and the row ids of its result (estimated as the larger input),
// plus the result pages.
uint64_t estimate_bytes(const hj_context* c, const hj_plan_desc& p) {
    std::vector<uint64_t> rows(p.num_nodes, 0);
    std::vector<int>      state(p.num_nodes, 0);
    uint64_t              bytes = 0;
    std::function<uint64_t(uint64_t)> walk = [&](uint64_t i) -> uint64_t {
        if (i >= p.num_nodes) throw Error(HJ_ERR_INVALID, "plan node out of range");
        if (state[i] == 2) return rows[i];
        if (state[i] == 1) throw Error(HJ_ERR_INVALID, "plan has a cycle");
        state[i]             = 1;
        const hj_node_desc& n = p.nodes[i];
        uint64_t            r = 0;
        if (n.kind == HJ_NODE_SCAN) {
            if (n.base_table_id >= p.num_inputs) throw Error(HJ_ERR_INVALID, "scan table out of range");
            const hj_table_desc& t = p.inputs[n.base_table_id];
            r                      = t.resident ? resident_rows(c, t.resident) : t.num_rows;
        } else {
            const uint64_t l = walk(n.left), rr = walk(n.right);
            const uint64_t b = n.build_left ? l : rr, q = n.build_left ? rr : l;
            r                = std::max(b, q);
            bytes += 8 * b + 8 * std::min<uint64_t>(next_pow2(b), 1ull << 22) + 24 * b;  // table + build temporaries
            bytes += 32 * q;                                                           // probe lists, counts
            bytes += 4 * r * std::max<uint32_t>(2, n.num_attrs);                       // result row ids
        }
        rows[i]  = r;
        state[i] = 2;
        return r;
    };
    const uint64_t out = walk(p.root);
    if (p.root < p.num_nodes) bytes += out * 12 * std::max<uint32_t>(1, p.nodes[p.root].num_attrs);  // pages
    return bytes + (1ull << 20);
}

struct Request {
    uint64_t          ticket = 0;
    PlanCopy          plan;
    uint64_t          est    = 0;
    Clock::time_point t_submit, t_start, t_done;
    hj_result*        res    = nullptr;
    int               status = HJ_OK;
    std::string       err;
    bool              done   = false;
    explicit Request(const hj_plan_desc& p) : plan(p) {}
};

}  // namespace
}  // namespace hj

struct hj_server {
    hj_context*                                       parent = nullptr;
    uint64_t                                          budget = 0;
    std::vector<hj_context*>                          slot_ctx;
    std::vector<std::thread>                          workers;
    std::mutex                                        mu;
    std::condition_variable                           cv_work, cv_done;
    std::deque<hj::Request*>                          queue;
    std::map<uint64_t, std::unique_ptr<hj::Request>>  reqs;
    uint64_t                                          next_ticket = 1;
    uint64_t                                          running = 0, running_bytes = 0, peak_bytes = 0;
    bool                                              stop = false;

    bool admissible() const {
        if (queue.empty()) return false;
        return running == 0 || running_bytes + queue.front()->est <= budget;
    }

    void work(size_t slot) {
        hj_context* c = slot_ctx[slot];
        for (;;) {
            hj::Request* r = nullptr;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_work.wait(lk, [&] { return admissible() || (stop && queue.empty()); });
                if (queue.empty()) return;
                r = queue.front();
                queue.pop_front();
                ++running;
                running_bytes += r->est;
                peak_bytes = std::max(peak_bytes, running_bytes);
                r->t_start = hj::Clock::now();
            }
            cv_work.notify_all();  // the next request may fit as well
            hj_result* res = nullptr;
            const int  rc  = hj_execute(c, &r->plan.desc, &res);
            // the caller frees the result later, through the server's context
            if (rc == HJ_OK) hj::result_rebind(res, hj::context_stream(parent));
            std::string err = rc == HJ_OK ? std::string() : std::string(hj_last_error(c));
            {
                std::lock_guard<std::mutex> g(mu);
                r->t_done = hj::Clock::now();
                r->res    = res;
                r->status = rc;
                r->err    = err;
                r->done   = true;
                --running;
                running_bytes -= r->est;
            }
            cv_done.notify_all();
            cv_work.notify_all();
        }
    }
};

extern "C" {

hj_server* hj_server_create(hj_context* ctx, const hj_server_options* opt) {
    if (!ctx || !opt || opt->slots == 0 || opt->slots > 256) return nullptr;
    auto* s   = new hj_server();
    s->parent = ctx;
    s->budget = opt->hbm_budget_bytes;
    try {
        for (uint32_t i = 0; i < opt->slots; ++i) s->slot_ctx.push_back(hj::context_clone(ctx));
        for (uint32_t i = 0; i < opt->slots; ++i) s->workers.emplace_back([s, i] { s->work(i); });
    } catch (const std::exception& e) {
        hj::context_set_error(ctx, e.what());
        {
            std::lock_guard<std::mutex> g(s->mu);
            s->stop = true;
        }
        s->cv_work.notify_all();
        for (auto& t : s->workers) t.join();
        for (auto* c : s->slot_ctx) hj_context_destroy(c);
        delete s;
        return nullptr;
    }
    return s;
}

int hj_server_submit(hj_server* s, const hj_plan_desc* plan, uint64_t* ticket) {
    if (!s || !plan || !ticket) return HJ_ERR_INVALID;
    std::unique_ptr<hj::Request> r;
    try {
        r      = std::make_unique<hj::Request>(*plan);
        r->est = hj::estimate_bytes(s->parent, r->plan.desc);
    } catch (const hj::Error& e) {
        hj::context_set_error(s->parent, e.what());
        return e.status;
    } catch (const std::exception& e) {
        hj::context_set_error(s->parent, e.what());
        return HJ_ERR_INVALID;
    }
    {
        std::lock_guard<std::mutex> g(s->mu);
        if (s->stop) return HJ_ERR_INVALID;
        r->ticket   = s->next_ticket++;
        r->t_submit = hj::Clock::now();
        *ticket     = r->ticket;
        s->queue.push_back(r.get());
        s->reqs[r->ticket] = std::move(r);
    }
    s->cv_work.notify_all();
    return HJ_OK;
}

int hj_server_wait(hj_server* s, uint64_t ticket, hj_result** out, hj_request_stats* stats, char* err,
                   uint32_t err_cap) {
    if (!s || !out) return HJ_ERR_INVALID;
    *out = nullptr;
    std::unique_ptr<hj::Request> r;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->reqs.find(ticket);
        if (it == s->reqs.end()) return HJ_ERR_INVALID;
        hj::Request* rp = it->second.get();
        s->cv_done.wait(lk, [&] { return rp->done; });
        r = std::move(it->second);
        s->reqs.erase(it);
    }
    if (stats) {
        stats->queue_ms   = hj::ms_between(r->t_submit, r->t_start);
        stats->service_ms = hj::ms_between(r->t_start, r->t_done);
        stats->latency_ms = hj::ms_between(r->t_submit, r->t_done);
        stats->est_bytes  = r->est;
    }
    if (err && err_cap) {
        std::strncpy(err, r->err.c_str(), err_cap - 1);
        err[err_cap - 1] = 0;
    }
    *out = r->res;
    return r->status;
}

int hj_server_info(hj_server* s, uint64_t* queued, uint64_t* running, uint64_t* running_bytes,
                   uint64_t* peak_bytes) {
    if (!s) return HJ_ERR_INVALID;
    std::lock_guard<std::mutex> g(s->mu);
    if (queued) *queued = s->queue.size();
    if (running) *running = s->running;
    if (running_bytes) *running_bytes = s->running_bytes;
    if (peak_bytes) *peak_bytes = s->peak_bytes;
    return HJ_OK;
}

void hj_server_destroy(hj_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;  // queued requests still run
    }
    s->cv_work.notify_all();
    for (auto& t : s->workers) t.join();
    for (auto& kv : s->reqs)
        if (kv.second->res) hj_result_free(kv.second->res);
    for (auto* c : s->slot_ctx) hj_context_destroy(c);
    delete s;
}

}  // extern "C"
