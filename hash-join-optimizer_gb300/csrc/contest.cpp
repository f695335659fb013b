// The contest entry points (include/plan.h: Contest::build_context,
// destroy_context, execute) over the engine's C ABI.  Same signatures and
// exception classes as the reference (src/execute.cpp:598-614): a harness that
// links the reference's execute.cpp can link this instead.
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/hj_api.h"
#include "../../include/plan.h"

namespace {

[[noreturn]] void raise(int rc, const char* msg) {
    const std::string m = msg ? msg : "hash-join engine error";
    if (rc == HJ_ERR_OUT_OF_RANGE) throw std::out_of_range(m);
    throw std::runtime_error(m);
}

// execute(plan, nullptr) runs on a per-thread default context, created once.
hj_context* default_context() {
    thread_local std::unique_ptr<hj_context, void (*)(hj_context*)> ctx(nullptr, hj_context_destroy);
    if (!ctx) {
        ctx.reset(hj_context_create(-1));
        if (!ctx) raise(HJ_ERR_NO_DEVICE, hj_last_error(nullptr));
    }
    return ctx.get();
}

}  // namespace

namespace Contest {

void* build_context() {
    hj_context* c = hj_context_create(-1);
    if (!c) raise(HJ_ERR_NO_DEVICE, hj_last_error(nullptr));
    return c;
}

void destroy_context(void* context) { hj_context_destroy(static_cast<hj_context*>(context)); }

ColumnarTable execute(const Plan& plan, void* context) {
    hj_context* c = context ? static_cast<hj_context*>(context) : default_context();

    // Flatten the plan; pages are borrowed, not copied.
    std::vector<std::vector<hj_attr>>        attrs(plan.nodes.size());
    std::vector<hj_node_desc>                nodes(plan.nodes.size());
    std::vector<std::vector<hj_column_desc>> cols(plan.inputs.size());
    std::vector<hj_table_desc>               tables(plan.inputs.size());
    for (size_t i = 0; i < plan.nodes.size(); ++i) {
        const PlanNode& pn = plan.nodes[i];
        for (const auto& [idx, ty] : pn.output_attrs) attrs[i].push_back(hj_attr{idx, int32_t(ty)});
        hj_node_desc& d = nodes[i];
        d               = hj_node_desc{};
        d.num_attrs     = uint32_t(attrs[i].size());
        d.attrs         = attrs[i].data();
        if (const auto* s = std::get_if<ScanNode>(&pn.data)) {
            d.kind          = HJ_NODE_SCAN;
            d.base_table_id = s->base_table_id;
        } else {
            const auto& j = std::get<JoinNode>(pn.data);
            d.kind        = HJ_NODE_JOIN;
            d.build_left  = j.build_left ? 1 : 0;
            d.left        = j.left;
            d.right       = j.right;
            d.left_attr   = j.left_attr;
            d.right_attr  = j.right_attr;
        }
    }
    for (size_t t = 0; t < plan.inputs.size(); ++t) {
        const ColumnarTable& ct = plan.inputs[t];
        for (const Column& col : ct.columns)
            cols[t].push_back(hj_column_desc{int32_t(col.type), col.pages.size(),
                                             reinterpret_cast<const void* const*>(col.pages.data())});
        tables[t] = hj_table_desc{ct.num_rows, uint32_t(cols[t].size()), cols[t].data(), 0};
    }
    hj_plan_desc desc{uint32_t(nodes.size()), nodes.data(), uint32_t(tables.size()), tables.data(),
                      plan.root};

    hj_result* res = nullptr;
    if (int rc = hj_execute(c, &desc, &res); rc != HJ_OK) raise(rc, hj_last_error(c));
    std::unique_ptr<hj_result, void (*)(hj_result*)> guard(res, hj_result_free);

    ColumnarTable out;
    uint64_t      nrows = 0;
    uint32_t      ncols = 0;
    hj_result_shape(res, &nrows, &ncols);
    out.num_rows = nrows;
    for (uint32_t i = 0; i < ncols; ++i) {
        int32_t  ty = 0;
        uint64_t np = 0;
        hj_result_column(res, i, &ty, &np);
        out.columns.emplace_back(static_cast<DataType>(ty));
        Column& col = out.columns.back();
        col.pages.reserve(np);
        for (uint64_t p = 0; p < np; ++p) col.new_page();
        if (np) {
            if (int rc = hj_result_copy_pages(c, res, i, reinterpret_cast<void* const*>(col.pages.data()));
                rc != HJ_OK)
                raise(rc, hj_last_error(c));
        }
    }
    return out;
}

}  // namespace Contest
