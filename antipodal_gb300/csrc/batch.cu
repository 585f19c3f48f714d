// Batched robust evaluation: many RobustMeshGwn meshes, each with its own query array of any size, in one
// persistent launch (no reference counterpart: the reference evaluates one mesh per
// eval_gwnr_mesh_batch_robust call, src/antipodal/gwn_mesh_robust.hh:441-456, and this computes the same values).
//
// Plan (agwn_batch_create): a device table of the meshes and a work list of items -- ranges of one mesh's
// queries sized so that every item carries a similar number of (query, segment) pairs -- ordered longest first,
// so that a persistent grid pulling items from a device queue ends evenly.  Tuner (agwn_batch_tune): times
// every launch configuration {block, queries per thread, segment tile, traversal stack} on a sample of items
// drawn from every mesh and keeps the fastest.  Run (agwn_batch_run): resets the queue head and launches the
// kernel, both captured once into a CUDA graph that later runs replay.

#include "batch.cuh"
#include "robust_handle.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

struct agwn_batch
{
    int device = 0;
    int policy = 0;
    int scalar_bytes = 8;
    int n_meshes = 0;
    int max_depth = 0;
    int64_t max_segments = 0;
    int64_t total_queries = 0;
    double total_pairs = 0;
    agwn::DevBuf meshes, items, sample, head;
    int n_items = 0, n_sample = 0;
    agwn::BConf conf{128, 1, 512, 64};
    bool tuned = false;
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    agwn::BConf graph_conf{0, 0, 0, 0};
    int graph_grid = 0;
    bool graph_mixed = false;
    double graph_term_err = 0;
    bool graph_counting = false;
    std::vector<double> tune_ms; // per candidate, in candidate order
    std::vector<agwn::BConf> candidates;
};

using namespace agwn;

namespace
{
const BatchPolicyOps& ops_of(int policy)
{
    return policy == 0 ? kBatchP64 : (policy == 1 ? kBatchP128 : kBatchPF);
}

bool is_device_ptr(const void* p, int device)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
    {
        cudaGetLastError();
        return false;
    }
    return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) && a.device == device;
}

bool mixed_of(const agwn_batch& b, const Context& ctx)
{
    return ops_of(b.policy).has_mixed && ctx.robust_mode == AGWN_ROBUST_MIXED && b.max_segments < (int64_t(1) << 24);
}

size_t smem_of(const agwn_batch& b, const BConf& c, bool mixed)
{
    // two tiles of segments, or of chain entries in the mixed form
    return 2 * size_t(c.seg_tile) * std::max(ops_of(b.policy).seg_bytes, mixed ? sizeof(RChain) : size_t(0));
}

int grid_of(const agwn_batch& b, const Context& ctx, const BConf& c, int* grid)
{
    int per_sm = 0;
    bool const mixed = mixed_of(b, ctx);
    AGWN_TRY(ops_of(b.policy).occupancy(b.scalar_bytes, c, mixed, smem_of(b, c, mixed), &per_sm));
    if (per_sm < 1)
        return fail(AGWN_ERR_UNSUPPORTED, "batch kernel configuration {%d, %d, %d, %d} does not fit on an SM", c.block,
                    c.k, c.seg_tile, c.stack);
    *grid = per_sm * ctx.sm_count;
    return AGWN_OK;
}

int launch(agwn_batch& b, Context& ctx, cudaStream_t st, const BConf& c, int grid, const BItem* items, int n_items)
{
    bool const mixed = mixed_of(b, ctx);
    AGWN_TRY_CUDA(cudaMemsetAsync(b.head.ptr, 0, sizeof(int), st));
    return ops_of(b.policy).launch(b.scalar_bytes, st, c, mixed, float(ctx.robust_term_err), grid,
                                   smem_of(b, c, mixed), static_cast<const BMesh*>(b.meshes.ptr), items, n_items,
                                   static_cast<int*>(b.head.ptr), ctx.d_flags, ctx.timing ? ctx.d_counters : nullptr);
}

void drop_graph(agwn_batch& b)
{
    if (b.exec)
        cudaGraphExecDestroy(b.exec);
    if (b.graph)
        cudaGraphDestroy(b.graph);
    b.exec = nullptr;
    b.graph = nullptr;
}

void batch_free(agwn_batch* b)
{
    drop_graph(*b);
    if (b->cap)
        cudaStreamDestroy(b->cap);
    b->meshes.release();
    b->items.release();
    b->sample.release();
    b->head.release();
}

// Cost of one query in units of one (query, boundary segment) pair: the segments plus the traversal.
double query_cost(const BMesh& m)
{
    return double(m.n_seg) + 4.0 + 2.0 * std::log2(double(m.n_tri) + 1.0);
}
} // namespace

extern "C" int agwn_batch_create(agwn_context* ctx, const agwn_robust* const* meshes, int32_t n_meshes,
                                 const void* const* positions, const int64_t* n_queries, void* const* out,
                                 int32_t* const* counts, agwn_batch** plan)
{
    AGWN_CHECK_ARG(ctx && plan && n_meshes > 0 && meshes && positions && n_queries && out, "bad arguments");
    clear_message();
    *plan = nullptr;
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    int const policy = meshes[0] ? meshes[0]->policy : -1;
    int const sb = meshes[0] ? meshes[0]->scalar_bytes : 0;
    std::vector<BMesh> hm(n_meshes);
    int max_depth = 0;
    int64_t max_segments = 0;
    int64_t total_q = 0;
    for (int i = 0; i < n_meshes; ++i)
    {
        const agwn_robust* r = meshes[i];
        AGWN_CHECK_ARG(r, "mesh %d is null", i);
        AGWN_CHECK_ARG(r->device == ctx->device, "mesh %d lives on device %d, the context on %d", i, r->device,
                       ctx->device);
        AGWN_CHECK_ARG(r->policy == policy && r->scalar_bytes == sb,
                       "all meshes of a batch must share the scalar type and the precision policy (mesh %d differs)",
                       i);
        AGWN_CHECK_ARG(n_queries[i] >= 0, "mesh %d: negative query count", i);
        if (n_queries[i] > 0)
        {
            AGWN_CHECK_ARG(positions[i] && out[i] && is_device_ptr(positions[i], ctx->device) &&
                               is_device_ptr(out[i], ctx->device) &&
                               (!counts || !counts[i] || is_device_ptr(counts[i], ctx->device)),
                           "mesh %d: positions, out and counts must be device memory of device %d", i, ctx->device);
        }
        BMesh& m = hm[i];
        m.nodes = static_cast<const BvhNode*>(r->hier.nodes.ptr);
        m.tri = r->tri;
        m.leaf_uv = static_cast<const float4*>(r->hier.leaf_uv.ptr);
        m.seg = r->seg;
        m.chain = r->chain;
        m.n_entries = r->n_entries;
        m.pos = positions[i];
        m.out = out[i];
        m.counts = counts ? counts[i] : nullptr;
        m.n_tri = r->n_tri;
        m.n_seg = r->n_seg;
        m.n_q = n_queries[i];
        for (int k = 0; k < 3; ++k)
            m.qc[k] = r->center[k];
        m.qs = r->scale;
        for (int k = 0; k < 9; ++k)
            m.frame[k] = r->hier.frame[k];
        m.scene_scale = float(r->hier.scale);
        if (r->n_tri > 1)
            max_depth = std::max(max_depth, int(r->hier.depth));
        max_segments = std::max(max_segments, r->n_seg);
        total_q += n_queries[i];
    }
    AGWN_CHECK_ARG(max_depth < 64, "hierarchy depth %d exceeds the traversal stack", max_depth);

    // work items: every item carries about the same number of pairs; enough items for ~8 per CTA slot
    double total_cost = 0;
    for (auto const& m : hm)
        total_cost += double(m.n_q) * query_cost(m);
    double const target = std::max(total_cost / (double(ctx->sm_count) * 4.0 * 8.0), double(1 << 18));
    constexpr int64_t kQuantum = 512; // largest block * queries per thread
    std::vector<BItem> items;
    std::vector<double> cost;
    std::vector<BItem> sample;
    for (int i = 0; i < n_meshes; ++i)
    {
        BMesh const& m = hm[i];
        if (m.n_q == 0)
            continue;
        double const c = query_cost(m);
        int64_t nq = int64_t(std::ceil(target / c));
        nq = std::max<int64_t>(kQuantum, (nq + kQuantum - 1) / kQuantum * kQuantum);
        for (int64_t q0 = 0; q0 < m.n_q; q0 += nq)
        {
            items.push_back({i, 0, q0, std::min(m.n_q, q0 + nq)});
            cost.push_back(double(items.back().q1 - q0) * c);
        }
        sample.push_back({i, 0, 0, std::min<int64_t>(m.n_q, 4 * kQuantum)});
    }
    AGWN_CHECK_ARG(items.size() < (size_t(1) << 30), "too many work items");
    std::vector<size_t> order(items.size());
    for (size_t j = 0; j < order.size(); ++j)
        order[j] = j;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
    std::vector<BItem> sorted(items.size());
    for (size_t j = 0; j < order.size(); ++j)
        sorted[j] = items[order[j]];

    auto* b = new agwn_batch;
    b->device = ctx->device;
    b->policy = policy;
    b->scalar_bytes = sb;
    b->n_meshes = n_meshes;
    b->max_depth = max_depth;
    b->max_segments = max_segments;
    b->total_queries = total_q;
    b->total_pairs = total_cost;
    b->n_items = int(sorted.size());
    b->n_sample = int(sample.size());
    int st = AGWN_OK;
    if ((st = b->meshes.reserve(sizeof(BMesh) * hm.size())) != AGWN_OK ||
        (st = b->items.reserve(sizeof(BItem) * std::max<size_t>(1, sorted.size()))) != AGWN_OK ||
        (st = b->sample.reserve(sizeof(BItem) * std::max<size_t>(1, sample.size()))) != AGWN_OK ||
        (st = b->head.reserve(sizeof(int))) != AGWN_OK)
    {
        batch_free(b);
        delete b;
        return st;
    }
    cudaError_t e = cudaMemcpy(b->meshes.ptr, hm.data(), sizeof(BMesh) * hm.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !sorted.empty())
        e = cudaMemcpy(b->items.ptr, sorted.data(), sizeof(BItem) * sorted.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !sample.empty())
        e = cudaMemcpy(b->sample.ptr, sample.data(), sizeof(BItem) * sample.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
    if (e != cudaSuccess)
    {
        batch_free(b);
        delete b;
        return fail(AGWN_ERR_CUDA, "batch plan: %s", cudaGetErrorString(e));
    }
    // candidate configurations; the 32-entry stack only where every hierarchy is shallow enough
    for (int block : {128, 256})
        for (int k : {1, 2})
            for (int tile : {256, 512, 1024})
                for (int stack : {32, 64})
                    if (stack == 64 || max_depth < 32)
                        b->candidates.push_back({block, k, tile, stack});
    b->conf = {128, 1, 512, max_depth < 32 ? 32 : 64};
    *plan = b;
    return AGWN_OK;
}

extern "C" int agwn_batch_destroy(agwn_batch* plan)
{
    if (!plan)
        return AGWN_OK;
    cudaSetDevice(plan->device);
    cudaDeviceSynchronize();
    batch_free(plan);
    delete plan;
    return AGWN_OK;
}

extern "C" int agwn_batch_set_config(agwn_batch* plan, const int32_t* config)
{
    AGWN_CHECK_ARG(plan && config, "null argument");
    clear_message();
    BConf const c{config[0], config[1], config[2], config[3]};
    AGWN_CHECK_ARG(c.block == 128 || c.block == 256, "block must be 128 or 256");
    AGWN_CHECK_ARG(c.k == 1 || c.k == 2, "queries per thread must be 1 or 2");
    AGWN_CHECK_ARG(c.seg_tile >= 32 && c.seg_tile <= 2048, "segment tile must be in [32, 2048]");
    AGWN_CHECK_ARG(c.stack == 32 || c.stack == 64, "stack must be 32 or 64");
    AGWN_CHECK_ARG(c.stack == 64 || plan->max_depth < 32, "a hierarchy of depth %d needs the 64-entry stack",
                   plan->max_depth);
    plan->conf = c;
    return AGWN_OK;
}

// config: block, queries per thread, segment tile, stack; tune_ms (nullable): the sample time of every candidate
// (up to *n_candidates entries); stats: items, total queries.
extern "C" int agwn_batch_info(const agwn_batch* plan, int32_t* config, int32_t* n_candidates, double* tune_ms,
                               int64_t* n_items, int64_t* total_queries, double* total_pairs)
{
    AGWN_CHECK_ARG(plan, "null plan");
    if (config)
    {
        config[0] = plan->conf.block;
        config[1] = plan->conf.k;
        config[2] = plan->conf.seg_tile;
        config[3] = plan->conf.stack;
    }
    if (n_candidates)
    {
        int const cap = *n_candidates;
        *n_candidates = int(plan->candidates.size());
        if (tune_ms)
            for (int i = 0; i < std::min(cap, int(plan->tune_ms.size())); ++i)
                tune_ms[i] = plan->tune_ms[i];
    }
    if (n_items)
        *n_items = plan->n_items;
    if (total_queries)
        *total_queries = plan->total_queries;
    if (total_pairs)
        *total_pairs = plan->total_pairs;
    return AGWN_OK;
}

extern "C" int agwn_batch_tune(agwn_context* ctx, agwn_batch* plan, int32_t repeats)
{
    AGWN_CHECK_ARG(ctx && plan && repeats >= 1, "bad arguments");
    AGWN_CHECK_ARG(ctx->device == plan->device, "plan and context are on different devices");
    clear_message();
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    if (plan->n_sample == 0)
        return AGWN_OK;
    cudaEvent_t e0, e1;
    AGWN_TRY_CUDA(cudaEventCreate(&e0));
    AGWN_TRY_CUDA(cudaEventCreate(&e1));
    plan->tune_ms.assign(plan->candidates.size(), -1.0);
    double best = 1e300;
    BConf best_c = plan->conf;
    int st = AGWN_OK;
    for (size_t i = 0; i < plan->candidates.size() && st == AGWN_OK; ++i)
    {
        BConf const& c = plan->candidates[i];
        int grid = 0;
        if (grid_of(*plan, *ctx, c, &grid) != AGWN_OK)
        {
            clear_message();
            continue; // does not fit: skip
        }
        const BItem* items = static_cast<const BItem*>(plan->sample.ptr);
        st = launch(*plan, *ctx, ctx->stream, c, grid, items, plan->n_sample); // warm-up
        double ms_min = 1e300;
        for (int r = 0; r < repeats && st == AGWN_OK; ++r)
        {
            cudaEventRecord(e0, ctx->stream);
            st = launch(*plan, *ctx, ctx->stream, c, grid, items, plan->n_sample);
            cudaEventRecord(e1, ctx->stream);
            if (cudaEventSynchronize(e1) != cudaSuccess)
                st = fail(AGWN_ERR_CUDA, "tuning launch failed: %s", cudaGetErrorString(cudaGetLastError()));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            ms_min = std::min(ms_min, double(ms));
        }
        ctx->launches[AGWN_K_ROBUST] += repeats + 1;
        plan->tune_ms[i] = ms_min;
        if (ms_min < best)
        {
            best = ms_min;
            best_c = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    AGWN_TRY(st);
    AGWN_TRY(ctx->check_flags());
    plan->conf = best_c;
    plan->tuned = true;
    return AGWN_OK;
}

extern "C" int agwn_batch_run(agwn_context* ctx, agwn_batch* plan, int32_t use_graph)
{
    AGWN_CHECK_ARG(ctx && plan, "null argument");
    AGWN_CHECK_ARG(ctx->device == plan->device, "plan and context are on different devices");
    clear_message();
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    if (plan->n_items == 0)
        return AGWN_OK;
    BConf const c = plan->conf;
    int grid = 0;
    AGWN_TRY(grid_of(*plan, *ctx, c, &grid));
    const BItem* items = static_cast<const BItem*>(plan->items.ptr);
    if (!use_graph)
    {
        AGWN_TRY(ctx->launch_begin(AGWN_K_ROBUST));
        AGWN_TRY(launch(*plan, *ctx, ctx->stream, c, grid, items, plan->n_items));
        return ctx->launch_end(AGWN_K_ROBUST);
    }
    bool const mixed = mixed_of(*plan, *ctx);
    bool const same = plan->exec && plan->graph_conf.block == c.block && plan->graph_conf.k == c.k &&
                      plan->graph_conf.seg_tile == c.seg_tile && plan->graph_conf.stack == c.stack &&
                      plan->graph_grid == grid && plan->graph_mixed == mixed &&
                      plan->graph_term_err == ctx->robust_term_err && plan->graph_counting == ctx->timing;
    if (!same)
    {
        drop_graph(*plan);
        AGWN_TRY_CUDA(cudaStreamBeginCapture(plan->cap, cudaStreamCaptureModeThreadLocal));
        int const s = launch(*plan, *ctx, plan->cap, c, grid, items, plan->n_items);
        cudaGraph_t g = nullptr;
        cudaError_t const e = cudaStreamEndCapture(plan->cap, &g);
        AGWN_TRY(s);
        AGWN_TRY_CUDA(e);
        plan->graph = g;
        AGWN_TRY_CUDA(cudaGraphInstantiate(&plan->exec, plan->graph, 0));
        plan->graph_conf = c;
        plan->graph_grid = grid;
        plan->graph_mixed = mixed;
        plan->graph_term_err = ctx->robust_term_err;
        plan->graph_counting = ctx->timing;
    }
    AGWN_TRY(ctx->launch_begin(AGWN_K_ROBUST));
    AGWN_TRY_CUDA(cudaGraphLaunch(plan->exec, ctx->stream));
    return ctx->launch_end(AGWN_K_ROBUST);
}
