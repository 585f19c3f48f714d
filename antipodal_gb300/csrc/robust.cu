// Robust mesh GWN on the device: RobustMeshGwn<T, Precision> and eval_gwnr_mesh_batch_robust
// (src/antipodal/gwn_mesh_robust.hh:170-456) with its exact predicates (src/antipodal/math/robust_predicates.hh).
//
// Both terms are decided by one exact predicate along the fixed -x ray, so they agree at every grazing
// configuration.  The predicate's coordinates are, by policy:
//   int64_grid   int32 on a 20-bit grid, 64-bit determinants;
//   int128_grid  int64 on a 50-bit grid, 128-bit determinants from 64x64 mul.lo / mul.hi;
//   exact_float  the doubles themselves, sign of the determinant by a forward-error filter and, when that cannot
//                decide, an exact fma / TwoSum expansion of its six products.
// Every double operation the integer count depends on (quantisation, the filter, the barycentric hit depth) is
// written unfused with rd, so counts equal the reference's bit for bit; the fractional term differs from it only
// by the last bits of atan2.
//
// Integer term: the triangles on the predicate's coordinates go into the ray-frame hierarchy of hier.cuh built
// for the direction -x (so (u, v) = (z, y) and w = -x); a leaf is tested with the reference's occluded rule
// (gwn_mesh_robust.hh:122-145): project_into_tri, then count -sign when q.x >= hit_x.  The hierarchy only culls,
// conservatively, replacing Embree's traversal.  Fractional term: the quantised, endpoint-swapped boundary
// (:198-206) is staged through shared memory like the mesh kernels; per segment the reference's branches
// (:264-325).

#include "robust.cuh"

#include <algorithm>

namespace agwn
{
namespace
{
struct RTmp
{
    void* p = nullptr;
    ~RTmp()
    {
        if (p)
            cudaFree(p);
    }
    int alloc(size_t bytes)
    {
        cudaError_t const e = cudaMalloc(&p, bytes ? bytes : 1);
        if (e != cudaSuccess)
        {
            cudaGetLastError();
            p = nullptr;
            return fail(e == cudaErrorMemoryAllocation ? AGWN_ERR_NOMEM : AGWN_ERR_CUDA, "cudaMalloc(%zu): %s", bytes,
                        cudaGetErrorString(e));
        }
        return AGWN_OK;
    }
};

void robust_free(Robust* r)
{
    if (!r)
        return;
    if (r->tri)
        cudaFree(r->tri);
    if (r->seg)
        cudaFree(r->seg);
    if (r->chain)
        cudaFree(r->chain);
    r->tri = r->seg = r->chain = nullptr;
    r->cells.release();
    r->hier.release();
}

template <class T, class P>
int robust_build(Context& ctx, const T* vertices, int64_t nv, const int32_t* indices, int64_t n_idx,
                 const T* boundary, int64_t n_seg, Robust* out)
{
    using C = typename P::C;
    AGWN_CHECK_ARG(nv >= 0 && n_idx >= 0 && n_idx % 3 == 0 && n_seg >= 0, "bad sizes");
    AGWN_CHECK_ARG(n_idx / 3 < (int64_t(1) << 31) - 1, "too many triangles");
    AGWN_CHECK_ARG((n_idx == 0 || (vertices && indices)) && (n_seg == 0 || boundary), "null geometry");
    int64_t const n_tri = n_idx / 3;
    out->n_tri = n_tri;
    out->n_seg = n_seg;
    out->device = ctx.device;
    out->scalar_bytes = int(sizeof(T));
    cudaStream_t const st = ctx.stream;
    const void *dv = nullptr, *di = nullptr, *db = nullptr;
    AGWN_TRY(stage_in(ctx, vertices, sizeof(T) * 3 * nv, S_MISC0, &dv));
    AGWN_TRY(stage_in(ctx, indices, sizeof(int32_t) * n_idx, S_MISC1, &di));
    AGWN_TRY(stage_in(ctx, boundary, sizeof(T) * 7 * n_seg, S_MISC2, &db));
    // quantisation frame, as RobustMeshGwn::build_quantization (gwn_mesh_robust.hh:354-378)
    Quant qz{{0, 0, 0}, 1.0};
    if (P::grid && nv > 0)
    {
        RTmp bb;
        AGWN_TRY(bb.alloc(sizeof(unsigned long long) * 6));
        unsigned long long init[6] = {~0ull, ~0ull, ~0ull, 0, 0, 0};
        AGWN_TRY_CUDA(cudaMemcpyAsync(bb.p, init, sizeof(init), cudaMemcpyHostToDevice, st));
        AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
        k_bbox<T><<<std::min(div_up(nv, 256), 4 * ctx.sm_count), 256, 0, st>>>(static_cast<const T*>(dv), nv,
                                                                              static_cast<unsigned long long*>(bb.p));
        AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
        unsigned long long back[6];
        AGWN_TRY_CUDA(cudaMemcpyAsync(back, bb.p, sizeof(back), cudaMemcpyDeviceToHost, st));
        AGWN_TRY_CUDA(cudaStreamSynchronize(st));
        double mn[3], mx[3], ext[3];
        for (int k = 0; k < 3; ++k)
        {
            mn[k] = dbl_unorder(back[k]);
            mx[k] = dbl_unorder(back[3 + k]);
            ext[k] = mx[k] - mn[k];
            qz.c[k] = mn[k] + ext[k] * 0.5;
        }
        double const half = 0.5 * std::max({ext[0], ext[1], ext[2]});
        constexpr double max_coord = double((1ll << P::bits) - 1);
        qz.s = half > 0.0 ? max_coord / half : 1.0;
    }
    for (int k = 0; k < 3; ++k)
        out->center[k] = qz.c[k];
    out->scale = qz.s;
    int const g = std::min(div_up(std::max<int64_t>(n_tri, n_seg), 256), 8 * ctx.sm_count);
    if (n_tri > 0)
    {
        RTmp tq, td, order;
        AGWN_TRY(tq.alloc(sizeof(C) * 9 * n_tri));
        AGWN_TRY(td.alloc(sizeof(double) * 9 * n_tri));
        AGWN_TRY(order.alloc(sizeof(unsigned) * n_tri));
        AGWN_TRY_CUDA(cudaMemsetAsync(ctx.d_flags + FLAG_COUNT - 1, 0, sizeof(int), st));
        AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
        k_robust_tris<T, P><<<g, 256, 0, st>>>(static_cast<const T*>(dv), nv, static_cast<const int32_t*>(di), n_tri,
                                              qz, static_cast<C*>(tq.p), static_cast<double*>(td.p), ctx.d_flags);
        AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
        int bad = 0;
        AGWN_TRY_CUDA(cudaMemcpyAsync(&bad, ctx.d_flags + FLAG_COUNT - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        AGWN_TRY_CUDA(cudaStreamSynchronize(st));
        if (bad)
        {
            AGWN_TRY_CUDA(cudaMemsetAsync(ctx.d_flags + FLAG_COUNT - 1, 0, sizeof(int), st));
            return fail(AGWN_ERR_INVALID, "triangle index out of range [0, %lld)", (long long)nv);
        }
        double const dir[3] = {-1.0, 0.0, 0.0};
        AGWN_TRY(build_hier<double>(ctx, static_cast<const double*>(td.p), n_tri, dir, out->hier,
                                    static_cast<unsigned*>(order.p)));
        out->hier.tri.release(); // the leaves are read from the predicate triangles below
        AGWN_TRY_CUDA(cudaMalloc(&out->tri, sizeof(C) * 9 * n_tri));
        AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
        k_gather_leaves<C><<<g, 256, 0, st>>>(static_cast<const C*>(tq.p), static_cast<const unsigned*>(order.p), n_tri,
                                             static_cast<C*>(out->tri));
        AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
        AGWN_TRY_CUDA(cudaStreamSynchronize(st));
    }
    AGWN_TRY_CUDA(cudaMalloc(&out->seg, sizeof(RSeg<C>) * std::max<int64_t>(1, n_seg)));
    if (n_seg > 0)
    {
        AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
        k_robust_segs<T, P><<<g, 256, 0, st>>>(static_cast<const T*>(db), n_seg, qz,
                                              static_cast<RSeg<C>*>(out->seg));
        AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
    }
    if constexpr (std::is_same_v<P, P64>)
        if (n_seg > 0 && n_seg < (int64_t(1) << 24))
        {
            // the chains of the mixed form's FP32 pairs
            AGWN_TRY_CUDA(cudaMalloc(&out->chain, sizeof(RChain) * 2 * size_t(n_seg)));
            RTmp order, cnt;
            AGWN_TRY(order.alloc(sizeof(int) * std::max<int64_t>(1, chain_scratch_ints(n_seg))));
            AGWN_TRY(cnt.alloc(sizeof(long long)));
            AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
            k_robust_chain<<<1, 1024, 0, st>>>(static_cast<const RSeg<int32_t>*>(out->seg), n_seg,
                                               static_cast<RChain*>(out->chain), static_cast<long long*>(cnt.p),
                                               static_cast<int*>(order.p));
            AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
            long long m = 0;
            AGWN_TRY_CUDA(cudaMemcpyAsync(&m, cnt.p, sizeof(m), cudaMemcpyDeviceToHost, st));
            AGWN_TRY_CUDA(cudaStreamSynchronize(st));
            out->n_entries = m;
        }
    AGWN_TRY_CUDA(cudaStreamSynchronize(st));
    return AGWN_OK;
}

// The evaluator's swapped exact_float segments back in input orientation, 7 doubles each (pos0, pos1, w).
__global__ void k_rseg_raw(const RSeg<double>* __restrict__ seg, int64_t n_seg, double* __restrict__ raw)
{
    for (int64_t s = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; s < n_seg; s += int64_t(gridDim.x) * blockDim.x)
    {
        RSeg<double> const g = seg[s];
        double* const o = raw + 7 * s;
        for (int k = 0; k < 3; ++k)
        {
            o[k] = g.p1[k];
            o[3 + k] = g.p0[k];
        }
        o[6] = g.w;
    }
}

__global__ void k_frac_plus_counts(const double* __restrict__ frac, const int32_t* __restrict__ counts,
                                   double* __restrict__ out, int64_t n)
{
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        out[i] = frac[i] + double(counts[i]);
}

// The exact_float counts of one chunk of queries through the cell grid (frac_mixed_robust_pf_chunked's callback).
struct RobustCountJob
{
    const Robust* r;
    Quant qz;
    Frame32 f;
};

int robust_count_chunk(void* user, Context& ctx, const double* d_pos, int64_t m, int32_t* d_counts)
{
    RobustCountJob const& j = *static_cast<const RobustCountJob*>(user);
    Robust const& r = *j.r;
    int const grid = int(std::min<int64_t>(div_up(m, kRobBlock), int64_t(ctx.sm_count) * 16));
    AGWN_TRY(ctx.launch_begin(AGWN_K_ROBUST));
    k_robust_cells<double, PF><<<grid, kRobBlock, 0, ctx.stream>>>(
        static_cast<const BvhNode*>(r.hier.nodes.ptr), static_cast<const typename PF::C*>(r.tri),
        static_cast<const float4*>(r.hier.leaf_uv.ptr), float(r.hier.scale), j.f, cell_view(r.cells), j.qz, d_pos, m,
        d_counts, ctx.d_flags, ctx.timing ? ctx.d_counters : nullptr);
    return ctx.launch_end(AGWN_K_ROBUST);
}

template <class T, class P>
int robust_run(Context& ctx, const Robust& r, const T* d_pos, int64_t n, T* d_out, int32_t* d_counts, T* d_frac,
               bool counts_ready = false)
{
    using C = typename P::C;
    Quant qz{{r.center[0], r.center[1], r.center[2]}, r.scale};
    cudaStream_t const st = ctx.stream;
    if constexpr (std::is_same_v<P, PF> && std::is_same_v<T, double>)
    {
        // mixed exact_float over many queries: counts and fractional term in chunks on two streams, so that one
        // chunk's counts (FP64 predicates) overlap another chunk's fractional term (FP32 pairs)
        if (!counts_ready && !d_frac && n >= (int64_t(1) << 21) && r.n_tri > 1 && ctx.integer_cells &&
            ctx.robust_mode == AGWN_ROBUST_MIXED && r.n_seg > 0 && r.n_seg < (int64_t(1) << 24) &&
            ctx.use_mixed(double(n) * double(r.n_seg), r.n_seg))
        {
            if (!r.cells.valid)
                AGWN_TRY(build_cells(ctx, r.hier, float(r.hier.scale), r.cells));
            if (r.cells.valid)
            {
                double* raw = nullptr;
                AGWN_TRY(ctx.scratch_reserve(S_MISC2, sizeof(double) * 7 * size_t(r.n_seg),
                                             reinterpret_cast<void**>(&raw)));
                AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
                k_rseg_raw<<<int(std::min<int64_t>(div_up(r.n_seg, 256), 4 * ctx.sm_count)), 256, 0, st>>>(
                    static_cast<const RSeg<double>*>(r.seg), r.n_seg, raw);
                AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
                RobustCountJob job{&r, qz, {}};
                for (int k = 0; k < 9; ++k)
                    job.f.r[k] = r.hier.frame[k];
                return frac_mixed_robust_pf_chunked(ctx, d_pos, n, d_out, d_counts, raw, r.n_seg, r.seg,
                                                    &robust_count_chunk, &job);
            }
        }
    }
    if (counts_ready)
        ;
    else if (r.n_tri == 0)
        AGWN_TRY_CUDA(cudaMemsetAsync(d_counts, 0, sizeof(int32_t) * n, st));
    else
    {
        Frame32 f;
        for (int k = 0; k < 9; ++k)
            f.r[k] = r.hier.frame[k];
        int const grid = int(std::min<int64_t>(div_up(n, kRobBlock), int64_t(ctx.sm_count) * 16));
        if (ctx.integer_cells && r.n_tri > 1 && !r.cells.valid)
            AGWN_TRY(build_cells(ctx, r.hier, float(r.hier.scale), r.cells));
        if (ctx.integer_cells && r.n_tri > 1 && r.cells.valid)
        {
            AGWN_TRY(ctx.launch_begin(AGWN_K_ROBUST));
            k_robust_cells<T, P><<<grid, kRobBlock, 0, st>>>(
                static_cast<const BvhNode*>(r.hier.nodes.ptr), static_cast<const C*>(r.tri),
                static_cast<const float4*>(r.hier.leaf_uv.ptr), float(r.hier.scale), f, cell_view(r.cells), qz, d_pos,
                n, d_counts, ctx.d_flags, ctx.timing ? ctx.d_counters : nullptr);
            AGWN_TRY(ctx.launch_end(AGWN_K_ROBUST));
        }
        else
        {
        AGWN_TRY(ctx.launch_begin(AGWN_K_ROBUST));
        k_robust_count<T, P><<<grid, kRobBlock, 0, st>>>(
            static_cast<const BvhNode*>(r.hier.nodes.ptr), static_cast<const C*>(r.tri),
            static_cast<const float4*>(r.hier.leaf_uv.ptr), r.n_tri, float(r.hier.scale), f, qz, d_pos, n, d_counts,
            ctx.d_flags);
        AGWN_TRY(ctx.launch_end(AGWN_K_ROBUST));
        }
    }
    using Seg = RSeg<C>;
    if constexpr (std::is_same_v<P, PF> && std::is_same_v<T, double>)
    {
        // mixed exact_float: the mesh functions' mixed kernel with the robust FP64 rule (frac.cu)
        // (on short boundaries and small calls the exact kernel is the faster one: Context::use_mixed)
        if (ctx.robust_mode == AGWN_ROBUST_MIXED && r.n_seg > 0 && r.n_seg < (int64_t(1) << 24) &&
            ctx.use_mixed(double(n) * double(r.n_seg), r.n_seg))
        {
            double* raw = nullptr;
            AGWN_TRY(ctx.scratch_reserve(S_MISC2, sizeof(double) * 7 * size_t(r.n_seg), reinterpret_cast<void**>(&raw)));
            AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
            k_rseg_raw<<<int(std::min<int64_t>(div_up(r.n_seg, 256), 4 * ctx.sm_count)), 256, 0, st>>>(
                static_cast<const RSeg<double>*>(r.seg), r.n_seg, raw);
            AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
            if (!d_frac)
                return frac_mixed_robust_pf(ctx, d_pos, n, d_out, d_counts, raw, r.n_seg, r.seg);
            AGWN_TRY(frac_mixed_robust_pf(ctx, d_pos, n, d_frac, nullptr, raw, r.n_seg, r.seg));
            AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
            k_frac_plus_counts<<<int(std::min<int64_t>(div_up(n, 256), 8 * ctx.sm_count)), 256, 0, st>>>(
                d_frac, d_counts, d_out, n);
            return ctx.launch_end(AGWN_K_OTHER);
        }
    }
    // the mixed form (int64_grid only) walks the vertex chains built with the evaluator
    bool const mixed = std::is_same_v<P, P64> && ctx.robust_mode == AGWN_ROBUST_MIXED && r.chain != nullptr;
    int64_t const n_elem = mixed ? r.n_entries : r.n_seg;
    int const tile = int(std::max<int64_t>(1, std::min<int64_t>(ctx.seg_tile, n_elem)));
    int const n_tiles = int((n_elem + tile - 1) / tile);
    size_t const smem = size_t(n_tiles <= 1 ? 1 : 2) * tile * (mixed ? sizeof(RChain) : sizeof(Seg));
    auto kern = k_robust_frac<T, P, false>;
    if constexpr (std::is_same_v<P, P64>)
        if (mixed)
            kern = k_robust_frac<T, P, true>;
    AGWN_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int per_sm = 0;
    AGWN_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kRobBlock, smem));
    if (per_sm < 1)
        return fail(AGWN_ERR_UNSUPPORTED, "robust kernel does not fit on an SM");
    int64_t const n_qtiles = (n + kRobBlock - 1) / kRobBlock;
    int const grid = int(std::max<int64_t>(1, std::min<int64_t>(n_qtiles, int64_t(per_sm) * ctx.sm_count)));
    AGWN_TRY(ctx.launch_begin(AGWN_K_ROBUST));
    kern<<<grid, kRobBlock, smem, st>>>(d_pos, n, qz, static_cast<const Seg*>(r.seg), r.n_seg,
                                        static_cast<const RChain*>(r.chain), r.n_entries, tile, d_counts, d_out,
                                        d_frac, ctx.d_flags, float(ctx.robust_term_err),
                                        ctx.timing ? ctx.d_counters : nullptr);
    return ctx.launch_end(AGWN_K_ROBUST);
}

template <class T>
int robust_create(agwn_context* ctx, int policy, const T* vertices, int64_t nv, const int32_t* indices, int64_t n_idx,
                  const T* boundary, int64_t n_seg, agwn_robust** out)
{
    AGWN_CHECK_ARG(ctx && out, "null context/out");
    AGWN_CHECK_ARG(policy >= 0 && policy <= 2, "policy must be 0 (int64_grid), 1 (int128_grid) or 2 (exact_float)");
    *out = nullptr;
    clear_message();
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    auto* r = new agwn_robust{};
    r->policy = policy;
    int s = AGWN_OK;
    switch (policy)
    {
    case 0:
        s = robust_build<T, P64>(*ctx, vertices, nv, indices, n_idx, boundary, n_seg, r);
        break;
    case 1:
        s = robust_build<T, P128>(*ctx, vertices, nv, indices, n_idx, boundary, n_seg, r);
        break;
    default:
        s = robust_build<T, PF>(*ctx, vertices, nv, indices, n_idx, boundary, n_seg, r);
        break;
    }
    if (s != AGWN_OK)
    {
        robust_free(r);
        delete r;
        return s;
    }
    *out = r;
    return AGWN_OK;
}

template <class T>
int robust_eval(agwn_context* ctx, const agwn_robust* r, const T* positions, int64_t n, T* out, int32_t* out_counts,
                T* out_frac)
{
    AGWN_CHECK_ARG(ctx && r, "null context/evaluator");
    AGWN_CHECK_ARG(n >= 0 && (n == 0 || (positions && out)), "bad positions/out");
    AGWN_CHECK_ARG(r->scalar_bytes == int(sizeof(T)), "evaluator precision does not match the queries");
    clear_message();
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    if (n == 0)
        return AGWN_OK;
    const void* dpos = nullptr;
    void *dout = nullptr, *dcnt = nullptr, *dfr = nullptr;
    bool h_out = false, h_cnt = false, h_fr = false;
    AGWN_TRY(stage_in(*ctx, positions, sizeof(T) * 3 * n, S_QUERIES, &dpos));
    AGWN_TRY(stage_out(*ctx, out, sizeof(T) * n, S_OUT, &dout, &h_out));
    if (out_counts)
        AGWN_TRY(stage_out(*ctx, out_counts, sizeof(int32_t) * n, S_COUNTS, &dcnt, &h_cnt));
    else
        AGWN_TRY(ctx->scratch_reserve(S_COUNTS, sizeof(int32_t) * n, &dcnt));
    if (out_frac)
        AGWN_TRY(stage_out(*ctx, out_frac, sizeof(T) * n, S_MISC3, &dfr, &h_fr));
    const T* p = static_cast<const T*>(dpos);
    T* o = static_cast<T*>(dout);
    int32_t* c = static_cast<int32_t*>(dcnt);
    T* fr = static_cast<T*>(dfr);
    bool ordered = false;
    if constexpr (std::is_same_v<T, double>)
    {
        // exact_float in mixed mode: an incoherent query order runs on a spatially sorted copy (order.cu), where the
        // mixed kernel certifies far more boundary groups; the values are the same bit for bit
        if (r->policy == 2 && ctx->robust_mode == AGWN_ROBUST_MIXED && !ctx->ordering && r->n_seg > 0 &&
            r->n_seg < (int64_t(1) << 24) && ctx->use_mixed(double(n) * double(r->n_seg), r->n_seg))
        {
            double const dir[3] = {-1.0, 0.0, 0.0}; // the evaluator's rays and fractional frame run along -x
            const int32_t* perm = nullptr;
            AGWN_TRY(query_order(*ctx, p, n, dir, dpos == positions, &perm));
            if (perm)
            {
                size_t const m = size_t(n);
                double* ps = nullptr;
                AGWN_TRY(ctx->scratch_reserve(S_ORDER1, m * (sizeof(double) * (fr ? 5 : 4) + sizeof(int32_t)),
                                              reinterpret_cast<void**>(&ps)));
                double* const os = ps + 3 * m;
                double* const fs = fr ? os + m : nullptr;
                int32_t* const cs = reinterpret_cast<int32_t*>(os + (fr ? 2 : 1) * m);
                AGWN_TRY(gather_queries(*ctx, p, perm, n, ps));
                ctx->ordering = true;
                int const rc = robust_run<T, PF>(*ctx, *r, ps, n, os, cs, fs);
                ctx->ordering = false;
                AGWN_TRY(rc);
                AGWN_TRY(scatter_back<double>(*ctx, os, perm, n, o));
                if (out_counts)
                    AGWN_TRY(scatter_back<int32_t>(*ctx, cs, perm, n, c));
                if (fs)
                    AGWN_TRY(scatter_back<double>(*ctx, fs, perm, n, fr));
                ordered = true;
            }
        }
    }
    if (!ordered)
    {
        switch (r->policy)
        {
        case 0:
            AGWN_TRY((robust_run<T, P64>(*ctx, *r, p, n, o, c, fr)));
            break;
        case 1:
            AGWN_TRY((robust_run<T, P128>(*ctx, *r, p, n, o, c, fr)));
            break;
        default:
            AGWN_TRY((robust_run<T, PF>(*ctx, *r, p, n, o, c, fr)));
            break;
        }
    }
    if (h_out)
        AGWN_TRY_CUDA(cudaMemcpyAsync(out, dout, sizeof(T) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (h_cnt)
        AGWN_TRY_CUDA(cudaMemcpyAsync(out_counts, dcnt, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (h_fr)
        AGWN_TRY_CUDA(cudaMemcpyAsync(out_frac, dfr, sizeof(T) * n, cudaMemcpyDeviceToHost, ctx->stream));
    bool const sync = dpos != positions || h_out || h_cnt || h_fr;
    return sync ? ctx->check_flags() : AGWN_OK;
}
// ---- RobustMeshGwn::eval over an axis-aligned grid ------------------------------------------------------------
// Cell (ix, iy, iz) is the point (T(s_x + ix h_x), T(s_y + iy h_y), T(s_z + iz h_z)), each coordinate computed in
// double, unfused, then rounded to T; h > 0.  The integer term needs no traversal: the -x crossing rule
// (robust_crossing) decides inclusion and the hit depth hx from the point's (y, z) alone, so for a column of cells
// (fixed iy, iz) a triangle either crosses none of them or crosses exactly those whose predicate x is >= hx, which
// -- x being monotone in ix -- are ix >= ix0.  The rasterizer adds the crossing's sign at (ix0, iy, iz) for every
// (triangle, column) and a prefix sum along x turns that into every cell's count, equal to robust_crossing summed
// over the triangles at that cell.  Columns a triangle can cover come from binary searches of its predicate-space
// box over the monotone grid coordinates.  The fractional term is the evaluator's own, on the materialised cells.
// The reference's OpenGL evaluator (gwn_mesh_opengl.hh:198-351) rasterizes the same way in float with ceil
// snapping; these counts are exact.

template <class T>
__device__ __forceinline__ T grid_coord(double s, double h, int64_t i)
{
    return T(__dadd_rn(s, __dmul_rn(double(i), h)));
}

// The predicate coordinate of grid index i along axis k (quantize, per axis).
template <class T, class P>
__device__ __forceinline__ typename P::C grid_pred(double s, double h, int64_t i, int k, Quant const& qz)
{
    double const v = double(grid_coord<T>(s, h, i));
    if constexpr (P::grid)
    {
        constexpr double max_q = double(1ll << (P::bits + 10));
        double const t = __dmul_rn(__dsub_rn(v, qz.c[k]), qz.s);
        double const cl = t < -max_q ? -max_q : (max_q < t ? max_q : t);
        return typename P::C(llround(cl));
    }
    else
        return v;
}

// First index in [0, n) whose predicate coordinate, seen as a double as robust_crossing compares it, is >= v
// (strict: > v), or n.  The coordinate is monotone in the index and so is its double, so the search is exact.
template <class T, class P>
__device__ __forceinline__ int64_t grid_first(double s, double h, int64_t n, int k, Quant const& qz, double v,
                                              bool strict)
{
    int64_t lo = 0, hi = n;
    while (lo < hi)
    {
        int64_t const mid = (lo + hi) >> 1;
        double const c = P::cdbl(grid_pred<T, P>(s, h, mid, k, qz));
        if (strict ? c > v : c >= v)
            hi = mid;
        else
            lo = mid + 1;
    }
    return lo;
}

struct GridSpec
{
    double s[3], h[3];
    int64_t n[3];
};

template <class T>
__global__ void k_grid_positions(GridSpec g, T* __restrict__ pos)
{
    int64_t const total = g.n[0] * g.n[1] * g.n[2];
    for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < total; c += int64_t(gridDim.x) * blockDim.x)
    {
        int64_t const ix = c % g.n[0], iy = (c / g.n[0]) % g.n[1], iz = c / (g.n[0] * g.n[1]);
        pos[3 * c] = grid_coord<T>(g.s[0], g.h[0], ix);
        pos[3 * c + 1] = grid_coord<T>(g.s[1], g.h[1], iy);
        pos[3 * c + 2] = grid_coord<T>(g.s[2], g.h[2], iz);
    }
}

template <class T, class P>
__global__ void k_grid_raster(const typename P::C* __restrict__ tri, int64_t n_tri, Quant qz, GridSpec g,
                              int32_t* __restrict__ counts)
{
    using C = typename P::C;
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n_tri; t += int64_t(gridDim.x) * blockDim.x)
    {
        const C* const v = tri + 9 * t;
        qv3<C> const a{v[0], v[1], v[2]}, b{v[3], v[4], v[5]}, c{v[6], v[7], v[8]};
        double const y0 = fmin(fmin(P::cdbl(a.y), P::cdbl(b.y)), P::cdbl(c.y));
        double const y1 = fmax(fmax(P::cdbl(a.y), P::cdbl(b.y)), P::cdbl(c.y));
        double const z0 = fmin(fmin(P::cdbl(a.z), P::cdbl(b.z)), P::cdbl(c.z));
        double const z1 = fmax(fmax(P::cdbl(a.z), P::cdbl(b.z)), P::cdbl(c.z));
        int64_t const iy0 = grid_first<T, P>(g.s[1], g.h[1], g.n[1], 1, qz, y0, false);
        int64_t const iy1 = grid_first<T, P>(g.s[1], g.h[1], g.n[1], 1, qz, y1, true);
        int64_t const iz0 = grid_first<T, P>(g.s[2], g.h[2], g.n[2], 2, qz, z0, false);
        int64_t const iz1 = grid_first<T, P>(g.s[2], g.h[2], g.n[2], 2, qz, z1, true);
        for (int64_t iz = iz0; iz < iz1; ++iz)
        {
            C const qzc = grid_pred<T, P>(g.s[2], g.h[2], iz, 2, qz);
            for (int64_t iy = iy0; iy < iy1; ++iy)
            {
                qv3<C> const q{C(0), grid_pred<T, P>(g.s[1], g.h[1], iy, 1, qz), qzc};
                int const e01 = edge_sign<P>(q, a, b);
                int const e12 = edge_sign<P>(q, b, c);
                int const e20 = edge_sign<P>(q, c, a);
                if (e01 == 0 || e01 != e12 || e01 != e20)
                    continue;
                // the hit depth of robust_crossing, with the same operations
                double const w0 = P::dbl(edge_det<P>(q, b, c));
                double const w1 = P::dbl(edge_det<P>(q, c, a));
                double const w2 = P::dbl(edge_det<P>(q, a, b));
                rd const hx = (rd(w0) * rd(P::cdbl(a.x)) + rd(w1) * rd(P::cdbl(b.x)) + rd(w2) * rd(P::cdbl(c.x))) /
                              (rd(w0) + rd(w1) + rd(w2));
                int64_t const ix0 = grid_first<T, P>(g.s[0], g.h[0], g.n[0], 0, qz, hx.v, false);
                if (ix0 < g.n[0])
                    atomicAdd(counts + (iz * g.n[1] + iy) * g.n[0] + ix0, -e01);
            }
        }
    }
}

// Inclusive prefix sum along x of every (y, z) row: one warp per row, 32 cells per step.
__global__ void k_grid_prefix(int32_t* __restrict__ counts, int64_t nx, int64_t rows)
{
    int const lane = threadIdx.x & 31;
    for (int64_t r = (blockIdx.x * int64_t(blockDim.x) + threadIdx.x) >> 5; r < rows;
         r += (int64_t(gridDim.x) * blockDim.x) >> 5)
    {
        int32_t* const row = counts + r * nx;
        int carry = 0;
        for (int64_t x0 = 0; x0 < nx; x0 += 32)
        {
            int64_t const x = x0 + lane;
            int v = x < nx ? row[x] : 0;
            for (int o = 1; o < 32; o <<= 1)
            {
                int const y = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o)
                    v += y;
            }
            v += carry;
            if (x < nx)
                row[x] = v;
            carry = __shfl_sync(0xffffffffu, v, 31);
        }
    }
}

template <class T, class P>
int robust_grid_counts(Context& ctx, const Robust& r, GridSpec const& g, int32_t* d_counts)
{
    using C = typename P::C;
    int64_t const cells = g.n[0] * g.n[1] * g.n[2];
    AGWN_TRY_CUDA(cudaMemsetAsync(d_counts, 0, sizeof(int32_t) * cells, ctx.stream));
    if (r.n_tri == 0)
        return AGWN_OK;
    Quant const qz{{r.center[0], r.center[1], r.center[2]}, r.scale};
    AGWN_TRY(ctx.launch_begin(AGWN_K_ROBUST));
    k_grid_raster<T, P><<<int(std::min<int64_t>(div_up(r.n_tri, 128), 16 * ctx.sm_count)), 128, 0, ctx.stream>>>(
        static_cast<const C*>(r.tri), r.n_tri, qz, g, d_counts);
    AGWN_TRY(ctx.launch_end(AGWN_K_ROBUST));
    int64_t const rows = g.n[1] * g.n[2];
    AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
    k_grid_prefix<<<int(std::min<int64_t>(div_up(rows * 32, 256), 16 * ctx.sm_count)), 256, 0, ctx.stream>>>(
        d_counts, g.n[0], rows);
    return ctx.launch_end(AGWN_K_OTHER);
}

template <class T>
int robust_eval_grid(agwn_context* ctx, const agwn_robust* r, const double* start, const double* spacing, int64_t nx,
                     int64_t ny, int64_t nz, T* out, int32_t* out_counts, T* out_frac)
{
    AGWN_CHECK_ARG(ctx && r && start && spacing, "null argument");
    AGWN_CHECK_ARG(nx >= 0 && ny >= 0 && nz >= 0, "negative grid size");
    AGWN_CHECK_ARG(r->scalar_bytes == int(sizeof(T)), "evaluator precision does not match the output");
    for (int k = 0; k < 3; ++k)
        AGWN_CHECK_ARG(std::isfinite(start[k]) && std::isfinite(spacing[k]) && spacing[k] > 0,
                       "grid start must be finite and spacing positive");
    clear_message();
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    int64_t const cells = nx * ny * nz;
    if (cells == 0)
        return AGWN_OK;
    AGWN_CHECK_ARG(out, "null output");
    AGWN_CHECK_ARG(nx < (int64_t(1) << 31) && ny < (int64_t(1) << 31) && nz < (int64_t(1) << 31) &&
                       cells < (int64_t(1) << 40),
                   "grid too large");
    GridSpec g{{start[0], start[1], start[2]}, {spacing[0], spacing[1], spacing[2]}, {nx, ny, nz}};
    void *dpos = nullptr, *dout = nullptr, *dcnt = nullptr, *dfr = nullptr;
    bool h_out = false, h_cnt = false, h_fr = false;
    AGWN_TRY(ctx->scratch_reserve(S_QUERIES, sizeof(T) * 3 * size_t(cells), &dpos));
    AGWN_TRY(stage_out(*ctx, out, sizeof(T) * cells, S_OUT, &dout, &h_out));
    if (out_counts)
        AGWN_TRY(stage_out(*ctx, out_counts, sizeof(int32_t) * cells, S_COUNTS, &dcnt, &h_cnt));
    else
        AGWN_TRY(ctx->scratch_reserve(S_COUNTS, sizeof(int32_t) * cells, &dcnt));
    if (out_frac)
        AGWN_TRY(stage_out(*ctx, out_frac, sizeof(T) * cells, S_MISC3, &dfr, &h_fr));
    AGWN_TRY(ctx->launch_begin(AGWN_K_OTHER));
    k_grid_positions<T><<<int(std::min<int64_t>(div_up(cells, 256), 16 * ctx->sm_count)), 256, 0, ctx->stream>>>(
        g, static_cast<T*>(dpos));
    AGWN_TRY(ctx->launch_end(AGWN_K_OTHER));
    const T* p = static_cast<const T*>(dpos);
    T* o = static_cast<T*>(dout);
    int32_t* c = static_cast<int32_t*>(dcnt);
    T* fr = static_cast<T*>(dfr);
    switch (r->policy)
    {
    case 0:
        AGWN_TRY((robust_grid_counts<T, P64>(*ctx, *r, g, c)));
        AGWN_TRY((robust_run<T, P64>(*ctx, *r, p, cells, o, c, fr, true)));
        break;
    case 1:
        AGWN_TRY((robust_grid_counts<T, P128>(*ctx, *r, g, c)));
        AGWN_TRY((robust_run<T, P128>(*ctx, *r, p, cells, o, c, fr, true)));
        break;
    default:
        AGWN_TRY((robust_grid_counts<T, PF>(*ctx, *r, g, c)));
        AGWN_TRY((robust_run<T, PF>(*ctx, *r, p, cells, o, c, fr, true)));
        break;
    }
    if (h_out)
        AGWN_TRY_CUDA(cudaMemcpyAsync(out, dout, sizeof(T) * cells, cudaMemcpyDeviceToHost, ctx->stream));
    if (h_cnt)
        AGWN_TRY_CUDA(cudaMemcpyAsync(out_counts, dcnt, sizeof(int32_t) * cells, cudaMemcpyDeviceToHost, ctx->stream));
    if (h_fr)
        AGWN_TRY_CUDA(cudaMemcpyAsync(out_frac, dfr, sizeof(T) * cells, cudaMemcpyDeviceToHost, ctx->stream));
    return (h_out || h_cnt || h_fr) ? ctx->check_flags() : AGWN_OK;
}

} // namespace
} // namespace agwn

using namespace agwn;

extern "C"
{
int agwn_robust_create_f64(agwn_context* ctx, int policy, const double* vertices, int64_t n_vertices,
                           const int32_t* indices, int64_t n_indices, const double* boundary, int64_t n_segments,
                           agwn_robust** out)
{
    return robust_create<double>(ctx, policy, vertices, n_vertices, indices, n_indices, boundary, n_segments, out);
}
int agwn_robust_create_f32(agwn_context* ctx, int policy, const float* vertices, int64_t n_vertices,
                           const int32_t* indices, int64_t n_indices, const float* boundary, int64_t n_segments,
                           agwn_robust** out)
{
    return robust_create<float>(ctx, policy, vertices, n_vertices, indices, n_indices, boundary, n_segments, out);
}
int agwn_robust_destroy(agwn_robust* r)
{
    if (!r)
        return AGWN_OK;
    cudaSetDevice(r->device);
    cudaDeviceSynchronize();
    robust_free(r);
    delete r;
    return AGWN_OK;
}
int agwn_robust_info(const agwn_robust* r, double* center, double* scale, int32_t* depth)
{
    AGWN_CHECK_ARG(r, "null evaluator");
    if (center)
        for (int k = 0; k < 3; ++k)
            center[k] = r->center[k];
    if (scale)
        *scale = r->scale;
    if (depth)
        *depth = r->hier.depth;
    return AGWN_OK;
}
int agwn_robust_eval_f64(agwn_context* ctx, const agwn_robust* r, const double* positions, int64_t n, double* out_gwn,
                         int32_t* out_counts, double* out_frac)
{
    return robust_eval<double>(ctx, r, positions, n, out_gwn, out_counts, out_frac);
}
int agwn_robust_eval_f32(agwn_context* ctx, const agwn_robust* r, const float* positions, int64_t n, float* out_gwn,
                         int32_t* out_counts, float* out_frac)
{
    return robust_eval<float>(ctx, r, positions, n, out_gwn, out_counts, out_frac);
}

int agwn_robust_eval_grid_f64(agwn_context* ctx, const agwn_robust* r, const double* start, const double* spacing,
                              int64_t nx, int64_t ny, int64_t nz, double* out_gwn, int32_t* out_counts,
                              double* out_frac)
{
    return robust_eval_grid<double>(ctx, r, start, spacing, nx, ny, nz, out_gwn, out_counts, out_frac);
}
int agwn_robust_eval_grid_f32(agwn_context* ctx, const agwn_robust* r, const double* start, const double* spacing,
                              int64_t nx, int64_t ny, int64_t nz, float* out_gwn, int32_t* out_counts, float* out_frac)
{
    return robust_eval_grid<float>(ctx, r, start, spacing, nx, ny, nz, out_gwn, out_counts, out_frac);
}
} // extern "C"
