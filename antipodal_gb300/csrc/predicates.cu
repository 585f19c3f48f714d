// The robust evaluator's exact predicates on caller-given coordinates, for testing them on the device against
// the reference's own vectors (test/math/test_robust_predicates.cc): the same device functions (robust.cuh) that
// the robust kernels call, one coordinate tuple per thread.  Also the 128-bit integer products those predicates
// are built from.

#include "agwn_internal.cuh"
#include "robust.cuh"

namespace agwn
{
namespace
{
// Per row i: edge_sign(q, q0, q1), atan2_num(q, q0, q1) as a double, and project_into_tri(q, q0, q1, q2) (its sign
// and, when weights is not null, its three weights).  Coordinates are C triples (int32, int64 or double).
template <class P>
__global__ void k_predicates(const typename P::C* __restrict__ q, const typename P::C* __restrict__ q0,
                             const typename P::C* __restrict__ q1, const typename P::C* __restrict__ q2, int64_t n,
                             int32_t* __restrict__ edge_sign_out, double* __restrict__ num_out,
                             int32_t* __restrict__ inside_out, double* __restrict__ weights)
{
    using C = typename P::C;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    {
        qv3<C> const a{q[3 * i], q[3 * i + 1], q[3 * i + 2]};
        qv3<C> const b{q0[3 * i], q0[3 * i + 1], q0[3 * i + 2]};
        qv3<C> const c{q1[3 * i], q1[3 * i + 1], q1[3 * i + 2]};
        qv3<C> const d{q2[3 * i], q2[3 * i + 1], q2[3 * i + 2]};
        edge_sign_out[i] = edge_sign<P>(a, b, c);
        num_out[i] = P::dbl(atan2_num<P>(a, b, c));
        TriProj const h = project_into_tri<P>(a, b, c, d);
        inside_out[i] = h.sign;
        if (weights)
        {
            weights[3 * i] = h.w0;
            weights[3 * i + 1] = h.w1;
            weights[3 * i + 2] = h.w2;
        }
    }
}

// a*b - c*d in the predicates' 128-bit arithmetic: both words and the correctly rounded double.
__global__ void k_i128_mul_sub(const int64_t* __restrict__ a, const int64_t* __restrict__ b,
                               const int64_t* __restrict__ c, const int64_t* __restrict__ d, int64_t n,
                               uint64_t* __restrict__ lo, int64_t* __restrict__ hi, double* __restrict__ dbl)
{
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    {
        I128 const r = P128::sub(i128_mul(a[i], b[i]), i128_mul(c[i], d[i]));
        lo[i] = r.lo;
        hi[i] = r.hi;
        dbl[i] = i128_to_double(r);
    }
}

int grid_for(Context& ctx, int64_t n)
{
    return int(std::max<int64_t>(1, std::min<int64_t>(div_up(n, 256), 4 * int64_t(ctx.sm_count))));
}
} // namespace
} // namespace agwn

using namespace agwn;

extern "C" int agwn_robust_predicates(agwn_context* ctx, int policy, const void* q, const void* q0, const void* q1,
                                      const void* q2, int64_t n, int32_t* edge_sign_out, double* num_out,
                                      int32_t* inside_out, double* weights)
{
    clear_message();
    AGWN_CHECK_ARG(ctx && n >= 0, "bad arguments");
    AGWN_CHECK_ARG(policy == AGWN_ROBUST_INT64_GRID || policy == AGWN_ROBUST_INT128_GRID ||
                       policy == AGWN_ROBUST_EXACT_FLOAT,
                   "unknown precision policy %d", policy);
    AGWN_CHECK_ARG(n == 0 || (q && q0 && q1 && q2 && edge_sign_out && num_out && inside_out), "null array");
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    if (n == 0)
        return AGWN_OK;
    size_t const coord = policy == AGWN_ROBUST_INT64_GRID ? sizeof(int32_t) : 8;
    size_t const in_bytes = 3 * coord * size_t(n);
    const void* d_in[4] = {};
    const void* const h_in[4] = {q, q0, q1, q2};
    for (int k = 0; k < 4; ++k)
        AGWN_TRY(stage_in(*ctx, h_in[k], in_bytes, S_MISC0 + k, &d_in[k]));
    void *d_es = nullptr, *d_num = nullptr, *d_ins = nullptr, *d_w = nullptr;
    bool h_es = false, h_num = false, h_ins = false, h_w = false;
    AGWN_TRY(stage_out(*ctx, edge_sign_out, sizeof(int32_t) * n, S_OUT, &d_es, &h_es));
    AGWN_TRY(stage_out(*ctx, num_out, sizeof(double) * n, S_QUERIES, &d_num, &h_num));
    AGWN_TRY(stage_out(*ctx, inside_out, sizeof(int32_t) * n, S_COUNTS, &d_ins, &h_ins));
    if (weights)
        AGWN_TRY(stage_out(*ctx, weights, 3 * sizeof(double) * n, S_PARTIAL, &d_w, &h_w));
    int const grid = grid_for(*ctx, n);
    auto launch = [&](auto tag)
    {
        using P = decltype(tag);
        using C = typename P::C;
        k_predicates<P><<<grid, 256, 0, ctx->stream>>>(
            static_cast<const C*>(d_in[0]), static_cast<const C*>(d_in[1]), static_cast<const C*>(d_in[2]),
            static_cast<const C*>(d_in[3]), n, static_cast<int32_t*>(d_es), static_cast<double*>(d_num),
            static_cast<int32_t*>(d_ins), static_cast<double*>(d_w));
    };
    if (policy == AGWN_ROBUST_INT64_GRID)
        launch(P64{});
    else if (policy == AGWN_ROBUST_INT128_GRID)
        launch(P128{});
    else
        launch(PF{});
    AGWN_TRY_CUDA(cudaGetLastError());
    if (h_es)
        AGWN_TRY_CUDA(cudaMemcpyAsync(edge_sign_out, d_es, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (h_num)
        AGWN_TRY_CUDA(cudaMemcpyAsync(num_out, d_num, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (h_ins)
        AGWN_TRY_CUDA(cudaMemcpyAsync(inside_out, d_ins, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (h_w)
        AGWN_TRY_CUDA(cudaMemcpyAsync(weights, d_w, 3 * sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    AGWN_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
    return AGWN_OK;
}

extern "C" int agwn_probe_i128_mul_sub(agwn_context* ctx, const int64_t* a, const int64_t* b, const int64_t* c,
                                       const int64_t* d, int64_t n, uint64_t* lo, int64_t* hi, double* dbl)
{
    clear_message();
    AGWN_CHECK_ARG(ctx && n >= 0, "bad arguments");
    AGWN_CHECK_ARG(n == 0 || (a && b && c && d && lo && hi && dbl), "null array");
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    if (n == 0)
        return AGWN_OK;
    size_t const bytes = sizeof(int64_t) * size_t(n);
    const void* d_in[4] = {};
    const void* const h_in[4] = {a, b, c, d};
    for (int k = 0; k < 4; ++k)
        AGWN_TRY(stage_in(*ctx, h_in[k], bytes, S_MISC0 + k, &d_in[k]));
    void *d_lo = nullptr, *d_hi = nullptr, *d_dbl = nullptr;
    bool h_lo = false, h_hi = false, h_dbl = false;
    AGWN_TRY(stage_out(*ctx, lo, bytes, S_OUT, &d_lo, &h_lo));
    AGWN_TRY(stage_out(*ctx, hi, bytes, S_COUNTS, &d_hi, &h_hi));
    AGWN_TRY(stage_out(*ctx, dbl, bytes, S_QUERIES, &d_dbl, &h_dbl));
    k_i128_mul_sub<<<grid_for(*ctx, n), 256, 0, ctx->stream>>>(
        static_cast<const int64_t*>(d_in[0]), static_cast<const int64_t*>(d_in[1]), static_cast<const int64_t*>(d_in[2]),
        static_cast<const int64_t*>(d_in[3]), n, static_cast<uint64_t*>(d_lo), static_cast<int64_t*>(d_hi),
        static_cast<double*>(d_dbl));
    AGWN_TRY_CUDA(cudaGetLastError());
    if (h_lo)
        AGWN_TRY_CUDA(cudaMemcpyAsync(lo, d_lo, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    if (h_hi)
        AGWN_TRY_CUDA(cudaMemcpyAsync(hi, d_hi, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    if (h_dbl)
        AGWN_TRY_CUDA(cudaMemcpyAsync(dbl, d_dbl, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    AGWN_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
    return AGWN_OK;
}
