// Throughput probe: the FP32 FMA rate this GPU sustains at its current clocks, the denominator of the
// fractional kernel's compute roofline (the kernel is bound by the FP32 pipe, not by HBM or tensor cores).

#include "agwn_internal.cuh"
#include "frac_kernels.cuh"

namespace agwn
{
namespace
{
constexpr int kChains = 8;

// Each thread runs kChains independent FMA chains for `iters` steps.  The result is stored only if it equals a
// value that cannot occur, so the chains are kept but nothing is written.
__global__ void __launch_bounds__(256) k_ffma(int iters, float a, float b, float* sink)
{
    float v[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c)
        v[c] = a + float(threadIdx.x + c);
    for (int i = 0; i < iters; ++i)
    {
#pragma unroll
        for (int c = 0; c < kChains; ++c)
            v[c] = fmaf(v[c], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; ++c)
        s += v[c];
    if (s == -1.2345e-30f)
        sink[0] = s;
}
// The same for FP64 fused multiply-add (the parametric integrator's pipe).
__global__ void __launch_bounds__(256) k_dfma(int iters, double a, double b, double* sink)
{
    double v[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c)
        v[c] = a + double(threadIdx.x + c);
    for (int i = 0; i < iters; ++i)
    {
#pragma unroll
        for (int c = 0; c < kChains; ++c)
            v[c] = fma(v[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; ++c)
        s += v[c];
    if (s == -1.2345e-300)
        sink[0] = s;
}
} // namespace
} // namespace agwn

using namespace agwn;

extern "C" int agwn_probe_fp64_peak(agwn_context* ctx, double* tflops)
{
    AGWN_CHECK_ARG(ctx && tflops, "null argument");
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    double* sink = nullptr;
    AGWN_TRY(ctx->scratch_reserve(S_MISC3, sizeof(double), reinterpret_cast<void**>(&sink)));
    int per_sm = 0;
    AGWN_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dfma, 256, 0));
    int const grid = ctx->sm_count * per_sm;
    int const iters = 1 << 10;
    cudaEvent_t e0, e1;
    AGWN_TRY_CUDA(cudaEventCreate(&e0));
    AGWN_TRY_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep)
    {
        AGWN_TRY_CUDA(cudaEventRecord(e0, ctx->stream));
        k_dfma<<<grid, 256, 0, ctx->stream>>>(iters, 0.9999, 1e-4, sink);
        AGWN_TRY_CUDA(cudaEventRecord(e1, ctx->stream));
        AGWN_TRY_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        AGWN_TRY_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0 && ms < best)
            best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    double const flops = 2.0 * kChains * double(iters) * double(grid) * 256.0;
    *tflops = flops / (double(best) * 1e-3) / 1e12;
    return AGWN_OK;
}

extern "C" int agwn_probe_fp32_peak(agwn_context* ctx, double* tflops)
{
    AGWN_CHECK_ARG(ctx && tflops, "null argument");
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    float* sink = nullptr;
    AGWN_TRY(ctx->scratch_reserve(S_MISC3, sizeof(float), reinterpret_cast<void**>(&sink)));
    int per_sm = 0;
    AGWN_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ffma, 256, 0));
    int const grid = ctx->sm_count * per_sm * 4;
    int const iters = 1 << 14;
    cudaEvent_t e0, e1;
    AGWN_TRY_CUDA(cudaEventCreate(&e0));
    AGWN_TRY_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep)
    {
        AGWN_TRY_CUDA(cudaEventRecord(e0, ctx->stream));
        k_ffma<<<grid, 256, 0, ctx->stream>>>(iters, 0.9999f, 1e-4f, sink);
        AGWN_TRY_CUDA(cudaEventRecord(e1, ctx->stream));
        AGWN_TRY_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        AGWN_TRY_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0 && ms < best)
            best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    double const flops = 2.0 * kChains * double(iters) * double(grid) * 256.0;
    *tflops = flops / (double(best) * 1e-3) / 1e12;
    return AGWN_OK;
}

namespace agwn
{
namespace
{
__global__ void k_atan2_pair(const float* __restrict__ y, const float* __restrict__ x, int64_t n,
                             float* __restrict__ ours, float* __restrict__ ref)
{
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    {
        ours[i] = atan2_fast(y[i], x[i]);
        ref[i] = atan2f(y[i], x[i]);
    }
}
} // namespace
} // namespace agwn

extern "C" int agwn_probe_atan2(agwn_context* ctx, const float* y, const float* x, int64_t n, float* ours, float* ref)
{
    AGWN_CHECK_ARG(ctx && n >= 0 && (n == 0 || (y && x && ours && ref)), "bad arguments");
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    if (n == 0)
        return AGWN_OK;
    const void *dy = nullptr, *dx = nullptr;
    void *d_ours = nullptr, *d_ref = nullptr;
    bool h1 = false, h2 = false;
    AGWN_TRY(stage_in(*ctx, y, sizeof(float) * n, S_MISC0, &dy));
    AGWN_TRY(stage_in(*ctx, x, sizeof(float) * n, S_MISC1, &dx));
    AGWN_TRY(stage_out(*ctx, ours, sizeof(float) * n, S_MISC2, &d_ours, &h1));
    AGWN_TRY(stage_out(*ctx, ref, sizeof(float) * n, S_MISC3, &d_ref, &h2));
    k_atan2_pair<<<std::min<int64_t>(div_up(n, 256), 4 * ctx->sm_count), 256, 0, ctx->stream>>>(
        static_cast<const float*>(dy), static_cast<const float*>(dx), n, static_cast<float*>(d_ours),
        static_cast<float*>(d_ref));
    AGWN_TRY_CUDA(cudaGetLastError());
    if (h1)
        AGWN_TRY_CUDA(cudaMemcpyAsync(ours, d_ours, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (h2)
        AGWN_TRY_CUDA(cudaMemcpyAsync(ref, d_ref, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
    AGWN_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
    return AGWN_OK;
}
