// Spatial order of the queries for the mixed kernels.
//
// The mixed fractional kernel certifies boundary groups per warp against the circles, across the ray, of the warp's
// query slots (32 consecutive queries each), so its speed depends on the order of the queries: warps of nearby
// queries certify most groups, warps of scattered queries almost none.  A query's value does not depend on the warp
// it lands in -- the certified and the per-pair paths give the same values bit for bit, and each query's pairs are
// summed in boundary order either way -- so an incoherent order can be replaced by a spatial one without changing a
// result: a 24-bit 2D Morton key of every query's position across the ray, a stable radix sort of (key, index) in
// three 8-bit passes (with a parallel scan of the digit counters), a gather of the queries, the evaluation on the
// sorted copy, and a scatter of the results.  (16-bit keys in two passes sorted faster but left the integer term's
// cell lookups less local: 400M against 430M queries/s on two tori of 1M triangles with 1e7 random queries.)
//
// The decision: a sample of the slots (one in 16) gives the mean slot radius across the ray and the sample's RMS
// spread; a mean radius above a quarter of the spread counts as incoherent (queries in grid order: ~0.15, in random
// order: ~1.4).  For the caller's own device arrays the decision is kept per (pointer, size, direction), so repeated
// calls on the same arrays take no host synchronisation; since it only affects speed, a stale decision after the
// data changed costs time, not results.
#include "agwn_internal.cuh"
#include "gwn_kernels.cuh"
#include "radix.cuh"

#include <cmath>

namespace agwn
{
namespace
{
// an orthonormal pair (u, v) across the direction
struct Across
{
    double u[3], v[3];
};

Across across_of(const double* dir)
{
    double const n = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    double const z[3] = {dir[0] / n, dir[1] / n, dir[2] / n};
    int m = 0;
    for (int k = 1; k < 3; ++k)
        if (std::fabs(z[k]) < std::fabs(z[m]))
            m = k;
    double a[3] = {0, 0, 0};
    a[m] = 1.0;
    double u[3] = {a[1] * z[2] - a[2] * z[1], a[2] * z[0] - a[0] * z[2], a[0] * z[1] - a[1] * z[0]};
    double const un = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    for (double& c : u)
        c /= un;
    Across r;
    for (int k = 0; k < 3; ++k)
        r.u[k] = u[k];
    r.v[0] = z[1] * u[2] - z[2] * u[1];
    r.v[1] = z[2] * u[0] - z[0] * u[2];
    r.v[2] = z[0] * u[1] - z[1] * u[0];
    return r;
}

__device__ __forceinline__ float2 across(const double* __restrict__ p, Across const& a)
{
    double const x = p[0], y = p[1], z = p[2];
    return make_float2(float(a.u[0] * x + a.u[1] * y + a.u[2] * z), float(a.v[0] * x + a.v[1] * y + a.v[2] * z));
}

constexpr int kSampleStride = 16; // one slot of 32 queries in every 16
constexpr int kOrderBlock = 256;

// acc (6 doubles): sampled slots, sum of slot radii, sum x, sum y, sum x^2, sum y^2 (across the ray).  One warp per
// sampled slot; only full slots are sampled.
__global__ void __launch_bounds__(kOrderBlock) k_order_sample(const double* __restrict__ pos, int64_t n, Across a,
                                                              double* __restrict__ acc)
{
    __shared__ double part[kOrderBlock / 32][6];
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t const n_samp = (n / 32 + kSampleStride - 1) / kSampleStride;
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int64_t w = int64_t(blockIdx.x) * (kOrderBlock / 32) + warp; w < n_samp;
         w += int64_t(gridDim.x) * (kOrderBlock / 32))
    {
        int64_t const i = w * kSampleStride * 32 + lane; // < n: the slot is full
        float2 const p = across(pos + 3 * i, a);
        float x0 = p.x, x1 = p.x, y0 = p.y, y1 = p.y;
        for (int o = 16; o > 0; o >>= 1)
        {
            x0 = fminf(x0, __shfl_xor_sync(0xffffffffu, x0, o));
            x1 = fmaxf(x1, __shfl_xor_sync(0xffffffffu, x1, o));
            y0 = fminf(y0, __shfl_xor_sync(0xffffffffu, y0, o));
            y1 = fmaxf(y1, __shfl_xor_sync(0xffffffffu, y1, o));
        }
        if (lane == 0)
        {
            s[0] += 1.0;
            s[1] += 0.5 * sqrt(double(x1 - x0) * double(x1 - x0) + double(y1 - y0) * double(y1 - y0));
        }
        s[2] += p.x;
        s[3] += p.y;
        s[4] += double(p.x) * p.x;
        s[5] += double(p.y) * p.y;
    }
    for (int k = 2; k < 6; ++k)
        for (int o = 16; o > 0; o >>= 1)
            s[k] += __shfl_xor_sync(0xffffffffu, s[k], o);
    if (lane == 0)
        for (int k = 0; k < 6; ++k)
            part[warp][k] = s[k];
    __syncthreads();
    if (threadIdx.x < 6)
    {
        double t = 0;
        for (int w = 0; w < kOrderBlock / 32; ++w)
            t += part[w][threadIdx.x];
        atomicAdd(&acc[threadIdx.x], t);
    }
}

__device__ __forceinline__ uint32_t spread12(uint32_t x)
{
    x &= 0xfffu;
    x = (x | (x << 8)) & 0x00ff00ffu;
    x = (x | (x << 4)) & 0x0f0f0f0fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
}

// 2D Morton key of each query across the ray, quantised to 12 bits per axis over [lo, lo + 4095 / scale] (the mean
// -+ 4 RMS spreads; positions outside clamp to the edge), and its index.  A cell is 1/512 of the RMS spread across:
// far below the reach of a boundary group, and fine enough that the integer term's cell lookups of neighbouring
// queries share their cache lines.
__global__ void k_order_keys(const double* __restrict__ pos, int64_t n, Across a, float lox, float loy, float scale,
                             uint32_t* __restrict__ keys, int32_t* __restrict__ idx)
{
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    {
        float2 const p = across(pos + 3 * i, a);
        float const qx = fminf(fmaxf((p.x - lox) * scale, 0.f), 4095.f);
        float const qy = fminf(fmaxf((p.y - loy) * scale, 0.f), 4095.f);
        // a NaN coordinate takes key 0 (fminf/fmaxf return the number)
        keys[i] = spread12(uint32_t(qx)) | (spread12(uint32_t(qy)) << 1);
        idx[i] = int32_t(i);
    }
}

__global__ void k_gather_queries(const double* __restrict__ pos, const int32_t* __restrict__ perm, int64_t n,
                                 double* __restrict__ out)
{
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    {
        int64_t const j = perm[i];
        out[3 * i] = pos[3 * j];
        out[3 * i + 1] = pos[3 * j + 1];
        out[3 * i + 2] = pos[3 * j + 2];
    }
}

template <class T>
__global__ void k_scatter_back(const T* __restrict__ src, const int32_t* __restrict__ perm, int64_t n,
                               T* __restrict__ dst)
{
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        dst[perm[i]] = src[i];
}
} // namespace

int query_order(Context& ctx, const double* d_pos, int64_t n, const double* dir, bool cacheable,
                const int32_t** perm)
{
    *perm = nullptr;
    if (n < kOrderMinQueries || n >= (int64_t(1) << 31) || !ctx.mixed_certify)
        return AGWN_OK;
    cudaStream_t const st = ctx.stream;
    Across const a = across_of(dir);
    bool const cached = cacheable && ctx.order_ptr == d_pos && ctx.order_n == n && ctx.order_dir[0] == dir[0] &&
                        ctx.order_dir[1] == dir[1] && ctx.order_dir[2] == dir[2];
    if (!cached)
    {
        double* acc = nullptr;
        AGWN_TRY(ctx.scratch_reserve(S_ORDER0, sizeof(double) * 6, reinterpret_cast<void**>(&acc)));
        AGWN_TRY_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * 6, st));
        int64_t const n_samp = (n / 32 + kSampleStride - 1) / kSampleStride;
        int const grid = int(std::max<int64_t>(1, std::min<int64_t>(div_up(n_samp, kOrderBlock / 32),
                                                                    int64_t(4) * ctx.sm_count)));
        AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
        k_order_sample<<<grid, kOrderBlock, 0, st>>>(d_pos, n, a, acc);
        AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
        double h[6] = {};
        AGWN_TRY_CUDA(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, st));
        AGWN_TRY_CUDA(cudaStreamSynchronize(st));
        double const m = std::max(1.0, h[0] * 32.0);
        double const mx = h[2] / m, my = h[3] / m;
        double const var = std::max(0.0, h[4] / m - mx * mx) + std::max(0.0, h[5] / m - my * my);
        double const rms = std::sqrt(var), mean_r = h[1] / std::max(1.0, h[0]);
        ctx.order_ptr = cacheable ? d_pos : nullptr;
        ctx.order_n = n;
        for (int k = 0; k < 3; ++k)
            ctx.order_dir[k] = dir[k];
        ctx.order_incoherent = std::isfinite(rms) && rms > 0 && mean_r > 0.25 * rms;
        ctx.order_lo[0] = float(mx - 4.0 * rms);
        ctx.order_lo[1] = float(my - 4.0 * rms);
        ctx.order_scale = float(4095.0 / std::max(8.0 * rms, 1e-30));
    }
    if (!ctx.order_incoherent)
        return AGWN_OK;
    // keys and indices, ping-pong buffers of the sort, its digit counters and their block sums
    int const n_rs_blocks = div_up(n, kRsTile);
    int64_t const n_cnt = int64_t(256) * n_rs_blocks;
    int64_t const n_cb = scan_sums_count(n_cnt);
    size_t const off_hist = sizeof(uint32_t) * 4 * size_t(n);
    void* base = nullptr;
    AGWN_TRY(ctx.scratch_reserve(S_ORDER0, off_hist + sizeof(unsigned) * (size_t(n_cnt) + size_t(n_cb)), &base));
    uint32_t* const ka = static_cast<uint32_t*>(base);
    uint32_t* const kb = ka + n;
    int32_t* const va = reinterpret_cast<int32_t*>(kb + n);
    int32_t* const vb = va + n;
    unsigned* const hist = reinterpret_cast<unsigned*>(static_cast<char*>(base) + off_hist);
    unsigned* const csum = hist + n_cnt;
    int const g = int(std::min<int64_t>(div_up(n, 256), int64_t(8) * ctx.sm_count));
    AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
    k_order_keys<<<g, 256, 0, st>>>(d_pos, n, a, ctx.order_lo[0], ctx.order_lo[1], ctx.order_scale, ka, va);
    AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
    uint32_t* kin = ka;
    uint32_t* kout = kb;
    int32_t* vin = va;
    int32_t* vout = vb;
    for (int pass = 0; pass < 3; ++pass) // the 24-bit keys
    {
        int const shift = 8 * pass;
        AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
        k_rs_hist<<<n_rs_blocks, kRsBlock, 0, st>>>(kin, n, shift, hist, n_rs_blocks);
        scan_counters(st, hist, n_cnt, csum);
        k_rs_scatter<<<n_rs_blocks, kRsBlock, 0, st>>>(kin, vin, n, shift, hist, n_rs_blocks, kout, vout);
        AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    *perm = vin; // the sorted indices (the second buffers after three passes)
    return AGWN_OK;
}

int gather_queries(Context& ctx, const double* d_pos, const int32_t* perm, int64_t n, double* d_sorted)
{
    int const g = int(std::min<int64_t>(div_up(n, 256), int64_t(8) * ctx.sm_count));
    AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
    k_gather_queries<<<g, 256, 0, ctx.stream>>>(d_pos, perm, n, d_sorted);
    return ctx.launch_end(AGWN_K_OTHER);
}

template <class T>
int scatter_back(Context& ctx, const T* d_sorted, const int32_t* perm, int64_t n, T* d_out)
{
    int const g = int(std::min<int64_t>(div_up(n, 256), int64_t(8) * ctx.sm_count));
    AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
    k_scatter_back<T><<<g, 256, 0, ctx.stream>>>(d_sorted, perm, n, d_out);
    return ctx.launch_end(AGWN_K_OTHER);
}
template int scatter_back<double>(Context&, const double*, const int32_t*, int64_t, double*);
template int scatter_back<int32_t>(Context&, const int32_t*, const int32_t*, int64_t, int32_t*);
} // namespace agwn
