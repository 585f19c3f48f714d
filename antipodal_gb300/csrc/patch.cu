// Integer term of the parametric GWN: signed crossings of the ray p + lambda x0 (lambda > 0) with bicubic Bezier
// patches, the Intersector that eval_gwnr_parametric_batch_integer / eval_gwnr_parametric_batch forward to
// (src/antipodal/gwn_parametric.hh:204-284).  The reference ships no parametric intersector (its README lists one
// as future work), so this one is specified by the mesh intersector's rule: every crossing in front of the query
// counts sign(N . x0), N = S_u x S_v the patch normal, whose orientation matches boundary curves that run
// counter-clockwise in (u, v) (the patch on their left).
//
// Method, per (query, patch).  In a right-handed frame whose third axis is the ray direction, the patch relative to
// the query is a map F(u, v) = (x, y) of the parameter square with a depth w, and the crossings are F's roots with
// w > 0.  Over a cell of the square whose depth is positive throughout, the signed root count is F's topological
// degree at the origin: the winding number about the origin of the image of the cell's boundary, 4 cubics.  So:
//   * a cell (its control net blossomed from the patch's) is dropped when its net's (x, y) box misses the origin or
//     its depths are all negative, gives its boundary's winding number when its depths are all positive, and is
//     split in four otherwise;
//   * a boundary cubic is split in two while its control points' box holds the origin; a piece whose box does not
//     contributes the crossing of its chord with the positive x axis (the chord and the piece wind alike about a
//     point outside the box).
// Every box test keeps a margin above the rounding of the values it compares (blossoms are taken from the patch's
// own net at dyadic parameters, so that rounding does not grow with the depth of a split), hence each decision,
// and the count, holds for the exact map.  Unlike Newton's iteration the degree needs no root to be isolated: two
// crossings near a fold of the map (a ray almost tangent to the patch) cancel in it as they should.
// Each pair runs first in float with a margin of 2^-16 of the coordinates' scale; a decision that float cannot
// make (a boundary image or the surface within that margin of the ray) sends the pair to FP64 with a margin of
// 2^-42.  What FP64 cannot make either is degenerate (the ray on a cell boundary's image within 2^-42 of the scale,
// or the query that close to the surface): it is decided by a fixed rule and counted.

#include "agwn_internal.cuh"
#include "hier.cuh"

#include <cmath>
#include <mutex>

namespace agwn
{
namespace
{
constexpr int kPatchBlock = 128;

template <class R>
struct PatchArith;

template <>
struct PatchArith<float>
{
    using Index = uint32_t; // cell indices below 2^kMaxCellLevel
    static constexpr int kMaxCellLevel = 16;
    static constexpr int kMaxEdgeLevel = 16;
    static constexpr bool kExact = false; // an unresolved decision abandons the pair (it is redone in FP64)
    __device__ static float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
    __device__ static float pow2(int e) { return __int_as_float((127 + e) << 23); } // 2^e, -126 <= e <= 127
};

template <>
struct PatchArith<double>
{
    using Index = uint64_t;
    // deep enough that the depth range of a cell (about 2^-level of the patch) falls below the margin first
    static constexpr int kMaxCellLevel = 45;
    static constexpr int kMaxEdgeLevel = 50;
    static constexpr bool kExact = true; // an unresolved decision is degenerate: fixed rule, counted
    __device__ static double fma(double a, double b, double c) { return __fma_rn(a, b, c); }
    __device__ static double pow2(int e) { return __longlong_as_double(int64_t(1023 + e) << 52); }
};

// Control values of the cubic c over [a, b] by blossoming: B(a,a,a), B(a,a,b), B(a,b,b), B(b,b,b).  B(t,t,t) takes
// the same steps whichever end t is, so neighbouring pieces share their end point bit for bit.
template <class R>
__device__ __forceinline__ void cubic_on(R c0, R c1, R c2, R c3, R a, R b, R (&o)[4])
{
    auto const lerp = [](R p, R q, R t) { return PatchArith<R>::fma(t, q - p, p); };
    R const a0 = lerp(c0, c1, a), a1 = lerp(c1, c2, a), a2 = lerp(c2, c3, a);
    R const b0 = lerp(c0, c1, b), b1 = lerp(c1, c2, b), b2 = lerp(c2, c3, b);
    R const aa0 = lerp(a0, a1, a), aa1 = lerp(a1, a2, a);
    R const ab0 = lerp(a0, a1, b), ab1 = lerp(a1, a2, b);
    R const bb0 = lerp(b0, b1, b), bb1 = lerp(b1, b2, b);
    o[0] = lerp(aa0, aa1, a);
    o[1] = lerp(aa0, aa1, b);
    o[2] = lerp(ab0, ab1, b);
    o[3] = lerp(bb0, bb1, b);
}

// The crossing of the chord a -> b with the positive x axis: +1 upwards with the origin on its left, -1 downwards
// with the origin on its right; half-open in y, so chords that meet on the axis count once.
template <class R>
__device__ __forceinline__ int chord_crossing(R ax, R ay, R bx, R by)
{
    R const cross = PatchArith<R>::fma(ax, by, -(ay * bx));
    if (ay <= R(0))
        return (by > R(0) && cross > R(0)) ? 1 : 0;
    return (by <= R(0) && cross < R(0)) ? -1 : 0;
}

// Winding number about the origin of the cubic with control points (x_k, y_k), by binary subdivision in a stackless
// walk (piece i of level L covers [i, i + 1] 2^-L).  unresolved: counts the pieces that hold the origin within the
// margin m and cannot be split further.
template <class R>
__device__ int cubic_winding(R x0, R x1, R x2, R x3, R y0, R y1, R y2, R y3, R m, int& unresolved, int& pieces)
{
    using A = PatchArith<R>;
    int w = 0, level = 0;
    int64_t i = 0;
    for (;;)
    {
        ++pieces;
        R px[4], py[4];
        if (level == 0)
        {
            px[0] = x0, px[1] = x1, px[2] = x2, px[3] = x3;
            py[0] = y0, py[1] = y1, py[2] = y2, py[3] = y3;
        }
        else
        {
            R const h = A::pow2(-level);
            R const t0 = R(i) * h, t1 = R(i + 1) * h;
            cubic_on(x0, x1, x2, x3, t0, t1, px);
            cubic_on(y0, y1, y2, y3, t0, t1, py);
        }
        R const xlo = fmin(fmin(px[0], px[1]), fmin(px[2], px[3])), xhi = fmax(fmax(px[0], px[1]), fmax(px[2], px[3]));
        R const ylo = fmin(fmin(py[0], py[1]), fmin(py[2], py[3])), yhi = fmax(fmax(py[0], py[1]), fmax(py[2], py[3]));
        if (!(xlo > m || xhi < -m || ylo > m || yhi < -m))
        {
            if (level < A::kMaxEdgeLevel && fmax(xhi - xlo, yhi - ylo) >= R(4) * m)
            {
                ++level;
                i *= 2;
                continue;
            }
            ++unresolved;
            if (!A::kExact)
                return 0;
        }
        bool const last = i + 1 == (int64_t(1) << level); // the piece ends at t = 1: the cubic's own end point
        w += chord_crossing(px[0], py[0], last ? x3 : px[3], last ? y3 : py[3]);
        while (level > 0 && (i & 1))
        {
            i >>= 1;
            --level;
        }
        if (level == 0)
            break;
        ++i;
    }
    return w;
}

// One coordinate of the net of cell (iu, iv) of level L, blossomed from the patch's net: c(4 r + q, k) is control
// point (r the v index, q the u index) coordinate k relative to the query.  out[4 r + q].
template <class R, class Net, class I>
__device__ __forceinline__ void cell_net(Net const& c, int k, int level, I iu, I iv, R (&out)[16])
{
    if (level == 0)
    {
#pragma unroll
        for (int j = 0; j < 16; ++j)
            out[j] = c(j, k);
        return;
    }
    R const h = PatchArith<R>::pow2(-level);
    R const u0 = R(iu) * h, u1 = R(iu + 1) * h, v0 = R(iv) * h, v1 = R(iv + 1) * h;
    R rows[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
        cubic_on(c(4 * r, k), c(4 * r + 1, k), c(4 * r + 2, k), c(4 * r + 3, k), u0, u1, rows[r]);
#pragma unroll
    for (int q = 0; q < 4; ++q)
    {
        R col[4];
        cubic_on(rows[0][q], rows[1][q], rows[2][q], rows[3][q], v0, v1, col);
#pragma unroll
        for (int r = 0; r < 4; ++r)
            out[4 * r + q] = col[r];
    }
}

template <class R>
__device__ __forceinline__ void range16(const R (&v)[16], R& lo, R& hi)
{
    lo = hi = v[0];
#pragma unroll
    for (int j = 1; j < 16; ++j)
    {
        lo = fmin(lo, v[j]);
        hi = fmax(hi, v[j]);
    }
}

// Winding number about the origin of a cell net's boundary, counter-clockwise in (u, v).
template <class R>
__device__ __forceinline__ int net_winding(const R (&x)[16], const R (&y)[16], R m, int& unresolved, int& pieces)
{
    int w = cubic_winding(x[0], x[1], x[2], x[3], y[0], y[1], y[2], y[3], m, unresolved, pieces);
    w += cubic_winding(x[3], x[7], x[11], x[15], y[3], y[7], y[11], y[15], m, unresolved, pieces);
    w += cubic_winding(x[15], x[14], x[13], x[12], y[15], y[14], y[13], y[12], m, unresolved, pieces);
    w += cubic_winding(x[12], x[8], x[4], x[0], y[12], y[8], y[4], y[0], m, unresolved, pieces);
    return w;
}

// Signed crossings in front of the query with one patch, c(j, k) its net relative to the query in the ray frame
// (k = x, y across the ray and w along it), m the margin.  Cells are walked depth first without a stack:
// (level, iu, iv), children 2 iu + (0|1), 2 iv + (0|1) in the order (0,0), (1,0), (0,1), (1,1).  unresolved counts
// the decisions the margin did not allow (float: the result is void and the pair is redone in FP64); cells and
// pieces count the work (cells tested, boundary-cubic pieces tested).
template <class R, class Net>
__device__ int patch_degree(Net const& c, R m, int& unresolved, int& cells, int& pieces)
{
    using A = PatchArith<R>;
    int sum = 0, level = 0;
    typename A::Index iu = 0, iv = 0;
    for (;;)
    {
        ++cells;
        R x[16], y[16], lo, hi;
        cell_net(c, 0, level, iu, iv, x);
        range16(x, lo, hi);
        bool descend = false;
        if (!(lo > m || hi < -m))
        {
            cell_net(c, 1, level, iu, iv, y);
            range16(y, lo, hi);
            if (!(lo > m || hi < -m))
            {
                R w[16];
                cell_net(c, 2, level, iu, iv, w);
                range16(w, lo, hi);
                if (lo >= m)
                    sum += net_winding(x, y, m, unresolved, pieces); // in front throughout
                else if (hi >= -m)
                {
                    // the depth changes sign over the cell, or lies within the margin of 0
                    if (level < A::kMaxCellLevel && hi - lo >= R(4) * m)
                        descend = true;
                    else
                    {
                        ++unresolved;
                        if (A::kExact && lo + hi >= R(0))
                            sum += net_winding(x, y, m, unresolved, pieces);
                    }
                }
                if (!A::kExact && unresolved)
                    return 0;
            }
        }
        if (descend)
        {
            ++level;
            iu *= 2;
            iv *= 2;
            continue;
        }
        while (level > 0 && (iu & 1) && (iv & 1))
        {
            iu >>= 1;
            iv >>= 1;
            --level;
        }
        if (level == 0)
            break;
        if (iu & 1)
        {
            iu -= 1;
            iv += 1;
        }
        else
            iu += 1;
    }
    return sum;
}

// The FP64 pass of one pair: the patch's FP64 net (ray frame) relative to the query, margin 2^-42 of `scale`.
__device__ __noinline__ int patch_degree_fp64(const double* __restrict__ net, double qx, double qy, double qw,
                                              double scale, int& degenerate, int& cells, int& pieces)
{
    auto const c = [=](int j, int k) { return net[3 * j + k] - (k == 0 ? qx : (k == 1 ? qy : qw)); };
    return patch_degree(c, scale * 0x1p-42, degenerate, cells, pieces);
}

// The patches' control points in the ray frame (rows of f): net in FP64, netf rounded to float, and per patch
// boxf[8 k ..] = xmin, xmax, ymin, ymax, wmin, wmax, largest |coordinate|, 0 in float (rounded to nearest: every
// test on them keeps a margin far above that rounding).
__global__ void k_patch_frame(const double* __restrict__ ctrl, int64_t n_patches, Frame64 f, double* __restrict__ net,
                              float* __restrict__ netf, float* __restrict__ boxf)
{
    for (int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; k < n_patches;
         k += int64_t(gridDim.x) * blockDim.x)
    {
        double b[7] = {INFINITY, -INFINITY, INFINITY, -INFINITY, INFINITY, -INFINITY, 0.0};
        for (int j = 0; j < 16; ++j)
        {
            const double* p = ctrl + 48 * k + 3 * j;
            for (int r = 0; r < 3; ++r)
            {
                double const x = f.r[3 * r] * p[0] + f.r[3 * r + 1] * p[1] + f.r[3 * r + 2] * p[2];
                net[48 * k + 3 * j + r] = x;
                netf[48 * k + 3 * j + r] = float(x);
                b[2 * r] = fmin(b[2 * r], x);
                b[2 * r + 1] = fmax(b[2 * r + 1], x);
                b[6] = fmax(b[6], fabs(x));
            }
        }
        for (int r = 0; r < 7; ++r)
            boxf[8 * k + r] = float(b[r]);
        boxf[8 * k + 7] = 0.f;
    }
}

// One query per thread against every patch.  counts / add: the crossing count is written to counts (int) or added
// to add (the fractional term already there); degenerate (nullable): per query, the decisions left to the fixed
// rule; stats (nullable): adds pairs past the box test, cells, pieces and FP64 pairs to stats[0..3].
__global__ void __launch_bounds__(kPatchBlock) k_patch_count(const double* __restrict__ net,
                                                             const float* __restrict__ netf,
                                                             const float4* __restrict__ boxf, int64_t n_patches,
                                                             Frame64 f, const double* __restrict__ pos, int64_t n,
                                                             int32_t* __restrict__ counts, double* __restrict__ add,
                                                             int32_t* __restrict__ degenerate,
                                                             long long* __restrict__ stats)
{
    int n_pairs = 0, n_cells = 0, n_pieces = 0, n_fp64 = 0;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    {
        double const px = pos[3 * i], py = pos[3 * i + 1], pz = pos[3 * i + 2];
        double q[3];
        for (int r = 0; r < 3; ++r)
            q[r] = f.r[3 * r] * px + f.r[3 * r + 1] * py + f.r[3 * r + 2] * pz;
        double const qscale = fmax(fmax(fabs(q[0]), fabs(q[1])), fabs(q[2]));
        float const qx = float(q[0]), qy = float(q[1]), qw = float(q[2]);
        int sum = 0, deg = 0;
        for (int64_t k = 0; k < n_patches; ++k)
        {
            float4 const b0 = boxf[2 * k], b1 = boxf[2 * k + 1];
            // 2^-16 of the scale: the float values compared below err by less than 2^-18.5 of it
            float const m = 1.52587890625e-5f * (float(qscale) + b1.z);
            if (b0.x - qx > m || b0.y - qx < -m || b0.z - qy > m || b0.w - qy < -m || b1.y - qw < -m)
                continue;
            // the net relative to the query, read again (from L1) by every cell rather than held in registers
            const float* nk = netf + 48 * k;
            auto const c = [=](int j, int kk) { return __ldg(nk + 3 * j + kk) - (kk == 0 ? qx : (kk == 1 ? qy : qw)); };
            int unresolved = 0;
            ++n_pairs;
            int const s = patch_degree(c, m, unresolved, n_cells, n_pieces);
            if (unresolved == 0)
                sum += s;
            else
            {
                ++n_fp64;
                sum += patch_degree_fp64(net + 48 * k, q[0], q[1], q[2], qscale + double(b1.z), deg, n_cells,
                                         n_pieces);
            }
        }
        if (add)
            add[i] += double(sum);
        else
            counts[i] = sum;
        if (degenerate)
            degenerate[i] = deg;
    }
    if (stats)
    {
        long long v[4] = {n_pairs, n_cells, n_pieces, n_fp64};
#pragma unroll
        for (int r = 0; r < 4; ++r)
        {
            for (int o = 16; o > 0; o >>= 1)
                v[r] += __shfl_xor_sync(0xffffffffu, v[r], o);
            if ((threadIdx.x & 31) == 0 && v[r])
                atomicAdd(reinterpret_cast<unsigned long long*>(stats + r), static_cast<unsigned long long>(v[r]));
        }
    }
}
} // namespace
} // namespace agwn

// The device copy of the patches and the ray-frame data of the last direction used.
struct agwn_patches
{
    int device = 0;
    int64_t n = 0;
    double* ctrl = nullptr; // n x 48
    double* net = nullptr;  // n x 48, in the frame of `dir`
    float* netf = nullptr;  // the same in float
    float* boxf = nullptr;  // n x 8 (k_patch_frame)
    double dir[3] = {0, 0, 0};
    bool framed = false;
    std::mutex mutex;
};

using namespace agwn;

namespace
{
int patches_prepare(Context& ctx, agwn_patches& pt, const double* x0, Frame64* f)
{
    double const nn = x0[0] * x0[0] + x0[1] * x0[1] + x0[2] * x0[2];
    AGWN_CHECK_ARG(nn > 0 && std::isfinite(nn), "x0 must be finite and nonzero");
    *f = ray_frame(x0);
    if (pt.framed && pt.dir[0] == x0[0] && pt.dir[1] == x0[1] && pt.dir[2] == x0[2])
        return AGWN_OK;
    if (pt.n > 0)
    {
        AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
        k_patch_frame<<<std::max(1, int(std::min<int64_t>(div_up(pt.n, 128), 4 * int64_t(ctx.sm_count)))), 128, 0,
                        ctx.stream>>>(pt.ctrl, pt.n, *f, pt.net, pt.netf, pt.boxf);
        AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
    }
    for (int k = 0; k < 3; ++k)
        pt.dir[k] = x0[k];
    pt.framed = true;
    return AGWN_OK;
}

int patch_integer(agwn_context* ctx, agwn_patches* pt, const double* positions, int64_t n, int32_t* out_counts,
                  double* add_out, int32_t* out_degenerate, const double* x0)
{
    AGWN_CHECK_ARG(ctx && pt && x0, "null context/patches/x0");
    AGWN_CHECK_ARG(pt->device == ctx->device, "the patches live on device %d, the context on %d", pt->device,
                   ctx->device);
    AGWN_CHECK_ARG(n >= 0 && (n == 0 || (positions && (out_counts || add_out))), "bad arguments");
    clear_message();
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    if (n == 0)
        return AGWN_OK;
    std::lock_guard<std::mutex> lock(pt->mutex);
    Frame64 f;
    AGWN_TRY(patches_prepare(*ctx, *pt, x0, &f));
    const void* dpos = nullptr;
    void* dout = nullptr;
    bool host_out = false;
    AGWN_TRY(stage_in(*ctx, positions, sizeof(double) * 3 * n, S_QUERIES, &dpos));
    if (add_out)
    {
        // the fractional term is already in add_out: a host array is added to on the device and copied back
        if (is_device_pointer(add_out))
            dout = add_out;
        else
        {
            AGWN_TRY(ctx->scratch_reserve(S_OUT, sizeof(double) * n, &dout));
            AGWN_TRY_CUDA(cudaMemcpyAsync(dout, add_out, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
            host_out = true;
        }
    }
    else
        AGWN_TRY(stage_out(*ctx, out_counts, sizeof(int32_t) * n, S_COUNTS, &dout, &host_out));
    void* ddeg = nullptr;
    bool host_deg = false;
    if (out_degenerate)
        AGWN_TRY(stage_out(*ctx, out_degenerate, sizeof(int32_t) * n, S_MISC0, &ddeg, &host_deg));
    int const grid = std::max(1, int(std::min<int64_t>(div_up(n, kPatchBlock), 16 * int64_t(ctx->sm_count))));
    AGWN_TRY(ctx->launch_begin(AGWN_K_PARAMETRIC));
    k_patch_count<<<grid, kPatchBlock, 0, ctx->stream>>>(
        pt->net, pt->netf, reinterpret_cast<const float4*>(pt->boxf), pt->n, f, static_cast<const double*>(dpos), n,
        add_out ? nullptr : static_cast<int32_t*>(dout), add_out ? static_cast<double*>(dout) : nullptr,
        static_cast<int32_t*>(ddeg), ctx->timing ? ctx->d_counters + 8 : nullptr);
    AGWN_TRY(ctx->launch_end(AGWN_K_PARAMETRIC));
    if (host_out)
        AGWN_TRY_CUDA(cudaMemcpyAsync(add_out ? static_cast<void*>(add_out) : static_cast<void*>(out_counts), dout,
                                      add_out ? sizeof(double) * n : sizeof(int32_t) * n, cudaMemcpyDeviceToHost,
                                      ctx->stream));
    if (host_deg)
        AGWN_TRY_CUDA(cudaMemcpyAsync(out_degenerate, ddeg, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    return ctx->check_flags();
}
} // namespace

extern "C" int agwn_patches_create_f64(agwn_context* ctx, const double* control_points, int64_t n_patches,
                                       agwn_patches** out)
{
    AGWN_CHECK_ARG(ctx && out, "null context/out");
    AGWN_CHECK_ARG(n_patches >= 0 && (n_patches == 0 || control_points), "bad patches");
    AGWN_CHECK_ARG(n_patches < (int64_t(1) << 40), "too many patches");
    clear_message();
    *out = nullptr;
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    auto* pt = new agwn_patches;
    pt->device = ctx->device;
    pt->n = n_patches;
    if (n_patches > 0)
    {
        size_t const bytes = sizeof(double) * 48 * size_t(n_patches);
        cudaError_t e = cudaMalloc(&pt->ctrl, bytes);
        if (e == cudaSuccess)
            e = cudaMalloc(&pt->net, bytes);
        if (e == cudaSuccess)
            e = cudaMalloc(&pt->netf, sizeof(float) * 48 * size_t(n_patches));
        if (e == cudaSuccess)
            e = cudaMalloc(&pt->boxf, sizeof(float) * 8 * size_t(n_patches));
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(pt->ctrl, control_points, bytes, cudaMemcpyDefault, ctx->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess)
        {
            cudaGetLastError();
            cudaFree(pt->ctrl);
            cudaFree(pt->net);
            cudaFree(pt->netf);
            cudaFree(pt->boxf);
            delete pt;
            return fail(e == cudaErrorMemoryAllocation ? AGWN_ERR_NOMEM : AGWN_ERR_CUDA, "patch upload: %s",
                        cudaGetErrorString(e));
        }
    }
    *out = pt;
    return AGWN_OK;
}

extern "C" int agwn_patches_destroy(agwn_patches* patches)
{
    if (!patches)
        return AGWN_OK;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(patches->device);
    cudaFree(patches->ctrl);
    cudaFree(patches->net);
    cudaFree(patches->netf);
    cudaFree(patches->boxf);
    cudaSetDevice(prev);
    delete patches;
    return AGWN_OK;
}

extern "C" int agwn_param_batch_integer_bezier3x3_f64(agwn_context* ctx, agwn_patches* patches,
                                                      const double* positions, int64_t n, int32_t* out_counts,
                                                      const double* x0)
{
    AGWN_CHECK_ARG(n == 0 || out_counts, "null out_counts");
    return patch_integer(ctx, patches, positions, n, out_counts, nullptr, nullptr, x0);
}

extern "C" int agwn_param_batch_integer_degenerate_bezier3x3_f64(agwn_context* ctx, agwn_patches* patches,
                                                                 const double* positions, int64_t n,
                                                                 int32_t* out_counts, int32_t* out_degenerate,
                                                                 const double* x0)
{
    AGWN_CHECK_ARG(n == 0 || (out_counts && out_degenerate), "null out_counts/out_degenerate");
    return patch_integer(ctx, patches, positions, n, out_counts, nullptr, out_degenerate, x0);
}

extern "C" int agwn_param_add_integer_bezier3x3_f64(agwn_context* ctx, agwn_patches* patches,
                                                    const double* positions, int64_t n, double* out_wnrs,
                                                    const double* x0)
{
    AGWN_CHECK_ARG(n == 0 || out_wnrs, "null out_wnrs");
    return patch_integer(ctx, patches, positions, n, nullptr, out_wnrs, nullptr, x0);
}
