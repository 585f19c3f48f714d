// Integer term of the parametric GWN: signed crossings of the ray p + lambda x0 (lambda >= 0) with bicubic Bezier
// patches, the Intersector that eval_gwnr_parametric_batch_integer / eval_gwnr_parametric_batch forward to
// (src/antipodal/gwn_parametric.hh:204-284).  The reference ships no parametric intersector (its README lists one
// as future work), so this one is specified by the mesh intersector's rule: every crossing in front of the query
// counts sign(N . x0), N = S_u x S_v the patch normal, whose orientation matches boundary curves that run
// counter-clockwise in (u, v) (the patch on their left).
//
// Method, per (query, patch), in FP64: in a frame whose third axis is the ray direction, the ray is the point
// (0, 0) of the plane and the patch's control points relative to the query are a 2D net with depths.  Crossings
// are the roots of the net's bicubic map in [0,1]^2 with depth >= 0.  The parameter square is subdivided (a stack
// of cells, each cell's net extracted from the patch's by blossoming) while the cell's net box, by the convex hull
// property, contains the origin and reaches depth 0; a cell of 1/32 x 1/32 runs Newton's iteration from its centre
// on the patch's own map and counts a converged root that lies in the cell (half-open, the square's far edges
// included) with depth >= 0, by the sign of the map's Jacobian (= sign(N . x0) in a right-handed frame).  A root is
// therefore found from the cell that owns it and counted once.  Rays tangent to a patch (a vanishing Jacobian)
// and roots exactly on a patch's edge are the degenerate cases, as edge hits are for the mesh rule.

#include "agwn_internal.cuh"
#include "hier.cuh"

#include <cmath>
#include <mutex>

namespace agwn
{
namespace
{
constexpr int kLeafLevel = 5;                 // Newton cells are 1/32 x 1/32 of the parameter square
constexpr int kCellStack = 3 * kLeafLevel + 1; // the depth-first stack never holds more
constexpr int kNewtonSteps = 16;
constexpr int kPatchBlock = 128;

// Bernstein basis of degree 3 and its derivative at x.
__device__ __forceinline__ void bernstein3(double x, double (&b)[4], double (&db)[4])
{
    double const y = 1.0 - x;
    b[0] = y * y * y;
    b[1] = 3.0 * x * y * y;
    b[2] = 3.0 * x * x * y;
    b[3] = x * x * x;
    db[0] = -3.0 * y * y;
    db[1] = 3.0 * y * y - 6.0 * x * y;
    db[2] = 6.0 * x * y - 3.0 * x * x;
    db[3] = 3.0 * x * x;
}

// The control values of a cubic restricted to [a, b]: the blossoms B(a,a,a), B(a,a,b), B(a,b,b), B(b,b,b).
__device__ __forceinline__ void cubic_restrict(double c0, double c1, double c2, double c3, double a, double b,
                                               double (&o)[4])
{
    auto const lerp = [](double p, double q, double x) { return p + x * (q - p); };
    double const a0 = lerp(c0, c1, a), a1 = lerp(c1, c2, a), a2 = lerp(c2, c3, a);
    double const b0 = lerp(c0, c1, b), b1 = lerp(c1, c2, b), b2 = lerp(c2, c3, b);
    double const aa0 = lerp(a0, a1, a), aa1 = lerp(a1, a2, a);
    double const ab0 = lerp(a0, a1, b), ab1 = lerp(a1, a2, b);
    double const bb0 = lerp(b0, b1, b), bb1 = lerp(b1, b2, b);
    o[0] = lerp(aa0, aa1, a);
    o[1] = lerp(aa0, aa1, b);
    o[2] = lerp(ab0, ab1, b);
    o[3] = lerp(bb0, bb1, b);
}

// The map of a net c ([16][3]: index 4 iv + iu, components x, y across the ray and w along it) at (u, v): the point
// s and its partial derivatives su, sv.
__device__ __forceinline__ void net_eval(const double (&c)[48], double u, double v, double (&s)[3], double (&su)[3],
                                         double (&sv)[3])
{
    double bu[4], dbu[4], bv[4], dbv[4];
    bernstein3(u, bu, dbu);
    bernstein3(v, bv, dbv);
    for (int k = 0; k < 3; ++k)
        s[k] = su[k] = sv[k] = 0.0;
#pragma unroll
    for (int iv = 0; iv < 4; ++iv)
#pragma unroll
        for (int iu = 0; iu < 4; ++iu)
#pragma unroll
            for (int k = 0; k < 3; ++k)
            {
                double const p = c[3 * (4 * iv + iu) + k];
                s[k] += bv[iv] * bu[iu] * p;
                su[k] += bv[iv] * dbu[iu] * p;
                sv[k] += dbv[iv] * bu[iu] * p;
            }
}

// Signed crossings of the ray (the origin of the x, y plane, depth w >= 0) with the patch whose net relative to the
// query is c.  m: the box margin, far above the rounding of the net (relative coordinates and blossoms).
__device__ int patch_crossings(const double (&c)[48], double m)
{
    int sum = 0;
    int stack[kCellStack];
    int sp = 0;
    stack[sp++] = 0; // (level << 16) | (iv << 8) | iu
    while (sp > 0)
    {
        int const cell = stack[--sp];
        int const level = cell >> 16, iv = (cell >> 8) & 0xff, iu = cell & 0xff;
        double const h = 1.0 / double(1 << level);
        double const u0 = iu * h, u1 = (iu + 1) * h, v0 = iv * h, v1 = (iv + 1) * h;
        // the cell's net: rows restricted in u, then columns in v; its box against the ray
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            double rows[4][4];
#pragma unroll
            for (int r = 0; r < 4; ++r)
                cubic_restrict(c[3 * (4 * r) + k], c[3 * (4 * r + 1) + k], c[3 * (4 * r + 2) + k],
                               c[3 * (4 * r + 3) + k], u0, u1, rows[r]);
#pragma unroll
            for (int q = 0; q < 4; ++q)
            {
                double col[4];
                cubic_restrict(rows[0][q], rows[1][q], rows[2][q], rows[3][q], v0, v1, col);
#pragma unroll
                for (int r = 0; r < 4; ++r)
                {
                    lo[k] = fmin(lo[k], col[r]);
                    hi[k] = fmax(hi[k], col[r]);
                }
            }
        }
        if (!(lo[0] <= m && hi[0] >= -m && lo[1] <= m && hi[1] >= -m && hi[2] >= -m))
            continue;
        if (level < kLeafLevel)
        {
#pragma unroll
            for (int d = 0; d < 4; ++d)
                stack[sp++] = ((level + 1) << 16) | ((2 * iv + (d >> 1)) << 8) | (2 * iu + (d & 1));
            continue;
        }
        // Newton's iteration on the patch's map from the cell's centre
        double u = 0.5 * (u0 + u1), v = 0.5 * (v0 + v1);
        double s[3], su[3], sv[3];
        bool ok = false;
        for (int it = 0; it < kNewtonSteps; ++it)
        {
            net_eval(c, u, v, s, su, sv);
            double const det = su[0] * sv[1] - sv[0] * su[1];
            if (!(det != 0.0) || !isfinite(det))
                break;
            double const du = -(sv[1] * s[0] - sv[0] * s[1]) / det;
            double const dv = -(su[0] * s[1] - su[1] * s[0]) / det;
            u += du;
            v += dv;
            if (!(fabs(u) < 4.0 && fabs(v) < 4.0))
                break;
            if (fabs(du) + fabs(dv) <= 1e-15)
            {
                ok = true;
                break;
            }
        }
        if (!ok)
            continue;
        net_eval(c, u, v, s, su, sv);
        bool const in_u = u >= u0 && (u < u1 || (u1 == 1.0 && u <= 1.0));
        bool const in_v = v >= v0 && (v < v1 || (v1 == 1.0 && v <= 1.0));
        if (!in_u || !in_v || !(fabs(s[0]) + fabs(s[1]) <= m) || !(s[2] >= 0.0))
            continue;
        double const det = su[0] * sv[1] - sv[0] * su[1];
        sum += det > 0.0 ? 1 : (det < 0.0 ? -1 : 0);
    }
    return sum;
}

// The patches' control points in the ray frame (rows of f), and per patch its box across the ray, its largest depth
// and its largest |coordinate|: box[6 k] = xmin, xmax, ymin, ymax, wmax, scale.
__global__ void k_patch_frame(const double* __restrict__ ctrl, int64_t n_patches, Frame64 f, double* __restrict__ net,
                              double* __restrict__ box)
{
    for (int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; k < n_patches;
         k += int64_t(gridDim.x) * blockDim.x)
    {
        double b[6] = {INFINITY, -INFINITY, INFINITY, -INFINITY, -INFINITY, 0.0};
        for (int j = 0; j < 16; ++j)
        {
            const double* p = ctrl + 48 * k + 3 * j;
            for (int r = 0; r < 3; ++r)
            {
                double const x = f.r[3 * r] * p[0] + f.r[3 * r + 1] * p[1] + f.r[3 * r + 2] * p[2];
                net[48 * k + 3 * j + r] = x;
                b[5] = fmax(b[5], fabs(x));
                if (r < 2)
                {
                    b[2 * r] = fmin(b[2 * r], x);
                    b[2 * r + 1] = fmax(b[2 * r + 1], x);
                }
                else
                    b[4] = fmax(b[4], x);
            }
        }
        for (int r = 0; r < 6; ++r)
            box[6 * k + r] = b[r];
    }
}

// One query per thread: every patch whose box the ray meets (with the margin) is subdivided.  counts and add: the
// crossing count is written to counts (int) or added to add (the fractional term already there).
__global__ void __launch_bounds__(kPatchBlock) k_patch_count(const double* __restrict__ net,
                                                             const double* __restrict__ box, int64_t n_patches,
                                                             Frame64 f, const double* __restrict__ pos, int64_t n,
                                                             int32_t* __restrict__ counts, double* __restrict__ add)
{
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    {
        double const px = pos[3 * i], py = pos[3 * i + 1], pz = pos[3 * i + 2];
        double q[3];
        for (int r = 0; r < 3; ++r)
            q[r] = f.r[3 * r] * px + f.r[3 * r + 1] * py + f.r[3 * r + 2] * pz;
        double const qscale = fmax(fmax(fabs(q[0]), fabs(q[1])), fabs(q[2]));
        int sum = 0;
        for (int64_t k = 0; k < n_patches; ++k)
        {
            const double* b = box + 6 * k;
            double const m = 1e-9 * (qscale + b[5]);
            if (!(b[0] - m <= q[0] && b[1] + m >= q[0] && b[2] - m <= q[1] && b[3] + m >= q[1] && b[4] + m >= q[2]))
                continue;
            double c[48];
#pragma unroll
            for (int j = 0; j < 48; ++j)
                c[j] = net[48 * k + j] - q[j % 3];
            sum += patch_crossings(c, m);
        }
        if (add)
            add[i] += double(sum);
        else
            counts[i] = sum;
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
    double* box = nullptr;  // n x 6
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
                        ctx.stream>>>(pt.ctrl, pt.n, *f, pt.net, pt.box);
        AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
    }
    for (int k = 0; k < 3; ++k)
        pt.dir[k] = x0[k];
    pt.framed = true;
    return AGWN_OK;
}

int patch_integer(agwn_context* ctx, agwn_patches* pt, const double* positions, int64_t n, int32_t* out_counts,
                  double* add_out, const double* x0)
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
    int const grid = std::max(1, int(std::min<int64_t>(div_up(n, kPatchBlock), 16 * int64_t(ctx->sm_count))));
    AGWN_TRY(ctx->launch_begin(AGWN_K_PARAMETRIC));
    k_patch_count<<<grid, kPatchBlock, 0, ctx->stream>>>(pt->net, pt->box, pt->n, f, static_cast<const double*>(dpos),
                                                        n, add_out ? nullptr : static_cast<int32_t*>(dout),
                                                        add_out ? static_cast<double*>(dout) : nullptr);
    AGWN_TRY(ctx->launch_end(AGWN_K_PARAMETRIC));
    if (host_out)
        AGWN_TRY_CUDA(cudaMemcpyAsync(add_out ? static_cast<void*>(add_out) : static_cast<void*>(out_counts), dout,
                                      add_out ? sizeof(double) * n : sizeof(int32_t) * n, cudaMemcpyDeviceToHost,
                                      ctx->stream));
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
            e = cudaMalloc(&pt->box, sizeof(double) * 6 * size_t(n_patches));
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(pt->ctrl, control_points, bytes, cudaMemcpyDefault, ctx->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess)
        {
            cudaGetLastError();
            cudaFree(pt->ctrl);
            cudaFree(pt->net);
            cudaFree(pt->box);
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
    cudaFree(patches->box);
    cudaSetDevice(prev);
    delete patches;
    return AGWN_OK;
}

extern "C" int agwn_param_batch_integer_bezier3x3_f64(agwn_context* ctx, agwn_patches* patches,
                                                      const double* positions, int64_t n, int32_t* out_counts,
                                                      const double* x0)
{
    AGWN_CHECK_ARG(n == 0 || out_counts, "null out_counts");
    return patch_integer(ctx, patches, positions, n, out_counts, nullptr, x0);
}

extern "C" int agwn_param_add_integer_bezier3x3_f64(agwn_context* ctx, agwn_patches* patches,
                                                    const double* positions, int64_t n, double* out_wnrs,
                                                    const double* x0)
{
    AGWN_CHECK_ARG(n == 0 || out_wnrs, "null out_wnrs");
    return patch_integer(ctx, patches, positions, n, nullptr, out_wnrs, x0);
}
