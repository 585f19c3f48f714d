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
// Each pair runs in float with a margin of 2^-17 of the coordinates' scale; a decision that float cannot make (a
// boundary image or the surface within that margin of the ray) is taken in FP64, with a margin of 2^-42, for that
// cell alone: its winding, or the walk of its subtree.  Since every decision holds for the exact patch, the cells'
// contributions add up to the count whichever arithmetic decided them.  What FP64 cannot decide either is
// degenerate (the ray on a cell boundary's image within 2^-42 of the scale, or the query that close to the
// surface): it is decided by a fixed rule and counted.

#include "agwn_internal.cuh"
#include "hier.cuh"

#include <cmath>
#include <mutex>

namespace agwn
{
namespace
{
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

// After cell (level, iu, iv) is done: the next cell of the walk over the subtree of level root, or false at its end.
template <class I>
__device__ __forceinline__ bool walk_next(int& level, I& iu, I& iv, int root)
{
    while (level > root && (iu & 1) && (iv & 1))
    {
        iu >>= 1;
        iv >>= 1;
        --level;
    }
    if (level == root)
        return false;
    if (iu & 1)
    {
        iu -= 1;
        iv += 1;
    }
    else
        iu += 1;
    return true;
}

// One step of the walk over a patch's parameter cells, depth first without a stack: cell (level, iu, iv), children
// 2 iu + (0|1), 2 iv + (0|1) in the order (0,0), (1,0), (0,1), (1,1), the walk covering the subtree of one cell of
// level root.  The step tests the cell (c(j, k): the patch's net relative to the query in the ray frame, k = x, y
// across the ray and w along it; m the margin), adds its boundary's winding number to sum when it lies in front,
// and moves to the next cell.  Returns false when the walk is over: every cell done, or (float) a decision the
// margin did not allow, counted in unresolved.  pieces counts the boundary-cubic pieces tested.
template <class R, class Net, class I>
__device__ __forceinline__ bool walk_cell(Net const& c, R m, int& level, I& iu, I& iv, int& sum, int& unresolved,
                                          int& pieces, int root = 0)
{
    using A = PatchArith<R>;
    R x[16], y[16], lo, hi;
    cell_net(c, 0, level, iu, iv, x);
    range16(x, lo, hi);
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
                {
                    ++level;
                    iu *= 2;
                    iv *= 2;
                    return true;
                }
                ++unresolved;
                if (A::kExact && lo + hi >= R(0))
                    sum += net_winding(x, y, m, unresolved, pieces);
            }
            if (!A::kExact && unresolved)
                return false;
        }
    }
    return walk_next(level, iu, iv, root);
}

// Signed crossings in front of the query with one patch: the whole walk.  unresolved counts the decisions left to
// the fixed rule (FP64) or that void the result (float); cells and pieces count the work.
template <class R, class Net>
__device__ int patch_degree(Net const& c, R m, int& unresolved, int& cells, int& pieces, int root = 0,
                            typename PatchArith<R>::Index root_iu = 0, typename PatchArith<R>::Index root_iv = 0)
{
    int sum = 0, level = root;
    typename PatchArith<R>::Index iu = root_iu, iv = root_iv;
    bool more = true;
    while (more)
    {
        ++cells;
        more = walk_cell(c, m, level, iu, iv, sum, unresolved, pieces, root);
    }
    return sum;
}

// The FP64 walk of the subtree of one cell (level, iu, iv) of a pair (a cell whose depth float could not resolve):
// the patch's FP64 net (ray frame) relative to the query, margin 2^-42 of `scale`.
__device__ __noinline__ int patch_subtree_fp64(const double* __restrict__ net, double qx, double qy, double qw,
                                               double scale, int level, uint64_t iu, uint64_t iv, int& degenerate,
                                               int& cells, int& pieces)
{
    auto const c = [=](int j, int k) { return net[3 * j + k] - (k == 0 ? qx : (k == 1 ? qy : qw)); };
    return patch_degree(c, scale * 0x1p-42, degenerate, cells, pieces, level, iu, iv);
}

// The FP64 winding number of one cell's boundary (a cell in front whose float winding the margin did not allow).
__device__ __noinline__ int patch_winding_fp64(const double* __restrict__ net, double qx, double qy, double qw,
                                               double scale, int level, uint64_t iu, uint64_t iv, int& degenerate,
                                               int& pieces)
{
    auto const c = [=](int j, int k) { return net[3 * j + k] - (k == 0 ? qx : (k == 1 ? qy : qw)); };
    double x[16], y[16];
    cell_net(c, 0, level, iu, iv, x);
    cell_net(c, 1, level, iu, iv, y);
    return net_winding(x, y, scale * 0x1p-42, degenerate, pieces);
}

// The float winding number of one cell's boundary, c its patch's float net relative to the query.
template <class Net>
__device__ __noinline__ int patch_winding_f(Net const c, float m, int level, uint32_t iu, uint32_t iv,
                                            int& unresolved, int& pieces)
{
    float x[16], y[16];
    cell_net(c, 0, level, iu, iv, x);
    cell_net(c, 1, level, iu, iv, y);
    return net_winding(x, y, m, unresolved, pieces);
}

// One coordinate (phase 0: x, 1: y, 2: w) of the float walk's current cell, c(j, 0) giving that coordinate of the
// patch's net relative to the query.  x and y drop the cell when their box misses the origin (the walk moves to the
// next cell) and otherwise pass it to the next phase.  w decides: a cell in front is left to a winding job (event 1),
// a cell whose depth float cannot resolve to an FP64 job over its subtree (event 2), both for the cell as it was on
// entry, and a cell whose depth changes sign is split.  Every call costs the same, so lanes in different phases stay
// together.
template <class Net>
__device__ __forceinline__ bool walk_phase(Net const& c, float m, int& level, uint32_t& iu, uint32_t& iv, int& phase,
                                           int& event)
{
    using A = PatchArith<float>;
    event = 0;
    float x[16], lo, hi;
    cell_net(c, 0, level, iu, iv, x);
    range16(x, lo, hi);
    if (phase < 2)
    {
        if (!(lo > m || hi < -m))
        {
            ++phase;
            return true;
        }
    }
    else if (lo >= m)
        event = 1;
    else if (hi >= -m)
    {
        if (level < A::kMaxCellLevel && hi - lo >= 4.f * m)
        {
            ++level;
            iu *= 2;
            iv *= 2;
            phase = 0;
            return true;
        }
        event = 2;
    }
    phase = 0;
    return walk_next(level, iu, iv, 0);
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

// Work is queued per warp, so that the lanes stay busy however unevenly it falls.  A warp owns 32 queries (one per
// lane) and tests them against the patches of the shared-memory tile one patch at a time; the (query, patch) pairs
// that pass the box test go to a ring of pairs.  Every lane that has no pair takes the next one, and each turn of
// the loop runs one coordinate of the current cell of every lane's float walk (walk_phase).  The two kinds of work whose length varies most leave the walk
// as jobs of their own, evaluated 32 at a time, one per lane, when 32 have gathered: the winding number of a cell
// in front (its boundary's control points blossomed again from the patch), and the FP64 walk of the subtree of a
// cell whose depth float could not resolve.  A winding that float cannot decide is taken in FP64 for that cell.
// Every decision, float or FP64, holds for the exact patch, so the cells' contributions add up to the count
// whichever arithmetic decided them.  The tile holds each patch's float net at a stride of 49 floats (lanes on
// different patches then fall in different banks) and its box.
constexpr int kPatchWarps = 4;
constexpr int kPatchQueue = 64;   // ring size: below 32 entries are topped up by at most 32, and drained to below 32
constexpr int kNetStride = 49;    // floats per patch net in shared memory
constexpr int kPatchTileMax = 512; // patches per shared-memory tile

struct PatchWarp
{
    double qd[32][3];              // the queries in the ray frame (FP64)
    float qf[32][3];               // ... in float
    float qscale[32];              // largest |coordinate| of each
    int sum[32];
    int deg[32];
    uint32_t queue[kPatchQueue];   // pairs: (patch in tile << 5) | lane
    uint32_t jcell[2][kPatchQueue]; // jobs, [0] windings, [1] FP64 subtrees: lane | patch << 5 | level << 14 ...
    uint32_t juv[2][kPatchQueue];   // ... and iu | iv << 16
};

// Margin of the float walk for query src and patch p.  With S the coordinates' scale and u = 2^-24, a float net value
// relative to the query errs by at most 2 u S (the net's and the query's rounding, the difference), each level of
// lerps adds 3 u S, so a cell's net errs by 20 u S (6 levels) and a boundary piece's control points by 29 u S (3
// more); the piece, its chord and the straight joins between their ends then keep within 41 u S of the piece's box.
// The margin m = 2^-17 S = 128 u S is three times that.
__device__ __forceinline__ float patch_margin(PatchWarp const& w, const float* s_box, int src, int p)
{
    return 7.62939453125e-6f * (w.qscale[src] + s_box[8 * p + 6]);
}

// The jobs j[head .. head + count) of kind 0 (windings) or 1 (FP64 subtrees), count <= 32, lane k taking entry k.
__device__ __forceinline__ void patch_jobs(PatchWarp& w, int kind, const double* __restrict__ net64,
                                           const float* s_net, const float* s_box, int64_t tile_base, uint32_t head,
                                           uint32_t count, int lane, int& n_cells, int& n_pieces, int& n_fp64)
{
    if (uint32_t(lane) < count)
    {
        uint32_t const e = w.jcell[kind][(head + lane) & (kPatchQueue - 1)];
        uint32_t const uv = w.juv[kind][(head + lane) & (kPatchQueue - 1)];
        int const src = int(e & 31u), p = int((e >> 5) & 511u), level = int(e >> 14);
        uint32_t const iu = uv & 0xffffu, iv = uv >> 16;
        double const scale = double(w.qscale[src]) + double(s_box[8 * p + 6]);
        const double* nk64 = net64 + 48 * (tile_base + p);
        int s = 0, deg = 0;
        if (kind == 0)
        {
            const float* nk = s_net + p * kNetStride;
            float const qx = w.qf[src][0], qy = w.qf[src][1], qw = w.qf[src][2];
            auto const c = [=](int j, int kk) { return nk[3 * j + kk] - (kk == 0 ? qx : (kk == 1 ? qy : qw)); };
            int unresolved = 0;
            s = patch_winding_f(c, patch_margin(w, s_box, src, p), level, iu, iv, unresolved, n_pieces);
            if (unresolved)
            {
                ++n_fp64;
                s = patch_winding_fp64(nk64, w.qd[src][0], w.qd[src][1], w.qd[src][2], scale, level, iu, iv, deg,
                                       n_pieces);
            }
        }
        else
        {
            ++n_fp64;
            s = patch_subtree_fp64(nk64, w.qd[src][0], w.qd[src][1], w.qd[src][2], scale, level, iu, iv, deg, n_cells,
                                   n_pieces);
        }
        if (s)
            atomicAdd(&w.sum[src], s);
        if (deg)
            atomicAdd(&w.deg[src], deg);
    }
    __syncwarp();
}

// counts / add: the crossing count is written to counts (int) or added to add (the fractional term already there);
// degenerate (nullable): per query, the decisions left to the fixed rule; stats (nullable): adds pairs past the box
// test, cells, pieces and FP64 jobs to stats[0..3].
__global__ void __launch_bounds__(32 * kPatchWarps) k_patch_count(
    const double* __restrict__ net64, const float* __restrict__ netf, const float* __restrict__ boxf,
    int64_t n_patches, int tile, Frame64 f, const double* __restrict__ pos, int64_t n, int32_t* __restrict__ counts,
    double* __restrict__ add, int32_t* __restrict__ degenerate, long long* __restrict__ stats)
{
    extern __shared__ __align__(16) float s_tile[]; // tile x kNetStride nets, then tile x 8 box values
    __shared__ PatchWarp s_warp[kPatchWarps];
    float* const s_net = s_tile;
    float* const s_box = s_tile + tile * kNetStride; // tile is a multiple of 4: 16-byte aligned
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned const lt = (1u << lane) - 1u;
    PatchWarp& w = s_warp[warp];
    int const n_ptiles = int((n_patches + tile - 1) / tile);
    int n_pairs = 0, n_cells = 0, n_pieces = 0, n_fp64 = 0;

    auto load_tile = [&](int pt)
    {
        int64_t const base = int64_t(pt) * tile;
        int const tn = int(n_patches - base < tile ? n_patches - base : int64_t(tile));
        for (int j = threadIdx.x; j < tn * 48; j += blockDim.x)
            s_net[(j / 48) * kNetStride + j % 48] = netf[48 * base + j];
        for (int j = threadIdx.x; j < tn * 8; j += blockDim.x)
            s_box[j] = boxf[8 * base + j];
    };
    if (n_ptiles == 1)
    {
        load_tile(0);
        __syncthreads();
    }

    int64_t const per_block = 32 * kPatchWarps;
    for (int64_t bt = blockIdx.x; bt * per_block < n; bt += gridDim.x)
    {
        int64_t const i = bt * per_block + 32 * warp + lane;
        bool const valid = i < n;
        double q[3] = {0.0, 0.0, 0.0};
        if (valid)
        {
            double const px = pos[3 * i], py = pos[3 * i + 1], pz = pos[3 * i + 2];
            for (int r = 0; r < 3; ++r)
                q[r] = f.r[3 * r] * px + f.r[3 * r + 1] * py + f.r[3 * r + 2] * pz;
        }
        float const my_x = float(q[0]), my_y = float(q[1]), my_w = float(q[2]);
        float const my_scale = float(fmax(fmax(fabs(q[0]), fabs(q[1])), fabs(q[2])));
        for (int r = 0; r < 3; ++r)
            w.qd[lane][r] = q[r];
        w.qf[lane][0] = my_x;
        w.qf[lane][1] = my_y;
        w.qf[lane][2] = my_w;
        w.qscale[lane] = my_scale;
        w.sum[lane] = 0;
        w.deg[lane] = 0;
        __syncwarp();

        for (int pt = 0; pt < n_ptiles; ++pt)
        {
            if (n_ptiles > 1)
            {
                __syncthreads();
                load_tile(pt);
                __syncthreads();
            }
            int64_t const tile_base = int64_t(pt) * tile;
            int const tn = int(n_patches - tile_base < tile ? n_patches - tile_base : int64_t(tile));
            uint32_t head = 0, tail = 0, jhead[2] = {0, 0}, jtail[2] = {0, 0};
            int kn = 0;
            // this lane's pair: its queue entry (or -1), its query and margin, and the walk's state
            int cur = -1;
            float cx = 0.f, cy = 0.f, cw = 0.f, cm = 0.f;
            int level = 0, phase = 0;
            uint32_t iu = 0, iv = 0;
            for (;;)
            {
                // top the queue up: the next patches' box tests for the warp's 32 queries
                while (tail - head < 32 && kn < tn)
                {
                    float4 const b0 = *reinterpret_cast<const float4*>(s_box + 8 * kn);
                    float4 const b1 = *reinterpret_cast<const float4*>(s_box + 8 * kn + 4);
                    float const m = 7.62939453125e-6f * (my_scale + b1.z);
                    bool const pass = valid && !(b0.x - my_x > m || b0.y - my_x < -m || b0.z - my_y > m ||
                                                 b0.w - my_y < -m || b1.y - my_w < -m);
                    unsigned const bal = __ballot_sync(0xffffffffu, pass);
                    if (pass)
                        w.queue[(tail + __popc(bal & lt)) & (kPatchQueue - 1)] = (uint32_t(kn) << 5) | uint32_t(lane);
                    tail += __popc(bal);
                    ++kn;
                }
                __syncwarp();
                // lanes without a pair take the next ones
                bool const idle = cur < 0;
                unsigned const ib = __ballot_sync(0xffffffffu, idle);
                uint32_t const rank = __popc(ib & lt);
                if (idle && head + rank < tail)
                {
                    cur = int(w.queue[(head + rank) & (kPatchQueue - 1)]);
                    int const src = cur & 31, p = cur >> 5;
                    cx = w.qf[src][0];
                    cy = w.qf[src][1];
                    cw = w.qf[src][2];
                    cm = patch_margin(w, s_box, src, p);
                    level = 0;
                    phase = 0;
                    iu = iv = 0;
                    ++n_pairs;
                }
                head += min(uint32_t(__popc(ib)), tail - head);
                if (__ballot_sync(0xffffffffu, cur >= 0) == 0)
                    break; // queue empty and every patch of the tile tested
                // one cell of every lane's walk
                int event = 0;
                int const e_level = level;
                uint32_t const e_iu = iu, e_iv = iv;
                bool finished = false;
                if (cur >= 0)
                {
                    // this phase's coordinate of the net relative to the query
                    const float* nk = s_net + (cur >> 5) * kNetStride + phase;
                    float const qk = phase == 0 ? cx : (phase == 1 ? cy : cw);
                    auto const c = [=](int j, int) { return nk[3 * j] - qk; };
                    n_cells += phase == 0;
                    finished = !walk_phase(c, cm, level, iu, iv, phase, event);
                }
                // the cell's job, if it left one
#pragma unroll
                for (int kind = 0; kind < 2; ++kind)
                {
                    bool const push = event == kind + 1;
                    unsigned const pb = __ballot_sync(0xffffffffu, push);
                    if (push)
                    {
                        uint32_t const slot = (jtail[kind] + __popc(pb & lt)) & (kPatchQueue - 1);
                        w.jcell[kind][slot] = uint32_t(cur & 31) | (uint32_t(cur >> 5) << 5) | (uint32_t(e_level) << 14);
                        w.juv[kind][slot] = e_iu | (e_iv << 16);
                    }
                    jtail[kind] += __popc(pb);
                }
                if (finished)
                    cur = -1;
                __syncwarp();
#pragma unroll
                for (int kind = 0; kind < 2; ++kind)
                    if (jtail[kind] - jhead[kind] >= 32)
                    {
                        patch_jobs(w, kind, net64, s_net, s_box, tile_base, jhead[kind], 32, lane, n_cells, n_pieces,
                                   n_fp64);
                        jhead[kind] += 32;
                    }
            }
#pragma unroll
            for (int kind = 0; kind < 2; ++kind)
                if (jtail[kind] != jhead[kind])
                    patch_jobs(w, kind, net64, s_net, s_box, tile_base, jhead[kind], jtail[kind] - jhead[kind], lane,
                               n_cells, n_pieces, n_fp64);
        }
        __syncwarp();
        if (valid)
        {
            int const sum = w.sum[lane];
            if (add)
                add[i] += double(sum);
            else
                counts[i] = sum;
            if (degenerate)
                degenerate[i] = w.deg[lane];
        }
        __syncwarp();
    }
    if (stats)
    {
        long long v[4] = {n_pairs, n_cells, n_pieces, n_fp64};
#pragma unroll
        for (int r = 0; r < 4; ++r)
        {
            for (int o = 16; o > 0; o >>= 1)
                v[r] += __shfl_xor_sync(0xffffffffu, v[r], o);
            if (lane == 0 && v[r])
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
    // one shared-memory tile of patches (a multiple of 4, so that the boxes after the nets stay 16-byte aligned),
    // and as many blocks as fit on the SMs at once
    int const tile = int(std::min<int64_t>(kPatchTileMax, std::max<int64_t>(4, div_up(pt->n, 4) * 4)));
    size_t const smem = sizeof(float) * size_t(tile) * (kNetStride + 8);
    int const block = 32 * kPatchWarps;
    AGWN_TRY_CUDA(cudaFuncSetAttribute(k_patch_count, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int per_sm = 0;
    AGWN_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_patch_count, block, smem));
    AGWN_CHECK_ARG(per_sm >= 1, "the patch kernel does not fit on an SM (smem %zu)", smem);
    int const grid = int(std::max<int64_t>(1, std::min<int64_t>(div_up(n, block), int64_t(per_sm) * ctx->sm_count)));
    AGWN_TRY(ctx->launch_begin(AGWN_K_PARAMETRIC));
    k_patch_count<<<grid, block, smem, ctx->stream>>>(
        pt->net, pt->netf, pt->boxf, pt->n, tile, f, static_cast<const double*>(dpos), n,
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
