// Parametric fractional GWN over cubic Bezier boundary curves with adaptive G7-K15 quadrature:
// eval_gwnr_parametric_batch_fractional (src/antipodal/gwn_parametric.hh:168-186) with IntegratorGK15
// (src/antipodal/math/integrate_gk15.hh:63-290) and the integrand of gwn_parametric.hh:73-103.
//
// One thread per query walks the curves in order (curves staged in shared memory by cp.async.bulk) and
// integrates each with an explicit stack instead of recursion.  A panel is (depth, index): its end points are the
// dyadic numbers index * 2^-depth and its local tolerance tol * 2^-depth, exactly what the reference's halving
// computes, so a panel fits in 32 bits.  A second stack of values replays the reference's `left + right`
// summation order (post-order), and the integrand and the G7/K15 sums are written unfused, so the result equals
// the CPU reference bit for bit.
//
// Proposal hook: a per-(query, curve) start depth s (from the learned proposal; 0 for the plain method).  Panels
// above depth s are split without being evaluated; every panel at depth >= s is evaluated and accepted or split by
// the reference's own rule.  When s does not exceed the shallowest leaf the plain method would accept, the two
// produce the same leaves and the same value; a larger s only refines further.

#include "agwn_internal.cuh"
#include "df32.cuh"
#include "mlp.cuh"
#include "tma.cuh"

#include <cmath>

namespace agwn
{
namespace
{
constexpr int kParamMaxDepth = 24; // deepest panel the integrator can reach (2^24 panels per curve)
constexpr int kParamBlock = 128;
constexpr int kParamTileMax = 1024; // curves staged per tile (96 KB of shared memory)
// The double-float form stages 384 curves (36 KB, room for the per-panel network's weights beside them), so that
// six blocks reside per SM, the number its 80 registers allow.  Measured on 256 bicubic patches at tol 1e-10:
// 40K queries, 768 was 10% faster than 1024 and flat down to 128; 250K queries (one work item per query block),
// 384 is 1.7% faster than 768 (three blocks per SM) and 256 1.4%.
constexpr int kParamTileDF = 384;

struct alignas(16) Bez
{
    double c[12];
};

// G7-K15 abscissae and weights: the published Gauss-Kronrod constants at the precision the reference carries
// (integrate_gk15.hh:13-36); identical doubles make the sums identical.
__constant__ double kGkX[8] = {0.0,
                               0.9914553711208126,
                               0.9491079123427585,
                               0.8648644233597691,
                               0.7415311855993945,
                               0.5860872354676911,
                               0.4058451513773972,
                               0.2077849550078985};
__constant__ double kGkWk[8] = {0.2094821410847278, 0.0229353220105292, 0.0630920926299786, 0.1047900103222502,
                                0.1406532597155259, 0.1690047266392679, 0.1903505780647854, 0.2044329400752989};
constexpr double kGkWgCenter = 0.4179591836734694;
constexpr double kGkWg2 = 0.1294849661688697;
constexpr double kGkWg4 = 0.2797053914892767;
constexpr double kGkWg6 = 0.3818300505051189;

struct dual
{
    rd v, d;
};
__device__ __forceinline__ dual dmul(dual a, dual b)
{
    return {a.v * b.v, a.d * b.v + a.v * b.d};
}
__device__ __forceinline__ dual smul(rd s, dual b)
{
    return {s * b.v, s * b.d};
}

// w(t) - d_eta(t) for the cubic Bezier curve c at parameter t, with the dual-number evaluation of the curve
// (Bernstein basis, summed c0*b0 + c1*b1 + c2*b2 + c3*b3) and normalize_fd (src/antipodal/math/fwd_diff.hh:497-532).
__device__ __forceinline__ double integrand(const double* c, ev3<rd> p, ev3<rd> x0, double tt)
{
    dual const t{rd(tt), rd(1.0)};
    dual const u{rd(1.0) - rd(tt), rd(-1.0)};
    dual const b0 = dmul(dmul(u, u), u);
    dual const b1 = dmul(dmul(smul(rd(3.0), u), u), t);
    dual const b2 = dmul(dmul(smul(rd(3.0), u), t), t);
    dual const b3 = dmul(dmul(t, t), t);
    rd phi[3], dphi[3];
    for (int k = 0; k < 3; ++k)
    {
        phi[k] = rd(c[k]) * b0.v + rd(c[3 + k]) * b1.v + rd(c[6 + k]) * b2.v + rd(c[9 + k]) * b3.v;
        dphi[k] = rd(c[k]) * b0.d + rd(c[3 + k]) * b1.d + rd(c[6 + k]) * b2.d + rd(c[9 + k]) * b3.d;
    }
    ev3<rd> const r{phi[0] - p.x, phi[1] - p.y, phi[2] - p.z};
    ev3<rd> const dr{dphi[0], dphi[1], dphi[2]};
    rd const q = r.x * r.x + r.y * r.y + r.z * r.z;
    rd const q1 = rd(2.0) * (r.x * dr.x + r.y * dr.y + r.z * dr.z);
    rd const s = ex_sqrt(q);
    rd const inv_s = rd(1.0) / s;
    rd const s1 = q1 * (rd(0.5) * inv_s);
    ev3<rd> G, Gp;
    G.x = r.x * inv_s;
    G.y = r.y * inv_s;
    G.z = r.z * inv_s;
    Gp.x = (dr.x - G.x * s1) * inv_s;
    Gp.y = (dr.y - G.y * s1) * inv_s;
    Gp.z = (dr.z - G.z * s1) * inv_s;
    ev3<rd> const x1{-x0.x, -x0.y, -x0.z};
    rd const a = edot(x0, G);
    rd const ap = edot(x0, Gp);
    ev3<rd> const X = x0 - ev3<rd>{G.x * a, G.y * a, G.z * a};
    ev3<rd> const Xp = ev3<rd>{G.x * -ap, G.y * -ap, G.z * -ap} - ev3<rd>{Gp.x * a, Gp.y * a, Gp.z * a};
    rd const d_eta = edot(G, ecross(X, Xp)) / edot(X, X);
    rd const b = edot(x1, G);
    rd const bp = edot(x1, Gp);
    ev3<rd> const v = G - ev3<rd>{x1.x * b, x1.y * b, x1.z * b};
    ev3<rd> const vp = Gp - ev3<rd>{x1.x * bp, x1.y * bp, x1.z * bp};
    rd const w = edot(x1, ecross(v, vp)) / edot(v, v);
    return (w - d_eta).v;
}

// One GK15 panel (depth, j) = [j 2^-depth, (j+1) 2^-depth] of curve c: the Kronrod and Gauss estimates in the
// reference's node and summation order (integrate_gk15.hh:155-217).  Returns Ik; *err = |Ik - Ig|.
__device__ __forceinline__ double gk15_panel(const double* c, ev3<rd> p, ev3<rd> x0, int depth, uint32_t j,
                                             double* err)
{
    double const scale = ldexp(1.0, -depth);
    double const aa = double(j) * scale, bb = double(j + 1) * scale; // exact: j < 2^24
    rd const cc = (rd(aa) + rd(bb)) * rd(0.5);
    rd const h = (rd(bb) - rd(aa)) * rd(0.5);
    double const f0 = integrand(c, p, x0, cc.v);
    double fm[8], fp[8];
#pragma unroll 1
    for (int k = 1; k <= 7; ++k)
    {
        rd const dx = h * rd(kGkX[k]);
        fm[k] = integrand(c, p, x0, (cc - dx).v);
        fp[k] = integrand(c, p, x0, (cc + dx).v);
    }
    rd ig = rd(kGkWgCenter) * rd(f0);
    rd ik = rd(kGkWk[0]) * rd(f0);
    ik = ik + rd(kGkWk[1]) * (rd(fm[1]) + rd(fp[1]));
    {
        rd const s2 = rd(fm[2]) + rd(fp[2]);
        ik = ik + rd(kGkWk[2]) * s2;
        ig = ig + rd(kGkWg2) * s2;
    }
    ik = ik + rd(kGkWk[3]) * (rd(fm[3]) + rd(fp[3]));
    {
        rd const s4 = rd(fm[4]) + rd(fp[4]);
        ik = ik + rd(kGkWk[4]) * s4;
        ig = ig + rd(kGkWg4) * s4;
    }
    ik = ik + rd(kGkWk[5]) * (rd(fm[5]) + rd(fp[5]));
    {
        rd const s6 = rd(fm[6]) + rd(fp[6]);
        ik = ik + rd(kGkWk[6]) * s6;
        ig = ig + rd(kGkWg6) * s6;
    }
    ik = ik + rd(kGkWk[7]) * (rd(fm[7]) + rd(fp[7]));
    ig = ig * h;
    ik = ik * h;
    *err = fabs((ik - ig).v);
    return ik.v;
}

// ---- double-float form ----------------------------------------------------------------------------------------
// The same integrand and panel rule in double-float arithmetic (df32.cuh, ~44 significant bits on the FP32 pipe):
// the curve relative to the query in power form about t = 1/2 (power_about_half) and w - d_eta in the closed form
// below -- the same quantities in fewer operations.  Not bit-identical to the reference (the value differs in the
// last ~1e-13 relative, and a panel whose |Ik - Ig| sits at the tolerance can be decided the other way); the tree
// rule, the tolerances and the summation order are the plain integrator's.
struct alignas(16) CurveDF
{
    df c[12];
};

constexpr float hi_of(double d)
{
    return float(d);
}
constexpr float lo_of(double d)
{
    return float(d - double(float(d)));
}
#define AGWN_DF(d) {hi_of(d), lo_of(d)}
__constant__ df kGkXdf[8] = {AGWN_DF(0.0),
                             AGWN_DF(0.9914553711208126),
                             AGWN_DF(0.9491079123427585),
                             AGWN_DF(0.8648644233597691),
                             AGWN_DF(0.7415311855993945),
                             AGWN_DF(0.5860872354676911),
                             AGWN_DF(0.4058451513773972),
                             AGWN_DF(0.2077849550078985)};
__constant__ df kGkWkdf[8] = {AGWN_DF(0.2094821410847278), AGWN_DF(0.0229353220105292), AGWN_DF(0.0630920926299786),
                              AGWN_DF(0.1047900103222502), AGWN_DF(0.1406532597155259), AGWN_DF(0.1690047266392679),
                              AGWN_DF(0.1903505780647854), AGWN_DF(0.2044329400752989)};
__constant__ df kGkWgdf[4] = {AGWN_DF(0.4179591836734694), AGWN_DF(0.1294849661688697), AGWN_DF(0.2797053914892767),
                              AGWN_DF(0.3818300505051189)};
#undef AGWN_DF

__device__ __forceinline__ df df_mulf(df a, float f)
{
    df const p = two_prod(a.hi, f);
    return fast_two_sum(p.hi, __fmaf_rn(a.lo, f, p.lo));
}

// w(t) - d_eta(t) with cp = the curve's control points minus the query, in closed form.  The plain kernel evaluates
// the reference's expression (integrand, gwn_parametric.hh:73-103): with G = r / |r|, G' its derivative, a = x0.G,
// X = x0 - G a, X' = -(G (x0.G') + G' a), v = G - x0 a, v' = G' - x0 (x0.G'), d_eta = G.(X x X') / |X|^2 and
// w = -x0.(v x v') / |v|^2.  Expanding (G x G = 0, G.(G x G') = 0, |G| = 1): G.(X x X') = a c and
// x0.(v x v') = c with c = x0.(G x G'), |X|^2 = n - a^2 = |x0 x G|^2 (Lagrange's identity) and
// |v|^2 = 1 + (n - 2) a^2 with n = |x0|^2.  In terms of r itself (s = |r|, q = s^2, m = x0.r, G x G' = r x r' / q,
// so c = T / q with T = x0.(r x r') = r'.(x0 x r)):
//   w - d_eta = -T / (q + (n - 2) m^2) - m T / (s |x0 x r|^2),
// and for a unit x0 (n = 1 to double precision) -T / (s (s - m)), free of the two terms' cancellation near
// m = -s.  Near m = s (the curve crossing the ray of x0 from the query) s - m, formed by subtraction, would keep
// only the square of the angle's relative precision; there it is |x0 x r|^2 / (s + m), whose cross product keeps
// the angle's own.  For a unit x0: one square root and one quotient, against the expression's square root and three
// quotients.
// pc: the pair's curve minus its query as power coefficients about t = 1/2 (power_about_half), dl = t - 1/2.
__device__ __forceinline__ df integrand_df(const df (&pc)[12], df3 x0, df x0n, bool unit, df dl)
{
    // r = a0 + dl (a1 + dl (a2 + dl a3)) and r' = a1 + dl (2 a2 + 3 dl a3), per coordinate
    df r3[3], dr3[3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
        df const a3d = pc[9 + c] * dl;
        r3[c] = pc[c] + dl * (pc[3 + c] + dl * (pc[6 + c] + a3d));
        dr3[c] = pc[3 + c] + dl * (df_scale(pc[6 + c], 2.f) + df_mulf(a3d, 3.f));
    }
    df3 const r{r3[0], r3[1], r3[2]}, dr{dr3[0], dr3[1], dr3[2]};
    df const q = dot(r, r);
    df const s = df_sqrt(q);
    df3 const xr = cross(x0, r);
    df const T = dot(dr, xr), m = dot(x0, r);
    if (unit)
    {
        bool const behind = m.hi < 0.f;
        df const num = behind ? T : T * (s + m);
        df const den = s * (behind ? s - m : dot(xr, xr));
        return df_neg(num / den);
    }
    return df_neg(T / (q + (x0n - df_make(2.f)) * (m * m))) - (m * T) / (s * dot(xr, xr));
}

// Control points c0..c3 (minus the query) to power coefficients about t = 1/2, in place: with s03 = c0 + c3,
// s12 = c1 + c2, d30 = c3 - c0 and d21 = c2 - c1, r(1/2) = (s03 + 3 s12) / 8, r'(1/2) = 3/4 (d30 + d21),
// r''(1/2) / 2 = 3/2 (s03 - s12) and r''' / 6 = d30 - 3 d21.  Evaluated at |t - 1/2| <= 1/2 the power form rounds
// a little worse than the Bernstein form (in FP32 on bicubic patch boundaries, relative error of r: median 1.2x at
// random pairs with a lower maximum, median 1.7x and p99 2.1x for queries 1e-4 to 1e-2 from a curve near their
// closest point), and takes 12 double-float products, 3 products by a float and 15 sums per node against the
// Bernstein form's 31, 5 and 21.
__device__ __forceinline__ void power_about_half(df (&cp)[12])
{
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
        df const s03 = cp[c] + cp[9 + c], s12 = cp[3 + c] + cp[6 + c];
        df const d30 = cp[9 + c] - cp[c], d21 = cp[6 + c] - cp[3 + c];
        cp[c] = df_scale(s03 + df_mulf(s12, 3.f), 0.125f);
        cp[3 + c] = df_mulf(d30 + d21, 0.75f);
        cp[6 + c] = df_mulf(s03 - s12, 1.5f);
        cp[9 + c] = d30 - df_mulf(d21, 3.f);
    }
}

__device__ __forceinline__ double gk15_panel_df(const df (&pc)[12], df3 x0, df x0n, bool unit, int depth, uint32_t j,
                                                float* err)
{
    float const scale = ldexpf(1.f, -depth);
    float const h = 0.5f * scale;
    // the centre (j + 1/2) 2^-depth less 1/2, exact: j 2^-depth - 1/2 is a multiple of 2^-depth below 1 in magnitude
    df const cc = two_sum(__fmaf_rn(float(j), scale, -0.5f), h);
    df const f0 = integrand_df(pc, x0, x0n, unit, cc);
    // the Kronrod and Gauss sums accumulated node pair by node pair, in the order of the sums above (the same
    // values), so no node value stays live
    df ig = kGkWgdf[0] * f0;
    df ik = kGkWkdf[0] * f0;
#pragma unroll 1
    for (int k = 1; k <= 7; ++k)
    {
        df const dx = df_scale(kGkXdf[k], h);
        df const s = integrand_df(pc, x0, x0n, unit, cc - dx) + integrand_df(pc, x0, x0n, unit, cc + dx);
        ik = ik + kGkWkdf[k] * s;
        if ((k & 1) == 0)
            ig = ig + kGkWgdf[k >> 1] * s;
    }
    df const diff = df_scale(ik - ig, h);
    *err = fabsf(diff.hi + diff.lo);
    return df_to(df_scale(ik, h));
}

__global__ void k_curves_df(const double* __restrict__ curves, int64_t n_curves, CurveDF* __restrict__ out)
{
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < 12 * n_curves;
         i += int64_t(gridDim.x) * blockDim.x)
        out[i / 12].c[i % 12] = df_from(curves[i]);
}

// out[q] = (sum over curves of the curve integral) / (4 pi).
//
// The cost of one (query, curve) integral is heavy-tailed: a query whose line along x0 passes close to a curve
// needs a deep tree there.  So the work is shared out by pair, not by query.  A block owns up to kParamBlock
// queries and, for each shared-memory tile of curves, the pool of (query, curve) pairs of that tile; a lane that
// finishes its pair takes the next one from the pool (one shared-memory atomic per warp).  Each lane walks its
// pair's panel tree without a stack: after a split the next panel is the left child (depth + 1, 2j); after an
// accepted leaf the walk climbs while the finished node is a right child (j odd), combining left + right from
// `pending` (the finished left sibling's value per level), then moves to the right sibling (depth, j + 1).
// Panels above the pair's start depth are not evaluated: the walk descends to the leftmost descendant at the
// start depth.  A finished pair's integral goes to the block's slab of `pair_vals`; after the tile each thread
// adds its query's row in curve order.  Every sum is the reference's (post-order left + right within a curve,
// curves in order), so the result does not depend on how the pairs were shared out.
//
// start_depth: per (query, curve), row-major [n][n_curves], nullable = all 0.  stats (nullable): per (query,
// curve) packed as leaves | shallowest leaf depth << 16 | deepest leaf depth << 24.  nodes_total (nullable):
// panels evaluated per query.  pair_vals: gridDim.x * kParamBlock * tile doubles.
// Optional work of the integrator kernel.
//   panel_log: training data for the per-panel network, 2 words per evaluated panel below max_depth -- the pair's
//     index (query * n_curves + curve) and (depth << 25) | (j << 1) | accepted; entries past log_cap are counted,
//     not written.
//   pwb / pparams (double-float kernel only): the per-panel network.  Before a panel below max_depth is evaluated
//     the warp runs the network on its lanes' panels; a panel whose predicted chance of being accepted is below
//     beta (logit margin < skip_logit) is split without evaluation.  Every evaluated panel is still accepted or split
//     by the plain error test.
struct ParamExtras
{
    uint32_t* panel_log;
    unsigned long long* log_count;
    long long log_cap;
    const __nv_bfloat16* pwb;
    const float* pparams;
    float skip_logit;
    float log10_tol;
    unsigned long long* skip_count;
};

// The per-panel network's shared memory, after the curve tile.
struct PanelSmem
{
    WeightsSmem w;
    uint32_t feat[kParamBlock / 32][32][kS16 - 4 + 1];
    float logit[kParamBlock / 32][32][2];
};

// DF: double-float panels.  PANEL (DF only): the per-panel network runs (its code and shared memory are compiled
// only into this instance, so the other instances keep their registers).  n_groups > 1 (DF only): the curve tiles
// of a query block are split into n_groups consecutive groups, one work item each, and each item writes its raw
// partial sum to partial[g * n + i] (a later kernel adds the groups in order) and adds its panel counts to
// nodes_total[i] (zeroed first).
template <bool DF, bool PANEL>
constexpr int param_min_blocks()
{
    return DF && !PANEL ? 6 : 1; // the double-float panels in 80 registers (no spills), six blocks per SM
}
template <bool DF, bool PANEL>
__global__ void __launch_bounds__(kParamBlock, param_min_blocks<DF, PANEL>()) k_param_gk15(const double* __restrict__ pos, int64_t n,
                                                            double* __restrict__ out, double x0x, double x0y,
                                                            double x0z, const Bez* __restrict__ curves,
                                                            int64_t n_curves, int tile, int min_depth, int max_depth,
                                                            double tol, const uint8_t* __restrict__ start_depth,
                                                            uint32_t* __restrict__ stats,
                                                            int32_t* __restrict__ nodes_total,
                                                            double* __restrict__ pair_vals, int* flags,
                                                            ParamExtras ex, int n_groups, double* __restrict__ partial)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ int s_next;
    __shared__ int s_nodes[kParamBlock];
    Bez* const buf = reinterpret_cast<Bez*>(smem);
    PanelSmem* const ps = reinterpret_cast<PanelSmem*>(smem + size_t(tile) * sizeof(Bez));
    bool const use_panel = PANEL && ex.pwb != nullptr;
    unsigned long long skips = 0;
    double* const slab = pair_vals + size_t(blockIdx.x) * kParamBlock * tile;
    ev3<rd> const x0{rd(x0x), rd(x0y), rd(x0z)};
    df3 const x0df{df_from(x0x), df_from(x0y), df_from(x0z)};
    double const x0n = x0x * x0x + x0y * x0y + x0z * x0z;
    bool const x0_unit = fabs(x0n - 1.0) <= 1e-15;
    df const x0n_df = df_from(x0n);
    int64_t const n_blocks_q = (n + kParamBlock - 1) / kParamBlock;
    int const n_tiles = int((n_curves + tile - 1) / tile);
    int const tiles_per_group = (n_tiles + n_groups - 1) / n_groups;
    int64_t const n_items = n_blocks_q * n_groups;
    unsigned const lane = threadIdx.x & 31u;
    // tol * 2^-depth by repeated halving, as the recursion computes it (exact unless it reaches subnormals)
    double tol_at[kParamMaxDepth + 1];
    tol_at[0] = tol;
    for (int l = 1; l <= kParamMaxDepth; ++l)
        tol_at[l] = __dmul_rn(tol_at[l - 1], 0.5);
    if (use_panel)
        load_weights(ps->w, ex.pwb, ex.pparams);
    float3 const x0f = make_float3(float(x0x), float(x0y), float(x0z));
    int const warp = int(threadIdx.x >> 5);
    if (threadIdx.x == 0)
    {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
    unsigned phase = 0;
    for (int64_t item = blockIdx.x; item < n_items; item += gridDim.x)
    {
        int64_t const qb = item / n_groups;
        int const grp = int(item - qb * n_groups);
        int const t_begin = grp * tiles_per_group;
        int const t_end = min(n_tiles, t_begin + tiles_per_group);
        int64_t const q0 = qb * kParamBlock;
        int const nq = int(n - q0 < kParamBlock ? n - q0 : int64_t(kParamBlock));
        rd sum = rd(0.0);
        s_nodes[threadIdx.x] = 0;
        for (int t = t_begin; t < t_end; ++t)
        {
            int64_t const c0 = int64_t(t) * tile;
            int const cnt = int(n_curves - c0 < tile ? n_curves - c0 : int64_t(tile));
            __syncthreads(); // the tile buffer and the slab are free
            if (threadIdx.x == 0)
            {
                s_next = 0;
                unsigned const bytes = unsigned(cnt) * unsigned(sizeof(Bez));
                mbar_arrive_expect_tx(&bar, bytes);
                bulk_copy_g2s(buf, curves + c0, bytes, &bar);
            }
            if (!mbar_wait_bounded(&bar, phase, flags, 4))
                return; // every thread of the block times out on the same barrier
            phase ^= 1u;

            int const total = cnt * nq; // pairs in this tile's pool, curve-major
            int pi = -1;                // this lane's pair, -1 = needs one
            bool drained = false;
            int k = 0, ql = 0, s = 0, d = 0, leaves = 0, dmin = 0, dmax = 0, pnodes = 0;
            uint32_t j = 0;
            ev3<rd> p{};
            df cp[DF ? 12 : 1]; // DF: this pair's curve minus its query, as power coefficients about t = 1/2
            double pending[kParamMaxDepth + 1];
            for (;;)
            {
                unsigned const want = __ballot_sync(0xffffffffu, pi < 0 && !drained);
                if (want)
                {
                    int base = 0;
                    unsigned const leader = __ffs(want) - 1;
                    if (lane == leader)
                        base = atomicAdd(&s_next, __popc(want));
                    base = __shfl_sync(0xffffffffu, base, leader);
                    if (want & (1u << lane))
                    {
                        int const mine = base + __popc(want & ((1u << lane) - 1u));
                        if (mine < total)
                        {
                            pi = mine;
                            k = mine / nq;
                            ql = mine - k * nq;
                            int64_t const q = q0 + ql;
                            p = ev3<rd>{rd(pos[3 * q]), rd(pos[3 * q + 1]), rd(pos[3 * q + 2])};
                            if constexpr (DF)
                            {
                                df const pd[3] = {df_from(p.x.v), df_from(p.y.v), df_from(p.z.v)};
                                CurveDF const& cv = reinterpret_cast<const CurveDF*>(buf)[k];
#pragma unroll
                                for (int e = 0; e < 12; ++e)
                                    cp[e] = cv.c[e] - pd[e % 3];
                                power_about_half(cp);
                            }
                            s = start_depth ? min(int(start_depth[q * n_curves + c0 + k]), max_depth) : 0;
                            d = s;
                            j = 0;
                            leaves = 0;
                            dmin = 255;
                            dmax = 0;
                            pnodes = 0;
                        }
                        else
                            drained = true;
                    }
                }
                if (!__any_sync(0xffffffffu, pi >= 0))
                    break;
                if constexpr (DF)
                {
                    // the per-panel network: up to four rounds of "split it without evaluating", all lanes together
                    for (int round = 0; PANEL && use_panel && round < 4; ++round)
                    {
                        bool const cand = pi >= 0 && d < max_depth;
                        float f[kF];
                        if (cand)
                        {
                            // the control points minus the query, as the network was trained on them
                            df const pd[3] = {df_from(p.x.v), df_from(p.y.v), df_from(p.z.v)};
                            CurveDF const& cv = reinterpret_cast<const CurveDF*>(buf)[k];
                            float cpf[12];
#pragma unroll
                            for (int e = 0; e < 12; ++e)
                                cpf[e] = (cv.c[e] - pd[e % 3]).hi;
                            panel_features(cpf, d, j, x0f, ex.log10_tol, f);
                        }
                        else
                        {
#pragma unroll
                            for (int e = 0; e < kF; ++e)
                                f[e] = 0.f;
                        }
                        uint32_t* const row = ps->feat[warp][lane];
#pragma unroll
                        for (int e = 0; e < kF / 2; ++e)
                            row[e] = pack_bf16(f[2 * e], f[2 * e + 1]);
                        row[6] = 0u;
                        row[7] = 0u;
                        __syncwarp();
                        int const g = int(lane >> 2), tig = int(lane & 3u);
#pragma unroll
                        for (int mt = 0; mt < 2; ++mt)
                        {
                            uint32_t a0[4] = {ps->feat[warp][mt * 16 + g][tig], ps->feat[warp][mt * 16 + g + 8][tig],
                                              ps->feat[warp][mt * 16 + g][4 + tig],
                                              ps->feat[warp][mt * 16 + g + 8][4 + tig]};
                            float z1[8][4], z2[8][4], z3[2][4];
                            mlp_forward(ps->w, a0, z1, z2, z3);
                            if (tig == 0) // columns 0 and 1: the split and accept logits
                            {
                                ps->logit[warp][mt * 16 + g][0] = z3[0][0];
                                ps->logit[warp][mt * 16 + g][1] = z3[0][1];
                                ps->logit[warp][mt * 16 + g + 8][0] = z3[0][2];
                                ps->logit[warp][mt * 16 + g + 8][1] = z3[0][3];
                            }
                        }
                        __syncwarp();
                        bool const skip =
                            cand && (ps->logit[warp][lane][1] - ps->logit[warp][lane][0]) < ex.skip_logit;
                        __syncwarp();
                        if (!__any_sync(0xffffffffu, skip))
                            break;
                        if (skip)
                        {
                            ++d; // split without evaluating: left child next
                            j <<= 1;
                            ++skips;
                        }
                    }
                }
                if (pi < 0)
                    continue;
                double err;
                double v;
                if constexpr (DF)
                {
                    float e32;
                    v = gk15_panel_df(cp, x0df, x0n_df, x0_unit, d, j, &e32);
                    err = double(e32);
                }
                else
                    v = gk15_panel(buf[k].c, p, x0, d, j, &err);
                ++pnodes;
                bool const accept = d >= max_depth || (d >= min_depth && err <= tol_at[d]);
                if (ex.panel_log && d < max_depth)
                {
                    unsigned long long const slot = atomicAdd(ex.log_count, 1ull);
                    if ((long long)slot < ex.log_cap)
                    {
                        ex.panel_log[2 * slot] = uint32_t((q0 + ql) * n_curves + c0 + k);
                        ex.panel_log[2 * slot + 1] = (uint32_t(d) << 25) | (j << 1) | (accept ? 1u : 0u);
                    }
                }
                if (!accept)
                {
                    ++d; // split: left child next
                    j <<= 1;
                    continue;
                }
                ++leaves;
                dmin = min(dmin, d);
                dmax = max(dmax, d);
                while (d > 0 && (j & 1u))
                {
                    v = __dadd_rn(pending[d], v); // left + right
                    --d;
                    j >>= 1;
                }
                if (d > 0)
                {
                    pending[d] = v; // a finished left child: its right sibling is next
                    ++j;
                    while (d < s)
                    {
                        ++d;
                        j <<= 1;
                    }
                    continue;
                }
                // the root is done: v is this pair's integral
                slab[size_t(k) * kParamBlock + ql] = v;
                if (stats)
                    stats[(q0 + ql) * n_curves + c0 + k] = uint32_t(min(leaves, 0xffff)) | (uint32_t(dmin) << 16) |
                                                           (uint32_t(dmax) << 24);
                atomicAdd(&s_nodes[ql], pnodes);
                pi = -1;
            }
            __syncthreads(); // the slab is complete
            if (int(threadIdx.x) < nq)
                for (int kk = 0; kk < cnt; ++kk)
                    sum = sum + rd(slab[size_t(kk) * kParamBlock + threadIdx.x]);
        }
        __syncthreads(); // s_nodes is complete
        if (int(threadIdx.x) < nq)
        {
            int64_t const i = q0 + threadIdx.x;
            if (n_groups == 1)
            {
                out[i] = (sum / (rd(4.0) * rd(3.141592653589793238462643383279502884))).v;
                if (nodes_total)
                    nodes_total[i] = s_nodes[threadIdx.x];
            }
            else
            {
                partial[int64_t(grp) * n + i] = sum.v;
                if (nodes_total)
                    atomicAdd(&nodes_total[i], s_nodes[threadIdx.x]);
            }
        }
    }
    if (ex.skip_count && skips)
        atomicAdd(ex.skip_count, skips);
}

// The groups' partial sums of each query added in group order (so in curve order by tiles), then normalised.
__global__ void k_param_groups(const double* __restrict__ partial, int n_groups, int64_t n, double* __restrict__ out)
{
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    {
        rd sum = rd(0.0);
        for (int g = 0; g < n_groups; ++g)
            sum = sum + rd(partial[int64_t(g) * n + i]);
        out[i] = (sum / (rd(4.0) * rd(3.141592653589793238462643383279502884))).v;
    }
}
} // namespace

int param_run(Context& ctx, const double* d_pos, int64_t n, double* d_out, const double* x0, const double* d_curves,
              int64_t n_curves, int min_depth, int max_depth, double tol, const uint8_t* d_start, uint32_t* d_stats,
              int32_t* d_nodes, uint32_t* d_panel_log, unsigned long long* d_log_count, long long log_cap)
{
    bool const dfm = ctx.param_mode == AGWN_PARAM_MIXED;
    bool const panel = dfm && ctx.panel_mlp && tol > 0;
    ParamExtras ex{};
    ex.panel_log = d_panel_log;
    ex.log_count = d_log_count;
    ex.log_cap = log_cap;
    if (panel)
    {
        const void* wb = nullptr;
        mlp_device_weights(ctx.panel_mlp, &wb, &ex.pparams);
        ex.pwb = static_cast<const __nv_bfloat16*>(wb);
        double const b = std::min(std::max(double(ctx.panel_beta), 1e-9), 1.0 - 1e-9);
        ex.skip_logit = float(std::log(b / (1.0 - b)));
        ex.log10_tol = float(std::log10(tol));
        ex.skip_count = ctx.timing ? reinterpret_cast<unsigned long long*>(ctx.d_counters + 2) : nullptr;
    }
    if (n == 0)
        return AGWN_OK;
    if (n_curves == 0)
    {
        AGWN_TRY_CUDA(cudaMemsetAsync(d_out, 0, sizeof(double) * n, ctx.stream));
        if (d_nodes)
            AGWN_TRY_CUDA(cudaMemsetAsync(d_nodes, 0, sizeof(int32_t) * n, ctx.stream));
        return AGWN_OK;
    }
    static_assert(sizeof(CurveDF) == sizeof(Bez), "both curve forms stage through the same tile");
    auto const kern = dfm ? (panel ? k_param_gk15<true, true> : k_param_gk15<true, false>) : k_param_gk15<false, false>;
    int tile = int(std::min<int64_t>(dfm ? kParamTileDF : kParamTileMax, n_curves));
    size_t smem = 0;
    int per_sm = 0;
    auto shape = [&](int t) -> int
    {
        smem = size_t(t) * sizeof(Bez) + (panel ? sizeof(PanelSmem) : 0);
        AGWN_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        AGWN_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kParamBlock, smem));
        if (per_sm < 1)
            return fail(AGWN_ERR_UNSUPPORTED, "parametric kernel does not fit on an SM");
        return AGWN_OK;
    };
    AGWN_TRY(shape(tile));
    int64_t const n_blocks_q = (n + kParamBlock - 1) / kParamBlock;
    int n_groups = 1;
    // two waves of work items; tiles of at least 128 curves (measured: more waves or other tiles change <1%)
    int64_t const waves = 2, min_tile = 128;
    if (dfm && n_blocks_q < waves * int64_t(per_sm) * ctx.sm_count)
    {
        // Few query blocks (a sample of queries, or many curves per query): the curves of each block are split
        // into groups of tiles, one work item each, so that every SM gets work.  Smaller tiles cost the
        // double-float kernel nothing (measured flat from 768 down to 128 curves) and let more blocks reside.
        int64_t const want = div_up(waves * int64_t(per_sm) * ctx.sm_count, n_blocks_q);
        int64_t const t = div_up(div_up(n_curves, want), 32) * 32;
        tile = int(std::max<int64_t>(std::min<int64_t>(t, tile), std::min<int64_t>(min_tile, n_curves)));
        AGWN_TRY(shape(tile));
        int const n_tiles = int(div_up(n_curves, tile));
        int64_t const groups =
            std::min<int64_t>(n_tiles, div_up(waves * int64_t(per_sm) * ctx.sm_count, n_blocks_q));
        int const tpg = int(div_up(n_tiles, groups));
        n_groups = int(div_up(n_tiles, tpg));
    }
    int64_t const n_items = n_blocks_q * n_groups;
    int const grid = int(std::max<int64_t>(1, std::min<int64_t>(n_items, int64_t(per_sm) * ctx.sm_count)));
    double* pair_vals = nullptr;
    AGWN_TRY(ctx.scratch_reserve(S_SEGS_RAW, sizeof(double) * size_t(grid) * kParamBlock * tile,
                                 reinterpret_cast<void**>(&pair_vals)));
    double* partial = nullptr;
    if (n_groups > 1)
    {
        AGWN_TRY(ctx.scratch_reserve(S_PARTIAL, sizeof(double) * size_t(n_groups) * size_t(n),
                                     reinterpret_cast<void**>(&partial)));
        if (d_nodes)
            AGWN_TRY_CUDA(cudaMemsetAsync(d_nodes, 0, sizeof(int32_t) * n, ctx.stream));
    }
    const void* tile_src = d_curves;
    if (dfm)
    {
        void* cdf = nullptr;
        AGWN_TRY(ctx.scratch_reserve(S_FRAME, sizeof(CurveDF) * size_t(n_curves), &cdf));
        AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
        k_curves_df<<<int(std::min<int64_t>(div_up(12 * n_curves, 256), 4 * ctx.sm_count)), 256, 0, ctx.stream>>>(
            d_curves, n_curves, static_cast<CurveDF*>(cdf));
        AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
        tile_src = cdf;
    }
    AGWN_TRY(ctx.launch_begin(AGWN_K_PARAMETRIC));
    kern<<<grid, kParamBlock, smem, ctx.stream>>>(d_pos, n, d_out, x0[0], x0[1], x0[2],
                                                 reinterpret_cast<const Bez*>(tile_src), n_curves, tile, min_depth,
                                                 max_depth, tol, d_start, d_stats, d_nodes, pair_vals, ctx.d_flags,
                                                 ex, n_groups, partial);
    AGWN_TRY(ctx.launch_end(AGWN_K_PARAMETRIC));
    if (n_groups == 1)
        return AGWN_OK;
    AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
    k_param_groups<<<int(std::min<int64_t>(div_up(n, 256), 8 * ctx.sm_count)), 256, 0, ctx.stream>>>(partial, n_groups,
                                                                                                     n, d_out);
    return ctx.launch_end(AGWN_K_OTHER);
}
} // namespace agwn

using namespace agwn;

namespace
{
// The parametric entry points: stage, optionally propose start depths with the learned network (mlp != NULL), run
// the integrator, copy host outputs back.
int param_entry(agwn_context* ctx, const agwn_mlp* mlp, int n_classes, float alpha, const double* positions, int64_t n,
                double* out, const double* x0, const double* curves, int64_t n_curves, int min_depth, int max_depth,
                double tol, const uint8_t* start_depth, uint32_t* pair_stats, int32_t* nodes_per_query)
{
    AGWN_CHECK_ARG(ctx && x0, "null context/x0");
    AGWN_CHECK_ARG(n >= 0 && n_curves >= 0 && (n == 0 || (positions && out)) && (n_curves == 0 || curves),
                   "bad arguments");
    AGWN_CHECK_ARG(min_depth >= 0 && max_depth >= 0 && max_depth <= kParamMaxDepth,
                   "depths must be in [0, %d] (max_depth bounds the explicit stack)", kParamMaxDepth);
    AGWN_CHECK_ARG(std::isfinite(tol) && tol >= 0, "tol must be finite and >= 0");
    AGWN_CHECK_ARG(n_curves < (int64_t(1) << 31), "too many curves");
    AGWN_CHECK_ARG(!mlp || tol > 0, "the learned proposal needs tol > 0");
    clear_message();
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    if (n == 0)
        return AGWN_OK;
    const void *dpos = nullptr, *dcur = nullptr, *dstart = nullptr;
    void *dout = nullptr, *dstats = nullptr, *dnodes = nullptr;
    bool h_out = false, h_stats = false, h_nodes = false;
    AGWN_TRY(stage_in(*ctx, positions, sizeof(double) * 3 * n, S_QUERIES, &dpos));
    AGWN_TRY(stage_in(*ctx, curves, sizeof(double) * 12 * n_curves, S_MISC0, &dcur));
    if (start_depth)
        AGWN_TRY(stage_in(*ctx, start_depth, size_t(n) * n_curves, S_MISC1, &dstart));
    AGWN_TRY(stage_out(*ctx, out, sizeof(double) * n, S_OUT, &dout, &h_out));
    if (pair_stats)
        AGWN_TRY(stage_out(*ctx, pair_stats, sizeof(uint32_t) * size_t(n) * n_curves, S_MISC2, &dstats, &h_stats));
    if (nodes_per_query)
        AGWN_TRY(stage_out(*ctx, nodes_per_query, sizeof(int32_t) * n, S_COUNTS, &dnodes, &h_nodes));
    // curves must be 16-byte aligned for the bulk copy; a host array was staged into aligned scratch
    if (reinterpret_cast<uintptr_t>(dcur) % 16 != 0)
    {
        void* aligned = nullptr;
        AGWN_TRY(ctx->scratch_reserve(S_SEGS, sizeof(double) * 12 * n_curves, &aligned));
        AGWN_TRY_CUDA(cudaMemcpyAsync(aligned, dcur, sizeof(double) * 12 * n_curves, cudaMemcpyDeviceToDevice,
                                      ctx->stream));
        dcur = aligned;
    }
    if (mlp && n_curves > 0)
    {
        void* proposed = nullptr;
        AGWN_TRY(ctx->scratch_reserve(S_MISC1, size_t(n) * n_curves, &proposed));
        AGWN_TRY(mlp_propose_run(*ctx, mlp, static_cast<const double*>(dpos), n, x0, static_cast<const double*>(dcur),
                                 n_curves, n_classes, min_depth, max_depth, tol, alpha,
                                 static_cast<uint8_t*>(proposed), nullptr));
        dstart = proposed;
    }
    AGWN_TRY(param_run(*ctx, static_cast<const double*>(dpos), n, static_cast<double*>(dout), x0,
                       static_cast<const double*>(dcur), n_curves, min_depth, max_depth, tol,
                       static_cast<const uint8_t*>(dstart), static_cast<uint32_t*>(dstats),
                       static_cast<int32_t*>(dnodes)));
    if (h_out)
        AGWN_TRY_CUDA(cudaMemcpyAsync(out, dout, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (h_stats)
        AGWN_TRY_CUDA(cudaMemcpyAsync(pair_stats, dstats, sizeof(uint32_t) * size_t(n) * n_curves,
                                      cudaMemcpyDeviceToHost, ctx->stream));
    if (h_nodes)
        AGWN_TRY_CUDA(cudaMemcpyAsync(nodes_per_query, dnodes, sizeof(int32_t) * n, cudaMemcpyDeviceToHost,
                                      ctx->stream));
    bool const sync = h_out || h_stats || h_nodes || dpos != positions || dcur != curves;
    return sync ? ctx->check_flags() : AGWN_OK;
}
} // namespace

extern "C" int agwn_param_batch_fractional_bezier3_f64(agwn_context* ctx, const double* positions, int64_t n,
                                                       double* out, const double* x0, const double* curves,
                                                       int64_t n_curves, int min_depth, int max_depth, double tol,
                                                       const uint8_t* start_depth, uint32_t* pair_stats,
                                                       int32_t* nodes_per_query)
{
    return param_entry(ctx, nullptr, 0, 0.f, positions, n, out, x0, curves, n_curves, min_depth, max_depth, tol,
                       start_depth, pair_stats, nodes_per_query);
}

extern "C" int agwn_param_batch_fractional_learned_bezier3_f64(agwn_context* ctx, const agwn_mlp* mlp,
                                                               const double* positions, int64_t n, double* out,
                                                               const double* x0, const double* curves,
                                                               int64_t n_curves, int n_classes, int min_depth,
                                                               int max_depth, double tol, float alpha,
                                                               uint32_t* pair_stats, int32_t* nodes_per_query)
{
    AGWN_CHECK_ARG(mlp, "null network");
    return param_entry(ctx, mlp, n_classes, alpha, positions, n, out, x0, curves, n_curves, min_depth, max_depth, tol,
                       nullptr, pair_stats, nodes_per_query);
}

extern "C" int agwn_param_set_panel_network(agwn_context* ctx, const agwn_mlp* mlp, float beta)
{
    AGWN_CHECK_ARG(ctx, "null context");
    AGWN_CHECK_ARG(beta > 0.f && beta < 1.f, "beta must be in (0, 1)");
    clear_message();
    ctx->panel_mlp = mlp;
    ctx->panel_beta = beta;
    return AGWN_OK;
}

extern "C" int agwn_param_panel_log_bezier3_f64(agwn_context* ctx, const double* positions, int64_t n,
                                                const double* x0, const double* curves, int64_t n_curves,
                                                int min_depth, int max_depth, double tol, uint32_t* log,
                                                int64_t capacity, int64_t* n_entries)
{
    AGWN_CHECK_ARG(ctx && x0 && n_entries && capacity >= 0 && (capacity == 0 || log), "bad arguments");
    AGWN_CHECK_ARG(n >= 0 && n_curves >= 0 && (n == 0 || positions) && (n_curves == 0 || curves), "bad arguments");
    AGWN_CHECK_ARG(n * n_curves < (int64_t(1) << 32), "the log indexes (query, curve) pairs in 32 bits");
    AGWN_CHECK_ARG(min_depth >= 0 && max_depth >= 0 && max_depth <= kParamMaxDepth, "bad depths");
    AGWN_CHECK_ARG(std::isfinite(tol) && tol >= 0, "tol must be finite and >= 0");
    clear_message();
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    *n_entries = 0;
    if (n == 0 || n_curves == 0)
        return AGWN_OK;
    const void *dpos = nullptr, *dcur = nullptr;
    void *dout = nullptr, *dlog = nullptr, *dcnt = nullptr;
    bool h_log = false;
    AGWN_TRY(stage_in(*ctx, positions, sizeof(double) * 3 * n, S_QUERIES, &dpos));
    AGWN_TRY(stage_in(*ctx, curves, sizeof(double) * 12 * n_curves, S_MISC0, &dcur));
    if (reinterpret_cast<uintptr_t>(dcur) % 16 != 0)
    {
        void* aligned = nullptr;
        AGWN_TRY(ctx->scratch_reserve(S_SEGS, sizeof(double) * 12 * n_curves, &aligned));
        AGWN_TRY_CUDA(cudaMemcpyAsync(aligned, dcur, sizeof(double) * 12 * n_curves, cudaMemcpyDeviceToDevice,
                                      ctx->stream));
        dcur = aligned;
    }
    AGWN_TRY(ctx->scratch_reserve(S_OUT, sizeof(double) * n, &dout));
    if (capacity > 0)
        AGWN_TRY(stage_out(*ctx, log, sizeof(uint32_t) * 2 * size_t(capacity), S_MISC2, &dlog, &h_log));
    AGWN_TRY(ctx->scratch_reserve(S_MISC3, sizeof(unsigned long long), &dcnt));
    AGWN_TRY_CUDA(cudaMemsetAsync(dcnt, 0, sizeof(unsigned long long), ctx->stream));
    AGWN_TRY(param_run(*ctx, static_cast<const double*>(dpos), n, static_cast<double*>(dout), x0,
                       static_cast<const double*>(dcur), n_curves, min_depth, max_depth, tol, nullptr, nullptr,
                       nullptr, static_cast<uint32_t*>(dlog), static_cast<unsigned long long*>(dcnt), capacity));
    unsigned long long cnt = 0;
    AGWN_TRY_CUDA(cudaMemcpyAsync(&cnt, dcnt, sizeof(cnt), cudaMemcpyDeviceToHost, ctx->stream));
    AGWN_TRY(ctx->check_flags());
    *n_entries = int64_t(cnt);
    if (h_log)
    {
        int64_t const rows = std::min<int64_t>(int64_t(cnt), capacity);
        AGWN_TRY_CUDA(cudaMemcpyAsync(log, dlog, sizeof(uint32_t) * 2 * size_t(rows), cudaMemcpyDeviceToHost,
                                      ctx->stream));
        AGWN_TRY(ctx->check_flags());
    }
    return AGWN_OK;
}
