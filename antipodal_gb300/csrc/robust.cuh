// Device side of the robust evaluator (RobustMeshGwn, src/antipodal/gwn_mesh_robust.hh:170-456): the exact
// predicates of src/antipodal/math/robust_predicates.hh under the three policies, quantisation, the integer-term
// leaf test and the fractional term's per-segment branches, and the two per-mesh kernels.  Shared by robust.cu
// (one mesh per call) and batch.cu (many meshes in one persistent launch).
#pragma once

#include "agwn_internal.cuh"
#include "frac_kernels.cuh"
#include "gwn_kernels.cuh"
#include "hier.cuh"

#include <cfloat>
#include <cmath>
#include <type_traits>

#include "robust_handle.cuh"

namespace agwn
{
namespace
{
// ---- 128-bit signed integers ------------------------------------------------------------------------------------
struct I128
{
    unsigned long long lo;
    long long hi;
};
__device__ __forceinline__ I128 i128_mul(long long a, long long b)
{
    return {static_cast<unsigned long long>(a) * static_cast<unsigned long long>(b), __mul64hi(a, b)};
}
__device__ __forceinline__ I128 i128_add(I128 a, I128 b)
{
    I128 r;
    r.lo = a.lo + b.lo;
    unsigned long long const carry = r.lo < a.lo ? 1ull : 0ull;
    r.hi = static_cast<long long>(static_cast<unsigned long long>(a.hi) + static_cast<unsigned long long>(b.hi) + carry);
    return r;
}
__device__ __forceinline__ I128 i128_neg(I128 a)
{
    I128 r;
    r.lo = ~a.lo + 1ull;
    r.hi = static_cast<long long>(~static_cast<unsigned long long>(a.hi) + (r.lo == 0 ? 1ull : 0ull));
    return r;
}
__device__ __forceinline__ int i128_sign(I128 a)
{
    return a.hi < 0 ? -1 : ((a.hi > 0 || a.lo != 0) ? 1 : 0);
}
// Correctly rounded conversion (what a native 128-bit integer to double conversion gives): the top 64 bits of the
// magnitude are rounded by the hardware conversion, with the bits below them folded into the lowest bit so that
// a discarded remainder breaks a tie the right way; the power of two is applied exactly.
__device__ __forceinline__ double i128_to_double(I128 a)
{
    bool const neg = a.hi < 0;
    I128 const m = neg ? i128_neg(a) : a;
    unsigned long long const H = static_cast<unsigned long long>(m.hi), L = m.lo;
    double r;
    if (H == 0)
        r = __ull2double_rn(L);
    else
    {
        int const lz = __clzll(static_cast<long long>(H));
        unsigned long long const top = lz ? (H << lz) | (L >> (64 - lz)) : H;
        unsigned long long const rest = lz ? (L << lz) : L;
        r = ldexp(__ull2double_rn(top | (rest ? 1ull : 0ull)), 64 - lz);
    }
    return neg ? -r : r;
}

template <class C>
struct qv3
{
    C x, y, z;
};

// ---- precision policies (robust_predicates.hh:186-215) ----------------------------------------------------------
struct P64 // int64_grid
{
    using C = int32_t;
    using W = long long;
    static constexpr int bits = 20;
    static constexpr bool grid = true;
    static __device__ __forceinline__ W mul(C a, C b) { return static_cast<W>(a) * static_cast<W>(b); }
    static __device__ __forceinline__ W add(W a, W b) { return a + b; }
    static __device__ __forceinline__ W sub(W a, W b) { return a - b; }
    static __device__ __forceinline__ int sgn(W a) { return a > 0 ? 1 : (a < 0 ? -1 : 0); }
    static __device__ __forceinline__ double dbl(W a) { return __ll2double_rn(a); }
    static __device__ __forceinline__ double cdbl(C a) { return double(a); }
};
struct P128 // int128_grid
{
    using C = int64_t;
    using W = I128;
    static constexpr int bits = 50;
    static constexpr bool grid = true;
    static __device__ __forceinline__ W mul(C a, C b) { return i128_mul(a, b); }
    static __device__ __forceinline__ W add(W a, W b) { return i128_add(a, b); }
    static __device__ __forceinline__ W sub(W a, W b) { return i128_add(a, i128_neg(b)); }
    static __device__ __forceinline__ int sgn(W a) { return i128_sign(a); }
    static __device__ __forceinline__ double dbl(W a) { return i128_to_double(a); }
    static __device__ __forceinline__ double cdbl(C a) { return __ll2double_rn(a); }
};
struct PF // exact_float
{
    using C = double;
    using W = double;
    static constexpr int bits = 0;
    static constexpr bool grid = false;
    static __device__ __forceinline__ int sgn(W a) { return a > 0 ? 1 : (a < 0 ? -1 : 0); }
    static __device__ __forceinline__ double dbl(W a) { return a; }
    static __device__ __forceinline__ double cdbl(C a) { return a; }
};

// x + y == a + b exactly.  robust_predicates.hh:227-233.
__device__ __forceinline__ void two_sum_d(double a, double b, double& x, double& y)
{
    x = __dadd_rn(a, b);
    double const bv = __dsub_rn(x, a);
    double const av = __dsub_rn(x, bv);
    y = __dadd_rn(__dsub_rn(a, av), __dsub_rn(b, bv));
}

// Exact sign of sum_i a[i] * b[i] through a nonoverlapping expansion.  robust_predicates.hh:238-264.
__device__ __noinline__ int sign_of_product_sum(const double* a, const double* b)
{
    double e[12];
    int n = 0;
    for (int i = 0; i < 6; ++i)
    {
        double const p = __dmul_rn(a[i], b[i]);
        double vals[2] = {fma(a[i], b[i], -p), p};
        for (int k = 0; k < 2; ++k)
        {
            double v = vals[k];
            for (int j = 0; j < n; ++j)
            {
                double s, r;
                two_sum_d(v, e[j], s, r);
                e[j] = r;
                v = s;
            }
            e[n++] = v;
        }
    }
    for (int i = n - 1; i >= 0; --i)
        if (e[i] != 0)
            return e[i] > 0 ? 1 : -1;
    return 0;
}

// 2x2 determinant of (q - q0, q1 - q0) in (y, z).  robust_predicates.hh:273-308.
template <class P>
__device__ __forceinline__ typename P::W edge_det(qv3<typename P::C> q, qv3<typename P::C> q0, qv3<typename P::C> q1)
{
    if constexpr (P::grid)
    {
        return P::add(P::mul(q.y - q0.y, q0.z - q1.z), P::mul(q.z - q0.z, q1.y - q0.y));
    }
    else
    {
        double const p1 = __dmul_rn(__dsub_rn(q.y, q0.y), __dsub_rn(q0.z, q1.z));
        double const p2 = __dmul_rn(__dsub_rn(q.z, q0.z), __dsub_rn(q1.y, q0.y));
        double const det = __dadd_rn(p1, p2);
        constexpr double eps = DBL_EPSILON / 2;
        constexpr double bound = (3.0 + 16.0 * eps) * eps;
        double const mag = __dadd_rn(fabs(p1), fabs(p2));
        if (fabs(det) > __dmul_rn(bound, mag))
            return det;
        if (mag == 0)
            return 0.0;
        double const a[6] = {q.y, -q.y, q0.y, q.z, -q.z, -q0.z};
        double const b[6] = {q0.z, q1.z, q1.z, q1.y, q0.y, q1.y};
        int const s = sign_of_product_sum(a, b);
        if (s == 0)
            return 0.0;
        return copysign(fmax(fabs(det), DBL_MIN), double(s));
    }
}

// robust_predicates.hh:314-331.
template <class P>
__device__ __forceinline__ int edge_sign(qv3<typename P::C> q, qv3<typename P::C> q0, qv3<typename P::C> q1)
{
    int const s = P::sgn(edge_det<P>(q, q0, q1));
    if (s)
        return s;
    if (q0.z != q1.z)
        return q0.z > q1.z ? 1 : -1;
    if (q1.y != q0.y)
        return q1.y > q0.y ? 1 : -1;
    return 0;
}

// robust_predicates.hh:339-356.
template <class P>
__device__ __forceinline__ typename P::W atan2_num(qv3<typename P::C> q, qv3<typename P::C> q0,
                                                   qv3<typename P::C> q1)
{
    using C = typename P::C;
    if constexpr (P::grid)
    {
        C const v0y = q0.y - q.y, v0z = q0.z - q.z, v1y = q1.y - q.y, v1z = q1.z - q.z;
        return P::sub(P::mul(v0z, v1y), P::mul(v0y, v1z));
    }
    else
    {
        double const t = edge_det<P>(q, q0, q1);
        if (t == 0)
            return 0.0;
        double const v0y = __dsub_rn(q0.y, q.y), v0z = __dsub_rn(q0.z, q.z);
        double const v1y = __dsub_rn(q1.y, q.y), v1z = __dsub_rn(q1.z, q.z);
        double const num = __dsub_rn(__dmul_rn(v0z, v1y), __dmul_rn(v0y, v1z));
        return copysign(fmax(fabs(num), DBL_MIN), -t);
    }
}

// a.y*b.y + a.z*b.z.  robust_predicates.hh:368-375.
template <class P>
__device__ __forceinline__ double dot_yz(qv3<typename P::C> a, qv3<typename P::C> b)
{
    if constexpr (P::grid)
        return P::dbl(P::add(P::mul(a.y, b.y), P::mul(a.z, b.z)));
    else
        return __dadd_rn(__dmul_rn(a.y, b.y), __dmul_rn(a.z, b.z));
}

// The query's projection into the predicate triangle (a, b, c) in (y, z): the common nonzero sign of its three
// edges (0 when it is outside or the edges disagree) and the unnormalised barycentric weights, each the edge
// determinant opposite its vertex.  robust_predicates.hh:390-402.
struct TriProj
{
    int sign;
    double w0, w1, w2;
};
template <class P>
__device__ __forceinline__ TriProj project_into_tri(qv3<typename P::C> q, qv3<typename P::C> a,
                                                    qv3<typename P::C> b, qv3<typename P::C> c)
{
    int const e01 = edge_sign<P>(q, a, b);
    int const e12 = edge_sign<P>(q, b, c);
    int const e20 = edge_sign<P>(q, c, a);
    if (e01 == 0 || e01 != e12 || e01 != e20)
        return TriProj{0, 0.0, 0.0, 0.0};
    return TriProj{e01, P::dbl(edge_det<P>(q, b, c)), P::dbl(edge_det<P>(q, c, a)), P::dbl(edge_det<P>(q, a, b))};
}

// Signed -x crossing of the predicate triangle (t0, t1, t2) for the query qi: robust_occluded_fn
// (gwn_mesh_robust.hh:122-145) with project_into_tri.
template <class P>
__device__ __forceinline__ int robust_crossing(qv3<typename P::C> q, const typename P::C* t)
{
    using C = typename P::C;
    qv3<C> const a{t[0], t[1], t[2]}, b{t[3], t[4], t[5]}, c{t[6], t[7], t[8]};
    TriProj const h = project_into_tri<P>(q, a, b, c);
    if (h.sign == 0)
        return 0;
    rd const hx = (rd(h.w0) * rd(P::cdbl(a.x)) + rd(h.w1) * rd(P::cdbl(b.x)) + rd(h.w2) * rd(P::cdbl(c.x))) /
                  (rd(h.w0) + rd(h.w1) + rd(h.w2));
    return P::cdbl(q.x) >= hx.v ? -h.sign : 0;
}

struct Quant
{
    double c[3];
    double s;
};

// The point as the predicate sees it: on the grid (clamped far out) or the doubles themselves.
// gwn_mesh_robust.hh:334-351.
template <class P>
__device__ __forceinline__ qv3<typename P::C> quantize(double x, double y, double z, Quant const& qz)
{
    using C = typename P::C;
    if constexpr (P::grid)
    {
        constexpr double max_q = double(1ll << (P::bits + 10));
        auto r = [&](double v, int k)
        {
            double const t = __dmul_rn(__dsub_rn(v, qz.c[k]), qz.s);
            double const cl = t < -max_q ? -max_q : (max_q < t ? max_q : t);
            return C(llround(cl));
        };
        return {r(x, 0), r(y, 1), r(z, 2)};
    }
    else
    {
        return {x, y, z};
    }
}

// Boundary segment on the predicate's coordinates, endpoints swapped (gwn_mesh_robust.hh:198-206).
template <class C>
struct alignas(16) RSeg
{
    C p0[3];
    C p1[3];
    double w;
};

// ---- build ------------------------------------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long dbl_order(double d)
{
    unsigned long long const u = __double_as_longlong(d);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__host__ __device__ inline double dbl_unorder(unsigned long long u)
{
    unsigned long long const b = (u & 0x8000000000000000ull) ? (u & 0x7fffffffffffffffull) : ~u;
    double d;
    std::memcpy(&d, &b, sizeof(d));
    return d;
}

// Exact bounding box of the vertices (as doubles) with order-preserving 64-bit atomics.
template <class T>
__global__ void k_bbox(const T* __restrict__ v, int64_t nv, unsigned long long* __restrict__ out)
{
    unsigned long long mn[3] = {~0ull, ~0ull, ~0ull}, mx[3] = {0, 0, 0};
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < nv; i += int64_t(gridDim.x) * blockDim.x)
        for (int k = 0; k < 3; ++k)
        {
            unsigned long long const o = dbl_order(double(v[3 * i + k]));
            mn[k] = o < mn[k] ? o : mn[k];
            mx[k] = o > mx[k] ? o : mx[k];
        }
    for (int k = 0; k < 3; ++k)
    {
        for (int off = 16; off > 0; off >>= 1)
        {
            unsigned long long const a = __shfl_xor_sync(0xffffffffu, mn[k], off);
            unsigned long long const b = __shfl_xor_sync(0xffffffffu, mx[k], off);
            mn[k] = a < mn[k] ? a : mn[k];
            mx[k] = b > mx[k] ? b : mx[k];
        }
        if ((threadIdx.x & 31) == 0)
        {
            atomicMin(out + k, mn[k]);
            atomicMax(out + 3 + k, mx[k]);
        }
    }
}

template <class T, class P>
__global__ void k_robust_tris(const T* __restrict__ v, int64_t nv, const int32_t* __restrict__ idx, int64_t n_tri,
                              Quant qz, typename P::C* __restrict__ tri_q, double* __restrict__ tri_d, int* flags)
{
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n_tri; t += int64_t(gridDim.x) * blockDim.x)
        for (int k = 0; k < 3; ++k)
        {
            int32_t const i = idx[3 * t + k];
            bool const ok = i >= 0 && i < nv;
            if (!ok)
                atomicOr(flags + FLAG_COUNT - 1, 1);
            int64_t const ii = ok ? i : 0;
            auto const q = quantize<P>(double(v[3 * ii]), double(v[3 * ii + 1]), double(v[3 * ii + 2]), qz);
            tri_q[9 * t + 3 * k] = q.x;
            tri_q[9 * t + 3 * k + 1] = q.y;
            tri_q[9 * t + 3 * k + 2] = q.z;
            tri_d[9 * t + 3 * k] = P::cdbl(q.x);
            tri_d[9 * t + 3 * k + 1] = P::cdbl(q.y);
            tri_d[9 * t + 3 * k + 2] = P::cdbl(q.z);
        }
}

template <class C>
__global__ void k_gather_leaves(const C* __restrict__ in, const unsigned* __restrict__ order, int64_t n,
                                C* __restrict__ out)
{
    for (int64_t l = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; l < n; l += int64_t(gridDim.x) * blockDim.x)
        for (int k = 0; k < 9; ++k)
            out[9 * l + k] = in[9 * int64_t(order[l]) + k];
}

template <class T, class P>
__global__ void k_robust_segs(const T* __restrict__ raw, int64_t n_seg, Quant qz, RSeg<typename P::C>* __restrict__ out)
{
    for (int64_t s = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; s < n_seg; s += int64_t(gridDim.x) * blockDim.x)
    {
        const T* w = raw + 7 * s;
        auto const a = quantize<P>(double(w[3]), double(w[4]), double(w[5]), qz); // swapped: pos1 first
        auto const b = quantize<P>(double(w[0]), double(w[1]), double(w[2]), qz);
        RSeg<typename P::C> r;
        r.p0[0] = a.x;
        r.p0[1] = a.y;
        r.p0[2] = a.z;
        r.p1[0] = b.x;
        r.p1[1] = b.y;
        r.p1[2] = b.z;
        r.w = double(w[6]);
        out[s] = r;
    }
}

// One block: the vertex chains of an int64_grid boundary (block_chains on the RSeg endpoints), then the entries;
// boundaries above kChainMax segments take one chain per segment.  *n_entries receives the count.  order:
// chain_scratch_ints(n_seg) ints of scratch.
__global__ void __launch_bounds__(1024) k_robust_chain(const RSeg<int32_t>* __restrict__ seg, int64_t n_seg,
                                                       RChain* __restrict__ out, long long* __restrict__ n_entries,
                                                       int* __restrict__ order)
{
    __shared__ int s_succ[kChainMax], s_pred[kChainMax];
    __shared__ unsigned char s_seen[kChainMax];
    __shared__ int s_m;
    bool const chain = n_seg <= kChainMax;
    int const ns = chain ? int(n_seg) : 0;
    int const mc = block_chains(
        ns, [&](int t) { return make_double3(seg[t].p0[0], seg[t].p0[1], seg[t].p0[2]); },
        [&](int t) { return make_double3(seg[t].p1[0], seg[t].p1[1], seg[t].p1[2]); }, order, order + 2 * ns,
        order + 4 * ns, s_succ, s_pred, s_seen, &s_m);
    int const m = chain ? mc : int(2 * n_seg);
    if (threadIdx.x == 0)
        *n_entries = m;
    for (int e = threadIdx.x; e < m; e += blockDim.x)
    {
        int si;
        bool start;
        if (chain)
        {
            int const o = order[e];
            start = o < 0;
            si = start ? ~o : o;
        }
        else
        {
            si = e >> 1;
            start = (e & 1) == 0;
        }
        RSeg<int32_t> const g = seg[si];
        RChain r{};
        for (int k = 0; k < 3; ++k)
            r.p[k] = start ? g.p0[k] : g.p1[k];
        r.s = start ? -1 : si;
        r.w = start ? 0.f : __double2float_rn(g.w);
        out[e] = r;
    }
}

// ---- evaluation -------------------------------------------------------------------------------------------------
constexpr int kRobBlock = 128;
constexpr int kRobCand = 8;

template <class T, class P>
__global__ void __launch_bounds__(kRobBlock) k_robust_count(const BvhNode* __restrict__ nodes,
                                                            const typename P::C* __restrict__ tri,
                                                            const float4* __restrict__ leaf_uv, int64_t n_tri,
                                                            float scene_scale, Frame32 f, Quant qz,
                                                            const T* __restrict__ pos, int64_t n,
                                                            int32_t* __restrict__ counts, int* flags)
{
    using C = typename P::C;
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    {
        qv3<C> const q = quantize<P>(double(pos[3 * i]), double(pos[3 * i + 1]), double(pos[3 * i + 2]), qz);
        int sum = 0;
        if (n_tri == 1)
            sum = robust_crossing<P>(q, tri);
        else if (n_tri > 1)
        {
            float const ox = float(P::cdbl(q.x)), oy = float(P::cdbl(q.y)), oz = float(P::cdbl(q.z));
            float const u = f.r[0] * ox + f.r[1] * oy + f.r[2] * oz;
            float const v = f.r[3] * ox + f.r[4] * oy + f.r[5] * oz;
            float const w = f.r[6] * ox + f.r[7] * oy + f.r[8] * oz;
            float const qmax = fmaxf(fmaxf(fabsf(ox), fabsf(oy)), fabsf(oz));
            float const tol = (qmax + scene_scale) * 3.8146973e-6f + 1e-30f;
            float const m8 = margin_permuted(qmax, scene_scale);
            int cand[kRobCand];
            int nc = 0;
            bool const ok = hier_walk(nodes, leaf_uv, u, v, w, tol, m8,
                                      [&](int leaf)
                                      {
                                          if (nc == kRobCand)
                                          {
                                              for (int j = 0; j < kRobCand; ++j)
                                                  sum += robust_crossing<P>(q, tri + 9 * int64_t(cand[j]));
                                              nc = 0;
                                          }
                                          cand[nc++] = leaf;
                                      });
            if (!ok)
                atomicOr(flags + FLAG_STACK, 1);
            for (int j = 0; j < nc; ++j)
                sum += robust_crossing<P>(q, tri + 9 * int64_t(cand[j]));
        }
        counts[i] = sum;
    }
}

// k_robust_count with the candidate leaves read from the cell grid of the evaluator's hierarchy (the walk for
// queries beyond the grid's tolerance), and most of them decided in float.  The hierarchy's frame for the -x ray is
// (u, v, w) = (z, y, -x), exact in double, and its leaf corners are the predicate's own coordinates, so
// certain_leaf's edge functions are the negated (y, z) edge determinants and its "in front" is q.x >= the hit's x:
// where it decides (all three edges, and the depth, beyond margins ~1e8 times the rounding of either
// computation) its value is robust_crossing's, -e01 or 0.  The other leaves -- within the margin of an edge, a
// vertex or the plane -- take robust_crossing itself.  The counts are the exact predicate's.
// The undecided leaves take robust_crossing a warp's worth at a time (leafq_push, hier.cuh); the loop over
// queries is warp-uniform.  stats: counters, or null.
template <class T, class P>
__global__ void __launch_bounds__(kRobBlock) k_robust_cells(const BvhNode* __restrict__ nodes,
                                                            const typename P::C* __restrict__ tri,
                                                            const float4* __restrict__ leaf_uv, float scene_scale,
                                                            Frame32 f, CellView g, Quant qz,
                                                            const T* __restrict__ pos, int64_t n,
                                                            int32_t* __restrict__ counts, int* flags,
                                                            long long* stats)
{
    using C = typename P::C;
    __shared__ int s_leaf[kRobBlock / 32][kLeafQCap];
    __shared__ long long s_query[kRobBlock / 32][kLeafQCap];
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    LeafQueue lq;
    lq.leaf = s_leaf[warp];
    lq.query = s_query[warp];
    auto const exact = [&](long long qi, int leaf) -> int
    {
        qv3<C> const q = quantize<P>(double(pos[3 * qi]), double(pos[3 * qi + 1]), double(pos[3 * qi + 2]), qz);
        return robust_crossing<P>(q, tri + 9 * int64_t(leaf));
    };
    long long n_q = 0, n_entries = 0, n_leaves = 0, n_exact = 0;
    int64_t const stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t base = blockIdx.x * int64_t(blockDim.x) + (threadIdx.x & ~31); base < n; base += stride)
    {
        int64_t const i = base + lane;
        int und[kUndecided];
        int nu = 0;
        if (i < n)
        {
            qv3<C> const q = quantize<P>(double(pos[3 * i]), double(pos[3 * i + 1]), double(pos[3 * i + 2]), qz);
            float const ox = float(P::cdbl(q.x)), oy = float(P::cdbl(q.y)), oz = float(P::cdbl(q.z));
            float const u = f.r[0] * ox + f.r[1] * oy + f.r[2] * oz;
            float const v = f.r[3] * ox + f.r[4] * oy + f.r[5] * oz;
            float const w = f.r[6] * ox + f.r[7] * oy + f.r[8] * oz;
            float const qmax = fmaxf(fmaxf(fabsf(ox), fabsf(oy)), fabsf(oz));
            float const tol = (qmax + scene_scale) * 3.8146973e-6f + 1e-30f;
            float const m8 = margin_permuted(qmax, scene_scale);
            int sum = 0;
            auto const consider = [&](int leaf)
            {
                ++n_leaves;
                int const c = certain_leaf(leaf_uv, leaf, u, v, w, m8);
                if (c != 2)
                {
                    sum += c;
                    return;
                }
                ++n_exact;
                if (nu < kUndecided)
                    und[nu++] = leaf;
                else
                    sum += robust_crossing<P>(q, tri + 9 * int64_t(leaf));
            };
            if (tol <= g.tol_max)
                n_entries += cell_candidates(g, leaf_uv, u, v, w, tol, m8, consider);
            else if (!hier_walk(nodes, leaf_uv, u, v, w, tol, m8, consider))
                atomicOr(flags + FLAG_STACK, 1);
            counts[i] = sum;
            ++n_q;
        }
        leafq_push(lq, und, nu, i, lane, counts, exact);
    }
    leafq_drain(lq, lane, counts, exact);
    if (stats)
        integer_stats(stats, n_q, n_entries, n_leaves, n_exact);
}

template <class P>
__device__ __forceinline__ double l_plus_x(qv3<typename P::C> v, double l)
{
    double const vx = P::cdbl(v.x);
    if (v.x >= 0)
        return __dadd_rn(l, vx);
    return __ddiv_rn(dot_yz<P>(v, v), __dsub_rn(l, vx));
}

// Half-area contribution of one boundary segment.  gwn_mesh_robust.hh:272-321.
template <class P>
__device__ __forceinline__ double robust_contrib(qv3<typename P::C> q, RSeg<typename P::C> const& s)
{
    using C = typename P::C;
    constexpr double pi = 3.141592653589793238462643383279502884;
    qv3<C> const p0{s.p0[0], s.p0[1], s.p0[2]}, p1{s.p1[0], s.p1[1], s.p1[2]};
    qv3<C> v0, v1;
    if constexpr (P::grid)
    {
        v0 = {C(p0.x - q.x), C(p0.y - q.y), C(p0.z - q.z)};
        v1 = {C(p1.x - q.x), C(p1.y - q.y), C(p1.z - q.z)};
    }
    else
    {
        v0 = {__dsub_rn(p0.x, q.x), __dsub_rn(p0.y, q.y), __dsub_rn(p0.z, q.z)};
        v1 = {__dsub_rn(p1.x, q.x), __dsub_rn(p1.y, q.y), __dsub_rn(p1.z, q.z)};
    }
    ev3<rd> const d0{rd(P::cdbl(v0.x)), rd(P::cdbl(v0.y)), rd(P::cdbl(v0.z))};
    ev3<rd> const d1{rd(P::cdbl(v1.x)), rd(P::cdbl(v1.y)), rd(P::cdbl(v1.z))};
    double const l0 = ex_sqrt(edot(d0, d0)).v;
    double const l1 = ex_sqrt(edot(d1, d1)).v;
    auto const num = atan2_num<P>(q, p0, p1);
    double const yz = dot_yz<P>(v0, v1);
    double const den = __dadd_rn(__dmul_rn(l_plus_x<P>(v0, l0), l_plus_x<P>(v1, l1)), yz);
    if (P::sgn(num) != 0)
        return atan2(P::dbl(num), den);
    if (v0.y == 0 && v0.z == 0 && v0.x < 0 && (v1.y != 0 || v1.z != 0))
        return v1.z != 0 ? atan2(P::cdbl(v1.z), -P::cdbl(v1.y)) : (v1.y > 0 ? -pi : 0.0);
    if (v1.y == 0 && v1.z == 0 && v1.x < 0 && (v0.y != 0 || v0.z != 0))
        return v0.z != 0 ? atan2(-P::cdbl(v0.z), -P::cdbl(v0.y)) : (v0.y > 0 ? pi : 0.0);
    int const sg = -edge_sign<P>(q, p0, p1);
    return den < 0.0 ? double(sg) * pi : 0.0;
}

// ---- mixed precision (int64_grid) -------------------------------------------------------------------------------
// Per-warp queue of the pairs the FP32 path turned down, evaluated in FP64 32 at a time (one per lane), so
// that the narrow FP64 pipe runs full warps instead of one diverged lane.  Entry: (segment << 8) | (lane << 3) | k,
// with the segment's index in the mesh's boundary array (below 2^24).
template <int K>
struct RQueue
{
    static constexpr unsigned kCap = 128u * K; // > 31 left over + 2 * 32 * K appended per pair of segments
    uint32_t* e;
    double* res;
    unsigned head = 0, tail = 0; // warp-uniform
};

// Appends this lane's pair if it was turned down (every lane of the warp calls it).
template <int K>
__device__ __forceinline__ void rq_push(RQueue<K>& fq, bool down, uint32_t seg, int lane, int k)
{
    unsigned const m = __ballot_sync(0xffffffffu, down);
    if (m)
    {
        if (down)
            fq.e[(fq.tail + __popc(m & ((1u << lane) - 1u))) & (RQueue<K>::kCap - 1)] =
                (seg << 8) | (uint32_t(lane) << 3) | uint32_t(k);
        fq.tail += __popc(m);
    }
}

// Evaluates the next c (<= 32) queued pairs, one per lane, and adds each result to its owner's half[k] in queue
// order (so each query's FP64 terms keep segment order).  Every lane of the warp calls it.
template <class P, int K>
__device__ __forceinline__ void rq_flush(RQueue<K>& fq, unsigned c, int lane, const RSeg<typename P::C>* gseg,
                                         const qv3<typename P::C> (&q)[K], double (&half)[K])
{
    using C = typename P::C;
    __syncwarp();
    uint32_t const e = fq.e[(fq.head + min(unsigned(lane), c - 1)) & (RQueue<K>::kCap - 1)];
    int const owner = int((e >> 3) & 31u), kk = int(e & 7u);
    qv3<C> qq = q[0];
#pragma unroll
    for (int k = 0; k < K; ++k)
    {
        C const x = __shfl_sync(0xffffffffu, q[k].x, owner), y = __shfl_sync(0xffffffffu, q[k].y, owner),
                z = __shfl_sync(0xffffffffu, q[k].z, owner);
        if (kk == k)
            qq = {x, y, z};
    }
    if (unsigned(lane) < c)
    {
        RSeg<C> const sg = gseg[e >> 8];
        fq.res[lane] = __dmul_rn(sg.w, robust_contrib<P>(qq, sg));
    }
    __syncwarp();
    for (unsigned j = 0; j < c; ++j)
    {
        uint32_t const ej = fq.e[(fq.head + j) & (RQueue<K>::kCap - 1)];
        if (int((ej >> 3) & 31u) == lane)
        {
            double const r = fq.res[j];
#pragma unroll
            for (int k = 0; k < K; ++k)
                if (int(ej & 7u) == k)
                    half[k] = __dadd_rn(half[k], r);
        }
    }
    __syncwarp();
    fq.head += c;
}

// The lane vectors of the chain loop: K = 1 query per thread as float, or K / 2 packed pairs (float2).
template <int K>
struct RLanes
{
    using V = std::conditional_t<K == 1, float, float2>;
    static constexpr int W = K == 1 ? 1 : 2; // queries per lane vector
    static constexpr int NP = K / W;         // lane vectors per thread
    static_assert(K == 1 || K % 2 == 0, "one query per thread or packed pairs");
};

// Per-vertex quantities of one chain vertex relative to the queries of a lane vector: v = p - q as floats (exact:
// below 2^24), and the half-angle pair (n, d) of l + x; d is NaN when a difference is 2^24 or more (the pairs at
// that vertex go to FP64).
template <class V>
struct RVState
{
    V x, y, z, n, d;
};

// One chain entry with K queries: its vertex into cv, then (a segment entry) the fractional term of the segment
// from the previous vertex pv, on the FP32 pipe, into the TwoSum accumulators -- or its bit (slot * K + k) set in
// `bits` for FP64.  Under int64_grid the differences v = p - q are exact integers; below 2^24 they are exact
// floats.  The atan2 numerator num = z0 y1 - y0 z1 and y0 y1 + z0 z1 come from TwoProduct FMAs (error ~2 ulp of the
// result; num is 0 exactly when the exact value is), |v| from an approximate rsqrt, and l + x in the reference's
// cancellation-free half-angle form (l + x, or (y^2 + z^2) / (l - x) for x < 0) with num and den scaled by the two
// denominators (no division).  With 4 eps32 per operand chain -- the estimate of the mesh kernel's mixed form --
// num errs by 4u |num| and den = A B + yz by 4u (|A B| + |yz|), so the angle errs by about
// (|num| E_d + |den| E_n) / (num^2 + den^2).  The pair stays in FP32 when that is at most term_err; num == 0 (where
// the reference takes its exact branches), a difference of 2^24 or more and ill-conditioned pairs go to FP64 with
// the reference's formula.  The arithmetic runs on lane vectors (RLanes), so one query per thread and packed
// pairs give the same bits; selects and comparisons per lane.
template <int K>
__device__ __forceinline__ void robust_chain_entry(RChain const& e, qv3<int32_t> const (&q)[K],
                                                   RVState<typename RLanes<K>::V> (&pv)[RLanes<K>::NP],
                                                   RVState<typename RLanes<K>::V> (&cv)[RLanes<K>::NP], float term_err,
                                                   typename RLanes<K>::V (&acc)[RLanes<K>::NP],
                                                   typename RLanes<K>::V (&comp)[RLanes<K>::NP], uint32_t& bits,
                                                   int slot)
{
    using L = RLanes<K>;
    using V = typename L::V;
    unsigned const lim = 1u << 25, off = 1u << 24;
#pragma unroll
    for (int p = 0; p < L::NP; ++p)
    {
        RVState<V>& c = cv[p];
        bool small[L::W];
#pragma unroll
        for (int h = 0; h < L::W; ++h)
        {
            int const k = p * L::W + h;
            int32_t const vx = e.p[0] - q[k].x, vy = e.p[1] - q[k].y, vz = e.p[2] - q[k].z;
            small[h] = unsigned(vx) + off < lim && unsigned(vy) + off < lim && unsigned(vz) + off < lim;
            ln(c.x, h) = float(vx);
            ln(c.y, h) = float(vy);
            ln(c.z, h) = float(vz);
        }
        V const yz = lv_fma(c.y, c.y, lv_mul(c.z, c.z));
        V const sq = lv_fma(c.x, c.x, yz);
        V rs;
#pragma unroll
        for (int h = 0; h < L::W; ++h)
            ln(rs, h) = rsqrtf(ln(sq, h));
        V const l = lv_mul(sq, rs);
        V const lpx = lv_add(l, c.x), lmx = lv_sub(l, c.x);
#pragma unroll
        for (int h = 0; h < L::W; ++h)
        {
            bool const xpos = ln(c.x, h) >= 0.f;
            ln(c.n, h) = xpos ? ln(lpx, h) : ln(yz, h);
            ln(c.d, h) = small[h] ? (xpos ? 1.f : ln(lmx, h)) : __int_as_float(0x7fffffff);
        }
    }
    if (e.s < 0)
        return; // a chain start: its vertex only
    V const m1 = lv_set<V>(-1.f);
#pragma unroll
    for (int p = 0; p < L::NP; ++p)
    {
        RVState<V> const& a = pv[p];
        RVState<V> const& b = cv[p];
        V const pn = lv_mul(a.y, b.z);
        V const npn = lv_mul(pn, m1);
        V const en = lv_fma(a.y, b.z, npn);
        V const numf = lv_sub(lv_fma(a.z, b.y, npn), en);
        V const pz = lv_mul(a.z, b.z);
        V const ez = lv_fma(a.z, b.z, lv_mul(pz, m1));
        V const yzf = lv_add(lv_fma(a.y, b.y, pz), ez);
        V const D = lv_mul(a.d, b.d), ab = lv_mul(a.n, b.n), yzs = lv_mul(yzf, D);
        V const num_s = lv_mul(numf, D), den_s = lv_add(ab, yzs);
        V an, ad, inv, sab;
        bool swap[L::W];
#pragma unroll
        for (int h = 0; h < L::W; ++h)
        {
            float const anh = fabsf(ln(num_s, h)), adh = fabsf(ln(den_s, h));
            swap[h] = anh > adh;
            ln(an, h) = anh;
            ln(ad, h) = adh;
            ln(inv, h) = __fdividef(1.f, fmaxf(swap[h] ? anh : adh, 1e-37f));
            ln(sab, h) = __fadd_rn(fabsf(ln(ab, h)), fabsf(ln(yzs, h)));
        }
        V const an1 = lv_mul(an, inv), ad1 = lv_mul(ad, inv);
        constexpr float k4u = 4.f * 5.9604645e-8f;
        V const bound = lv_mul(lv_set<V>(k4u), lv_fma(an1, lv_mul(sab, inv), lv_mul(ad1, an1)));
        V const rhs = lv_mul(lv_set<V>(term_err), lv_fma(an1, an1, lv_mul(ad1, ad1)));
        V t, x;
#pragma unroll
        for (int h = 0; h < L::W; ++h)
            ln(t, h) = swap[h] ? ln(ad1, h) : ln(an1, h);
        // atan2(num_s, den_s): atan(t), then the octant
        V th = atan_unit_lv(t);
        V const th_sw = lv_sub(lv_set<V>(1.5707963267948966f), th);
#pragma unroll
        for (int h = 0; h < L::W; ++h)
            ln(th, h) = swap[h] ? ln(th_sw, h) : ln(th, h);
        V const th_neg = lv_sub(lv_set<V>(3.141592653589793f), th);
        V const w = lv_set<V>(e.w);
#pragma unroll
        for (int h = 0; h < L::W; ++h)
            ln(th, h) = copysignf(ln(den_s, h) < 0.f ? ln(th_neg, h) : ln(th, h), ln(num_s, h));
        V const term = lv_mul(w, th);
#pragma unroll
        for (int h = 0; h < L::W; ++h)
        {
            // num == 0 (the reference's exact branches), an out-of-range difference (NaN d) or an ill-conditioned
            // pair
            bool const need = ln(numf, h) == 0.f || !(ln(bound, h) <= ln(rhs, h));
            bits |= need ? (1u << (slot * K + p * L::W + h)) : 0u;
            ln(x, h) = need ? 0.f : ln(term, h);
        }
        two_sum_lv(acc[p], comp[p], x);
    }
}

// Two chain entries (sb[s], sb[s + 1]; ne of them) with K queries; entries at even positions of the stream write
// st0, odd ones st1 (tiles start at even positions).  Pairs turned down are pushed to the FP64 queue in stream
// order only when a lane of the warp has one; the queue is then drained in full batches.  Shared by k_robust_frac
// and the batch kernel, so their sums agree bit for bit.
template <class P, int K>
__device__ __forceinline__ void robust_chain_step(RChain const* sb, int s, int ne, qv3<int32_t> const (&q)[K],
                                                  RVState<typename RLanes<K>::V> (&st0)[RLanes<K>::NP],
                                                  RVState<typename RLanes<K>::V> (&st1)[RLanes<K>::NP],
                                                  float term_err, typename RLanes<K>::V (&acc)[RLanes<K>::NP],
                                                  typename RLanes<K>::V (&comp)[RLanes<K>::NP], RQueue<K>& fq,
                                                  int lane, RSeg<typename P::C> const* gseg, double (&half)[K])
{
    uint32_t bits = 0;
    robust_chain_entry<K>(sb[s], q, st1, st0, term_err, acc, comp, bits, 0);
    if (ne > 1)
        robust_chain_entry<K>(sb[s + 1], q, st0, st1, term_err, acc, comp, bits, 1);
    if (__any_sync(0xffffffffu, bits != 0u))
    {
#pragma unroll
        for (int e = 0; e < 2; ++e)
        {
            if (e >= ne)
                break;
            uint32_t const si = uint32_t(sb[s + e].s);
#pragma unroll
            for (int k = 0; k < K; ++k)
                rq_push(fq, ((bits >> (e * K + k)) & 1u) != 0u, si, lane, k);
        }
        while (fq.tail - fq.head >= 32)
            rq_flush<P, K>(fq, 32, lane, gseg, q, half);
    }
}

// Mixed = true (int64_grid only): FP32 pairs on the boundary's vertex chains (robust_chain_step) with TwoSum
// accumulation, the others in FP64.
template <class T, class P, bool Mixed = false>
__global__ void __launch_bounds__(kRobBlock) k_robust_frac(const T* __restrict__ pos, int64_t n, Quant qz,
                                                           const RSeg<typename P::C>* __restrict__ seg, int64_t n_seg,
                                                           const RChain* __restrict__ chain, int64_t n_entries,
                                                           int tile, const int32_t* __restrict__ counts,
                                                           T* __restrict__ out, T* __restrict__ out_frac, int* flags,
                                                           float term_err, long long* counters)
{
    using Seg = RSeg<typename P::C>;
    // the mixed form walks the boundary's vertex chains (RChain), the exact form its segments
    using Elem = std::conditional_t<Mixed, RChain, Seg>;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ int abort_cta;
    int64_t const n_elem = Mixed ? n_entries : n_seg;
    TilePipe<Elem> pipe;
    pipe.n_tiles = int((n_elem + tile - 1) / tile);
    pipe.single = pipe.n_tiles <= 1;
    pipe.buf[0] = reinterpret_cast<Elem*>(smem);
    pipe.buf[1] = pipe.buf[0] + (pipe.single ? 0 : tile);
    pipe.bar = bars;
    if constexpr (Mixed)
        pipe.gseg = chain;
    else
        pipe.gseg = seg;
    pipe.n_seg = n_elem;
    pipe.tile = tile;
    constexpr int kWarps = kRobBlock / 32;
    __shared__ uint32_t q_entries[Mixed ? kWarps : 1][RQueue<1>::kCap];
    __shared__ double q_results[Mixed ? kWarps : 1][32];
    int const lane = threadIdx.x & 31;
    RQueue<1> fq;
    fq.e = q_entries[Mixed ? threadIdx.x / 32 : 0];
    fq.res = q_results[Mixed ? threadIdx.x / 32 : 0];
    int64_t const per_tile = blockDim.x;
    int64_t const n_qtiles = (n + per_tile - 1) / per_tile;
    int const my_qtiles = blockIdx.x < n_qtiles ? int((n_qtiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;
    int const n_items = n_seg == 0 ? 0 : (pipe.single ? (my_qtiles > 0 ? 1 : 0) : my_qtiles * pipe.n_tiles);
    if (threadIdx.x == 0)
    {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_barrier_init();
        abort_cta = 0;
        if (n_items > 0)
            pipe.issue(0);
        if (n_items > 1)
            pipe.issue(1);
    }
    __syncthreads();
    constexpr double f_norm = 2.0 / (4.0 * 3.141592653589793238462643383279502884);
    int it = 0;
    for (int j = 0; j < my_qtiles; ++j)
    {
        int64_t const i = (blockIdx.x + int64_t(j) * gridDim.x) * per_tile + threadIdx.x;
        int64_t const ii = i < n ? i : n - 1;
        auto const q = quantize<P>(double(pos[3 * ii]), double(pos[3 * ii + 1]), double(pos[3 * ii + 2]), qz);
        double half = 0.0;
        float acc[1] = {0.f}, comp[1] = {0.f};
        decltype(q) qarr[1] = {q};
        double harr[1] = {0.0};
        RVState<float> st0[1] = {}, st1[1] = {};
        for (int st = 0; st < pipe.n_tiles && n_seg > 0; ++st)
        {
            int const b = it & 1;
            // a single tile stays in shared memory for every query tile: only the first waits for it, and the warps then
            // run the others without meeting at a barrier
            bool const landed = !pipe.single || j == 0;
            if (landed)
            {
                if (!mbar_wait_bounded(&bars[b], unsigned((it >> 1) & 1), flags, 3))
                    abort_cta = 1;
                __syncthreads();
                if (abort_cta)
                    return;
            }
            Elem const* sb = pipe.buf[b];
            int const cnt = pipe.tile_count(st);
            if constexpr (Mixed)
            {
                // tiles start at even stream positions (the tile is even), so the state alternation runs across them
                for (int s = 0; s < cnt; s += 2)
                    robust_chain_step<P, 1>(sb, s, cnt - s < 2 ? cnt - s : 2, qarr, st0, st1, term_err, acc, comp, fq,
                                            lane, seg, harr);
            }
            else
            {
                for (int s = 0; s < cnt; ++s)
                {
                    Seg const sgm = sb[s];
                    half = __dadd_rn(half, __dmul_rn(sgm.w, robust_contrib<P>(q, sgm)));
                }
            }
            if (!pipe.single)
            {
                __syncthreads();
                if (threadIdx.x == 0 && it + 2 < n_items)
                    pipe.issue(it + 2);
                ++it;
            }
        }
        if constexpr (Mixed)
        {
            while (fq.tail != fq.head)
                rq_flush<P, 1>(fq, min(32u, fq.tail - fq.head), lane, seg, qarr, harr);
            half = __dadd_rn(harr[0], __dadd_rn(double(acc[0]), double(comp[0])));
            if (counters && lane == 0)
            {
                atomicAdd(reinterpret_cast<unsigned long long*>(counters), (unsigned long long)fq.tail);
                atomicAdd(reinterpret_cast<unsigned long long*>(counters + 1), 32ull * (unsigned long long)n_seg);
            }
            fq.tail = fq.head = 0; // the queue is empty; every lane restarts its copy of the counters

        }
        if (i < n)
        {
            T const fr = T(__dmul_rn(half, f_norm));
            T const c = T(counts ? counts[i] : 0);
            out[i] = fr + c;
            if (out_frac)
                out_frac[i] = fr;
        }
    }
}
} // namespace
} // namespace agwn
