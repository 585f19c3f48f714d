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

#include "agwn_internal.cuh"
#include "frac_kernels.cuh"
#include "gwn_kernels.cuh"
#include "hier.cuh"

#include <algorithm>
#include <cfloat>
#include <cmath>

namespace agwn
{
struct Robust
{
    int device = 0;
    int scalar_bytes = 8;
    int policy = 0;
    int64_t n_tri = 0;
    int64_t n_seg = 0;
    double center[3] = {0, 0, 0};
    double scale = 1.0;
    void* tri = nullptr; // predicate triangles in leaf order
    void* seg = nullptr; // quantised, swapped boundary segments
    Hier hier;
};
} // namespace agwn

struct agwn_robust : agwn::Robust
{
};

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

// Signed -x crossing of the predicate triangle (t0, t1, t2) for the query qi: robust_occluded_fn
// (gwn_mesh_robust.hh:122-145) with project_into_tri (robust_predicates.hh:390-402).
template <class P>
__device__ __forceinline__ int robust_crossing(qv3<typename P::C> q, const typename P::C* t)
{
    using C = typename P::C;
    qv3<C> const a{t[0], t[1], t[2]}, b{t[3], t[4], t[5]}, c{t[6], t[7], t[8]};
    int const e01 = edge_sign<P>(q, a, b);
    int const e12 = edge_sign<P>(q, b, c);
    int const e20 = edge_sign<P>(q, c, a);
    if (e01 == 0 || e01 != e12 || e01 != e20)
        return 0;
    double const w0 = P::dbl(edge_det<P>(q, b, c));
    double const w1 = P::dbl(edge_det<P>(q, c, a));
    double const w2 = P::dbl(edge_det<P>(q, a, b));
    rd const hx = (rd(w0) * rd(P::cdbl(a.x)) + rd(w1) * rd(P::cdbl(b.x)) + rd(w2) * rd(P::cdbl(c.x))) /
                  (rd(w0) + rd(w1) + rd(w2));
    return P::cdbl(q.x) >= hx.v ? -e01 : 0;
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
            float const m8 = 8.0f * 1e-6f * (qmax + scene_scale);
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

template <class T, class P>
__global__ void __launch_bounds__(kRobBlock) k_robust_frac(const T* __restrict__ pos, int64_t n, Quant qz,
                                                           const RSeg<typename P::C>* __restrict__ seg, int64_t n_seg,
                                                           int tile, const int32_t* __restrict__ counts,
                                                           T* __restrict__ out, T* __restrict__ out_frac, int* flags)
{
    using Seg = RSeg<typename P::C>;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ int abort_cta;
    TilePipe<Seg> pipe;
    pipe.n_tiles = int((n_seg + tile - 1) / tile);
    pipe.single = pipe.n_tiles <= 1;
    pipe.buf[0] = reinterpret_cast<Seg*>(smem);
    pipe.buf[1] = pipe.buf[0] + (pipe.single ? 0 : tile);
    pipe.bar = bars;
    pipe.gseg = seg;
    pipe.n_seg = n_seg;
    pipe.tile = tile;
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
        for (int st = 0; st < pipe.n_tiles && n_seg > 0; ++st)
        {
            int const b = it & 1;
            if (!pipe.single || j == 0)
                if (!mbar_wait_bounded(&bars[b], unsigned((it >> 1) & 1), flags, 3))
                    abort_cta = 1;
            __syncthreads();
            if (abort_cta)
                return;
            Seg const* sb = pipe.buf[b];
            int const cnt = pipe.tile_count(st);
            for (int s = 0; s < cnt; ++s)
            {
                Seg const sgm = sb[s];
                half = __dadd_rn(half, __dmul_rn(sgm.w, robust_contrib<P>(q, sgm)));
            }
            if (!pipe.single)
            {
                __syncthreads();
                if (threadIdx.x == 0 && it + 2 < n_items)
                    pipe.issue(it + 2);
                ++it;
            }
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
    r->tri = r->seg = nullptr;
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
    AGWN_TRY_CUDA(cudaStreamSynchronize(st));
    return AGWN_OK;
}

template <class T, class P>
int robust_run(Context& ctx, const Robust& r, const T* d_pos, int64_t n, T* d_out, int32_t* d_counts, T* d_frac)
{
    using C = typename P::C;
    Quant qz{{r.center[0], r.center[1], r.center[2]}, r.scale};
    cudaStream_t const st = ctx.stream;
    if (r.n_tri == 0)
        AGWN_TRY_CUDA(cudaMemsetAsync(d_counts, 0, sizeof(int32_t) * n, st));
    else
    {
        Frame32 f;
        for (int k = 0; k < 9; ++k)
            f.r[k] = r.hier.frame[k];
        int const grid = int(std::min<int64_t>(div_up(n, kRobBlock), int64_t(ctx.sm_count) * 16));
        AGWN_TRY(ctx.launch_begin(AGWN_K_ROBUST));
        k_robust_count<T, P><<<grid, kRobBlock, 0, st>>>(
            static_cast<const BvhNode*>(r.hier.nodes.ptr), static_cast<const C*>(r.tri),
            static_cast<const float4*>(r.hier.leaf_uv.ptr), r.n_tri, float(r.hier.scale), f, qz, d_pos, n, d_counts,
            ctx.d_flags);
        AGWN_TRY(ctx.launch_end(AGWN_K_ROBUST));
    }
    using Seg = RSeg<C>;
    int const tile = int(std::max<int64_t>(1, std::min<int64_t>(ctx.seg_tile, r.n_seg)));
    int const n_tiles = int((r.n_seg + tile - 1) / tile);
    size_t const smem = size_t(n_tiles <= 1 ? 1 : 2) * tile * sizeof(Seg);
    auto kern = k_robust_frac<T, P>;
    AGWN_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int per_sm = 0;
    AGWN_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kRobBlock, smem));
    if (per_sm < 1)
        return fail(AGWN_ERR_UNSUPPORTED, "robust kernel does not fit on an SM");
    int64_t const n_qtiles = (n + kRobBlock - 1) / kRobBlock;
    int const grid = int(std::max<int64_t>(1, std::min<int64_t>(n_qtiles, int64_t(per_sm) * ctx.sm_count)));
    AGWN_TRY(ctx.launch_begin(AGWN_K_ROBUST));
    kern<<<grid, kRobBlock, smem, st>>>(d_pos, n, qz, static_cast<const Seg*>(r.seg), r.n_seg, tile, d_counts, d_out,
                                        d_frac, ctx.d_flags);
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
    if (h_out)
        AGWN_TRY_CUDA(cudaMemcpyAsync(out, dout, sizeof(T) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (h_cnt)
        AGWN_TRY_CUDA(cudaMemcpyAsync(out_counts, dcnt, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (h_fr)
        AGWN_TRY_CUDA(cudaMemcpyAsync(out_frac, dfr, sizeof(T) * n, cudaMemcpyDeviceToHost, ctx->stream));
    bool const sync = dpos != positions || h_out || h_cnt || h_fr;
    return sync ? ctx->check_flags() : AGWN_OK;
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
} // extern "C"
