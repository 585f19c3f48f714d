// CPU oracle for the batch generalized-winding-number path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in plain C++, the algorithms of
// the antipodal library's batch GWN functions so that the CUDA path can be
// checked against them.  Only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg load it, and only as the checker or the timed CPU baseline.
// The product library (antipodal_gb300) never links, loads or calls it.
//
// Every function names the reference location it follows.  Paths are relative
// to the antipodal project root.  The library is compiled with
// -ffp-contract=off so that each product and sum is rounded on its own, which is
// what the reference's default x86-64 build (no -march, no FMA) does; with the
// same operation order the restatement reproduces the reference's doubles.
//
// Threading: every batch function runs an OpenMP loop with dynamic blocks of
// 256 indices, the same work split as the reference's PoolDispatcher
// (src/antipodal/dispatcher/dispatcher_threadpool.hh:51, :112).

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <utility>
#include <vector>

#include <omp.h>

namespace orc
{
template <class T>
struct v3
{
    T x, y, z;
};

template <class T>
constexpr T kPi = T(3.141592653589793238462643383279502884L);

template <class T>
inline v3<T> sub(v3<T> a, v3<T> b)
{
    return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <class T>
inline v3<T> neg(v3<T> a)
{
    return {-a.x, -a.y, -a.z};
}
// dot / cross / length evaluate left to right like src/antipodal/math/common.hh:73-96.
template <class T>
inline T dot(v3<T> a, v3<T> b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <class T>
inline v3<T> cross(v3<T> a, v3<T> b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T>
inline T norm(v3<T> a)
{
    return std::sqrt(dot(a, a));
}
template <class T>
inline v3<T> ld3(T const* p)
{
    return {p[0], p[1], p[2]};
}

// ---------------------------------------------------------------------------------------------------------------
// Mesh fractional term
// ---------------------------------------------------------------------------------------------------------------

// Half the signed solid angle of the spherical triangle (x1, v0, v1), unnormalised Van Oosterom-Strackee form.
// Follows src/antipodal/math/common.hh:181-189.
template <class T>
inline T vos_half(v3<T> x1, v3<T> v0, v3<T> v1)
{
    T const l0 = norm(v0);
    T const l1 = norm(v1);
    T const num = dot(x1, cross(v0, v1));
    T const den = l0 * l1 + l1 * dot(x1, v0) + l0 * dot(x1, v1) + dot(v0, v1);
    return std::atan2(num, den);
}

// Fractional GWN at one point: sum of weight * half-area over the boundary, divided by 2 pi.
// Follows src/antipodal/gwn_mesh.hh:34-46.  A boundary segment is 7 scalars: pos0, pos1, weight
// (the layout of weighted_segment3<T>, src/antipodal/math/common.hh:60-65).
template <class T>
inline T frac_single(v3<T> p, v3<T> x0, T const* seg, int64_t n_seg)
{
    v3<T> const x1 = neg(x0);
    T area = T(0);
    for (int64_t s = 0; s < n_seg; ++s)
    {
        T const* w = seg + 7 * s;
        v3<T> const v0 = sub(ld3(w), p);
        v3<T> const v1 = sub(ld3(w + 3), p);
        area += w[6] * vos_half(x1, v0, v1);
    }
    return area / (T(2) * kPi<T>);
}

// Signed Moller-Trumbore crossing count of the ray (p, dir) over a triangle list.
// Follows NaiveIntersector::signed_intersection_count, src/antipodal/intersector/intersector.hh:61-100,
// including its early rejections, so edge/vertex hits are double counted exactly as there.
template <class T>
inline int naive_count(v3<T> p, v3<T> dir, T const* verts, int32_t const* idx, int64_t n_tri)
{
    int sum = 0;
    for (int64_t t = 0; t < n_tri; ++t)
    {
        v3<T> const a = ld3(verts + 3 * int64_t(idx[3 * t + 0]));
        v3<T> const b = ld3(verts + 3 * int64_t(idx[3 * t + 1]));
        v3<T> const c = ld3(verts + 3 * int64_t(idx[3 * t + 2]));
        v3<T> const e1 = sub(b, a);
        v3<T> const e2 = sub(c, a);
        v3<T> const h = cross(dir, e2);
        T const det = dot(e1, h);
        if (det == T(0))
            continue;
        T const inv_det = T(1) / det;
        v3<T> const s = sub(p, a);
        T const u = inv_det * dot(s, h);
        if (u < T(0) || u > T(1))
            continue;
        v3<T> const q = cross(s, e1);
        T const v = inv_det * dot(dir, q);
        if (v < T(0) || u + v > T(1))
            continue;
        T const t_hit = inv_det * dot(e2, q);
        if (t_hit < T(0))
            continue;
        v3<T> const ng = cross(e1, e2);
        sum += dot(ng, dir) > T(0) ? +1 : -1;
    }
    return sum;
}

// Brute-force triangle solid-angle GWN, the reference test suite's independent oracle
// (test/gwn_baseline.hh:20-43).
template <class T>
inline T gwn_baseline(v3<T> p, T const* verts, int32_t const* idx, int64_t n_tri)
{
    T solid = T(0);
    for (int64_t i = 0; i < n_tri; ++i)
    {
        v3<T> a = sub(ld3(verts + 3 * int64_t(idx[3 * i + 0])), p);
        v3<T> b = sub(ld3(verts + 3 * int64_t(idx[3 * i + 1])), p);
        v3<T> c = sub(ld3(verts + 3 * int64_t(idx[3 * i + 2])), p);
        T const la = norm(a), lb = norm(b), lc = norm(c);
        a = {a.x / la, a.y / la, a.z / la};
        b = {b.x / lb, b.y / lb, b.z / lb};
        c = {c.x / lc, c.y / lc, c.z / lc};
        T const num = dot(a, cross(b, c));
        T const den = T(1) + dot(a, b) + dot(b, c) + dot(c, a);
        solid += T(2) * std::atan2(num, den);
    }
    return solid / (T(4) * kPi<T>);
}

// Open boundary of a triangle mesh: net +1 per min->max traversal and -1 per max->min traversal of each
// undirected edge; zero-sum edges are dropped and the survivors are emitted with positive weight, flipped
// when the net count is negative.  Follows build_boundary_segments, src/antipodal/math/common.hh:123-174.
// The reference emits in hash-map order; this restatement sorts by (lo, hi) so the order is reproducible.
template <class T>
inline std::vector<T> boundary_segments(T const* verts, int32_t const* idx, int64_t n_tri)
{
    std::vector<std::pair<uint64_t, int>> edges;
    edges.reserve(size_t(3 * n_tri));
    for (int64_t t = 0; t < n_tri; ++t)
    {
        for (int e = 0; e < 3; ++e)
        {
            int32_t const u = idx[3 * t + e];
            int32_t const v = idx[3 * t + (e + 1) % 3];
            uint32_t const lo = uint32_t(std::min(u, v));
            uint32_t const hi = uint32_t(std::max(u, v));
            edges.push_back({(uint64_t(lo) << 32) | hi, u < v ? +1 : -1});
        }
    }
    std::sort(edges.begin(), edges.end(), [](auto const& a, auto const& b) { return a.first < b.first; });
    std::vector<T> out;
    for (size_t i = 0; i < edges.size();)
    {
        size_t j = i;
        int sum = 0;
        while (j < edges.size() && edges[j].first == edges[i].first)
            sum += edges[j++].second;
        if (sum != 0)
        {
            int32_t const lo = int32_t(edges[i].first >> 32);
            int32_t const hi = int32_t(edges[i].first & 0xffffffffu);
            T const* a = verts + 3 * int64_t(lo);
            T const* b = verts + 3 * int64_t(hi);
            T const* first = sum > 0 ? a : b;
            T const* second = sum > 0 ? b : a;
            out.insert(out.end(), first, first + 3);
            out.insert(out.end(), second, second + 3);
            out.push_back(T(sum > 0 ? sum : -sum));
        }
        i = j;
    }
    return out;
}

// ---------------------------------------------------------------------------------------------------------------
// Exact predicates and the robust evaluator
// ---------------------------------------------------------------------------------------------------------------

using i64 = int64_t;
__extension__ typedef __int128 i128;

template <class C>
struct wide;
template <>
struct wide<int32_t>
{
    using type = i64;
};
template <>
struct wide<int64_t>
{
    using type = i128;
};
template <>
struct wide<double>
{
    using type = double;
};
template <class C>
using wide_t = typename wide<C>::type;

template <class C>
inline wide_t<C> mulw(C a, C b)
{
    return wide_t<C>(a) * wide_t<C>(b);
}

// Knuth's two-sum: s + e == a + b exactly.  src/antipodal/math/robust_predicates.hh:227-233.
inline void two_sum(double a, double b, double& s, double& e)
{
    s = a + b;
    double const bv = s - a;
    double const av = s - bv;
    e = (a - av) + (b - bv);
}

// Exact sign of sum_i a[i]*b[i] (six products) through an fma-split nonoverlapping expansion.
// src/antipodal/math/robust_predicates.hh:238-264.
inline int sign_of_product_sum(double const (&a)[6], double const (&b)[6])
{
    double e[12];
    int n = 0;
    auto grow = [&](double v)
    {
        for (int i = 0; i < n; ++i)
        {
            double s, r;
            two_sum(v, e[i], s, r);
            e[i] = r;
            v = s;
        }
        e[n++] = v;
    };
    for (int i = 0; i < 6; ++i)
    {
        double const p = a[i] * b[i];
        grow(std::fma(a[i], b[i], -p));
        grow(p);
    }
    for (int i = n - 1; i >= 0; --i)
        if (e[i] != 0)
            return e[i] > 0 ? 1 : -1;
    return 0;
}

// 2x2 determinant of (q - q0, q1 - q0) in the (y, z) plane: exact for integer coordinates; for doubles the
// value has the exact sign and a magnitude of at least DBL_MIN when nonzero.
// src/antipodal/math/robust_predicates.hh:273-308.
template <class C>
inline wide_t<C> edge_det(v3<C> q, v3<C> q0, v3<C> q1)
{
    if constexpr (std::is_same_v<C, double>)
    {
        double const p1 = (q.y - q0.y) * (q0.z - q1.z);
        double const p2 = (q.z - q0.z) * (q1.y - q0.y);
        double const det = p1 + p2;
        constexpr double eps = std::numeric_limits<double>::epsilon() / 2;
        constexpr double bound = (3.0 + 16.0 * eps) * eps;
        double const mag = std::abs(p1) + std::abs(p2);
        if (std::abs(det) > bound * mag)
            return det;
        if (mag == 0)
            return 0.0;
        double const a[6] = {q.y, -q.y, q0.y, q.z, -q.z, -q0.z};
        double const b[6] = {q0.z, q1.z, q1.z, q1.y, q0.y, q1.y};
        int const s = sign_of_product_sum(a, b);
        if (s == 0)
            return 0.0;
        return std::copysign(std::max(std::abs(det), std::numeric_limits<double>::min()), double(s));
    }
    else
    {
        return mulw<C>(q.y - q0.y, q0.z - q1.z) + mulw<C>(q.z - q0.z, q1.y - q0.y);
    }
}

// Side of the directed projected edge, with the (eps2 on y, eps3 on z) tie-break.
// src/antipodal/math/robust_predicates.hh:314-331.
template <class C>
inline int edge_sign(v3<C> q, v3<C> q0, v3<C> q1)
{
    wide_t<C> const t = edge_det(q, q0, q1);
    if (t != 0)
        return t > 0 ? 1 : -1;
    if (q0.z != q1.z)
        return q0.z > q1.z ? 1 : -1;
    if (q1.y != q0.y)
        return q1.y > q0.y ? 1 : -1;
    return 0;
}

// atan2 numerator with exact sign (== -edge_det).  src/antipodal/math/robust_predicates.hh:339-356.
template <class C>
inline wide_t<C> atan2_num(v3<C> q, v3<C> q0, v3<C> q1)
{
    v3<C> const v0 = sub(q0, q);
    v3<C> const v1 = sub(q1, q);
    if constexpr (std::is_same_v<C, double>)
    {
        double const t = edge_det(q, q0, q1);
        if (t == 0)
            return 0.0;
        double const num = v0.z * v1.y - v0.y * v1.z;
        return std::copysign(std::max(std::abs(num), std::numeric_limits<double>::min()), -t);
    }
    else
    {
        return mulw<C>(v0.z, v1.y) - mulw<C>(v0.y, v1.z);
    }
}

// a.y*b.y + a.z*b.z, exact for integer coordinates until the conversion.  robust_predicates.hh:368-375.
template <class C>
inline double dot_yz(v3<C> a, v3<C> b)
{
    if constexpr (std::is_same_v<C, double>)
        return a.y * b.y + a.z * b.z;
    else
        return double(mulw<C>(a.y, b.y) + mulw<C>(a.z, b.z));
}

struct tri_proj
{
    int sign = 0;
    double w0 = 0, w1 = 0, w2 = 0;
};

// robust_predicates.hh:390-402.
template <class C>
inline tri_proj project_into_tri(v3<C> q, v3<C> q0, v3<C> q1, v3<C> q2)
{
    int const e01 = edge_sign(q, q0, q1);
    int const e12 = edge_sign(q, q1, q2);
    int const e20 = edge_sign(q, q2, q0);
    if (e01 == 0 || e01 != e12 || e01 != e20)
        return {};
    return {e01, double(edge_det(q, q1, q2)), double(edge_det(q, q2, q0)), double(edge_det(q, q0, q1))};
}

// Robust mesh GWN along the fixed -x ray.  Follows RobustMeshGwn, src/antipodal/gwn_mesh_robust.hh:170-424:
// quantizer (:334-378), swapped boundary (:198-206), fractional (:264-325) and the integer term, whose
// Embree traversal is replaced by a scan of every triangle through the same occluded test (:122-145).
// The Embree boxes only cull, conservatively (:82-90), so the scan gives the same count.
// GRID_BITS == 0 selects exact_float (double coordinates, no grid).
template <class T, class C, int GRID_BITS>
struct robust_mesh
{
    static constexpr bool grid = GRID_BITS > 0;
    v3<double> center{0, 0, 0};
    double scale = 1.0;
    std::vector<std::array<v3<C>, 3>> tri;
    struct qseg
    {
        v3<C> p0, p1;
        double w;
    };
    std::vector<qseg> seg;

    v3<C> quantize(v3<double> p) const
    {
        if constexpr (grid)
        {
            static constexpr double max_q = double(i64(1) << (GRID_BITS + 10));
            v3<double> const q = {(p.x - center.x) * scale, (p.y - center.y) * scale, (p.z - center.z) * scale};
            auto r = [](double v) { return C(std::llround(std::clamp(v, -max_q, max_q))); };
            return {r(q.x), r(q.y), r(q.z)};
        }
        else
        {
            return p;
        }
    }

    robust_mesh(T const* verts, int64_t nv, int32_t const* idx, int64_t n_tri, T const* segs, int64_t n_seg)
    {
        auto to_d = [](T const* p) { return v3<double>{double(p[0]), double(p[1]), double(p[2])}; };
        if constexpr (grid)
        {
            if (nv > 0)
            {
                v3<double> mn = to_d(verts), mx = mn;
                for (int64_t i = 0; i < nv; ++i)
                {
                    v3<double> const d = to_d(verts + 3 * i);
                    mn = {std::min(mn.x, d.x), std::min(mn.y, d.y), std::min(mn.z, d.z)};
                    mx = {std::max(mx.x, d.x), std::max(mx.y, d.y), std::max(mx.z, d.z)};
                }
                v3<double> const ext = sub(mx, mn);
                center = {mn.x + ext.x * 0.5, mn.y + ext.y * 0.5, mn.z + ext.z * 0.5};
                double const half = 0.5 * std::max({ext.x, ext.y, ext.z});
                constexpr double max_coord = double((i64(1) << GRID_BITS) - 1);
                scale = half > 0.0 ? max_coord / half : 1.0;
            }
        }
        tri.reserve(size_t(n_tri));
        for (int64_t t = 0; t < n_tri; ++t)
            tri.push_back({quantize(to_d(verts + 3 * int64_t(idx[3 * t + 0]))),
                           quantize(to_d(verts + 3 * int64_t(idx[3 * t + 1]))),
                           quantize(to_d(verts + 3 * int64_t(idx[3 * t + 2])))});
        seg.reserve(size_t(n_seg));
        for (int64_t s = 0; s < n_seg; ++s)
        {
            T const* w = segs + 7 * s;
            seg.push_back({quantize(to_d(w + 3)), quantize(to_d(w)), double(w[6])});
        }
    }

    int count(v3<C> qi) const
    {
        int sum = 0;
        for (auto const& t : tri)
        {
            tri_proj const h = project_into_tri(qi, t[0], t[1], t[2]);
            if (h.sign == 0)
                continue;
            double const hit_x = (h.w0 * double(t[0].x) + h.w1 * double(t[1].x) + h.w2 * double(t[2].x))
                               / (h.w0 + h.w1 + h.w2);
            if (double(qi.x) >= hit_x)
                sum += -h.sign;
        }
        return sum;
    }

    static double l_plus_x(v3<C> v, double l)
    {
        if (v.x >= 0)
            return l + double(v.x);
        return dot_yz(v, v) / (l - double(v.x));
    }

    T fractional(v3<C> qi) const
    {
        constexpr double f_norm = 2.0 / (4.0 * kPi<double>);
        constexpr double pi = kPi<double>;
        double half_area = 0.0;
        for (auto const& s : seg)
        {
            v3<C> const v0 = sub(s.p0, qi);
            v3<C> const v1 = sub(s.p1, qi);
            v3<double> const d0{double(v0.x), double(v0.y), double(v0.z)};
            v3<double> const d1{double(v1.x), double(v1.y), double(v1.z)};
            double const l0 = norm(d0);
            double const l1 = norm(d1);
            wide_t<C> const num = atan2_num(qi, s.p0, s.p1);
            double const yz = dot_yz(v0, v1);
            double const den = l_plus_x(v0, l0) * l_plus_x(v1, l1) + yz;
            double contrib;
            if (num != 0)
                contrib = std::atan2(double(num), den);
            else if (v0.y == 0 && v0.z == 0 && v0.x < 0 && (v1.y != 0 || v1.z != 0))
                contrib = v1.z != 0 ? std::atan2(double(v1.z), -double(v1.y)) : (v1.y > 0 ? -pi : 0.0);
            else if (v1.y == 0 && v1.z == 0 && v1.x < 0 && (v0.y != 0 || v0.z != 0))
                contrib = v0.z != 0 ? std::atan2(-double(v0.z), -double(v0.y)) : (v0.y > 0 ? pi : 0.0);
            else
            {
                int const sg = -edge_sign(qi, s.p0, s.p1);
                contrib = den < 0.0 ? double(sg) * pi : 0.0;
            }
            half_area += s.w * contrib;
        }
        return T(half_area * f_norm);
    }
};

// ---------------------------------------------------------------------------------------------------------------
// Parametric fractional term with adaptive G7-K15
// ---------------------------------------------------------------------------------------------------------------

// G7-K15 abscissae and weights: the published Gauss-Kronrod 15-point constants at the 16 decimals the
// reference carries (src/antipodal/math/integrate_gk15.hh:13-36), so that the restated integrator rounds
// exactly like the reference one.
namespace gk
{
constexpr double x[8] = {0.0,
                         0.9914553711208126,
                         0.9491079123427585,
                         0.8648644233597691,
                         0.7415311855993945,
                         0.5860872354676911,
                         0.4058451513773972,
                         0.2077849550078985};
constexpr double wk[8] = {0.2094821410847278, 0.0229353220105292, 0.0630920926299786, 0.1047900103222502,
                          0.1406532597155259, 0.1690047266392679, 0.1903505780647854, 0.2044329400752989};
constexpr double wg_center = 0.4179591836734694;
constexpr double wg2 = 0.1294849661688697;
constexpr double wg4 = 0.2797053914892767;
constexpr double wg6 = 0.3818300505051189;
} // namespace gk

struct integ_stats
{
    double err = 0;
    int leaves = 0;
    int max_depth = 0;
};

// Adaptive GK15 in evaluate mode: accept at depth >= max_depth, or at depth >= min_depth with
// |Ik - Ig| <= local tolerance; otherwise halve the tolerance and return left + right.
// Follows integrate_gk15<evaluate>, src/antipodal/math/integrate_gk15.hh:63-276 (node order :155-183,
// sums :187-217, acceptance :219-233).
template <class F>
double gk15_node(F const& f, double a, double b, double tol, int depth, int min_depth, int max_depth,
                 integ_stats& st)
{
    double const c = (a + b) * 0.5;
    double const h = (b - a) * 0.5;
    double fm[8], fp[8];
    double const f0 = f(c);
    for (int k = 1; k <= 7; ++k)
    {
        double const dx = h * gk::x[k];
        fm[k] = f(c - dx);
        fp[k] = f(c + dx);
    }
    double ig = gk::wg_center * f0;
    double ik = gk::wk[0] * f0;
    ik = ik + gk::wk[1] * (fm[1] + fp[1]);
    {
        double const s = fm[2] + fp[2];
        ik = ik + gk::wk[2] * s;
        ig = ig + gk::wg2 * s;
    }
    ik = ik + gk::wk[3] * (fm[3] + fp[3]);
    {
        double const s = fm[4] + fp[4];
        ik = ik + gk::wk[4] * s;
        ig = ig + gk::wg4 * s;
    }
    ik = ik + gk::wk[5] * (fm[5] + fp[5]);
    {
        double const s = fm[6] + fp[6];
        ik = ik + gk::wk[6] * s;
        ig = ig + gk::wg6 * s;
    }
    ik = ik + gk::wk[7] * (fm[7] + fp[7]);
    ig = ig * h;
    ik = ik * h;
    double const err = std::abs(ik - ig);
    if (depth >= max_depth || (depth >= min_depth && err <= tol))
    {
        st.err = st.err + err;
        st.leaves += 1;
        st.max_depth = std::max(st.max_depth, depth);
        return ik;
    }
    double const half = tol * 0.5;
    double const left = gk15_node(f, a, c, half, depth + 1, min_depth, max_depth, st);
    double const right = gk15_node(f, c, b, half, depth + 1, min_depth, max_depth, st);
    return left + right;
}

template <class F>
double gk15(F const& f, double a, double b, int min_depth, int max_depth, double tol, integ_stats& st)
{
    st = {};
    if (a == b)
        return 0.0;
    return gk15_node(f, a, b, tol, 0, min_depth, max_depth, st);
}

// Dual number (value, derivative) with the product / sum rules of fwd_diff, src/antipodal/math/fwd_diff.hh:45-92
// (operator* at :198-201 of that file's arithmetic block: d = a.d*b.v + a.v*b.d).
struct dual
{
    double v, d;
};
inline dual dmul(dual a, dual b)
{
    return {a.v * b.v, a.d * b.v + a.v * b.d};
}
inline dual smul(double s, dual b)
{
    return {s * b.v, s * b.d};
}

// Cubic Bezier curve point and tangent: Bernstein basis in dual numbers, summed c0*b0 + c1*b1 + c2*b2 + c3*b3.
// The reference ships no curve type (README.md:300-305); this is the project's own curve, evaluated with the
// same dual-number rules as the project's curve functor in oracle/ref_driver.cc.
inline void bezier3(double const* c, double t, v3<double>& pos, v3<double>& tan)
{
    dual const tt{t, 1.0};
    dual const u{1.0 - t, -1.0};
    dual const b0 = dmul(dmul(u, u), u);
    dual const b1 = dmul(dmul(smul(3.0, u), u), tt);
    dual const b2 = dmul(dmul(smul(3.0, u), tt), tt);
    dual const b3 = dmul(dmul(tt, tt), tt);
    double const* c0 = c;
    double const* c1 = c + 3;
    double const* c2 = c + 6;
    double const* c3 = c + 9;
    for (int k = 0; k < 3; ++k)
    {
        double const pv = c0[k] * b0.v + c1[k] * b1.v + c2[k] * b2.v + c3[k] * b3.v;
        double const pd = c0[k] * b0.d + c1[k] * b1.d + c2[k] * b2.d + c3[k] * b3.d;
        (&pos.x)[k] = pv;
        (&tan.x)[k] = pd;
    }
}

// w(t) - d_eta(t) for one boundary curve.  Follows detail::parametric_gwn_integrand,
// src/antipodal/gwn_parametric.hh:73-103, with normalize_fd from src/antipodal/math/fwd_diff.hh:497-532.
inline double param_integrand(double const* ctrl, v3<double> p, v3<double> x0, double t)
{
    v3<double> const x1 = neg(x0);
    v3<double> phi, dphi;
    bezier3(ctrl, t, phi, dphi);
    v3<double> const r = sub(phi, p);
    // normalize_fd
    double const q = r.x * r.x + r.y * r.y + r.z * r.z;
    double const q1 = 2.0 * (r.x * dphi.x + r.y * dphi.y + r.z * dphi.z);
    double const s = std::sqrt(q);
    double const inv_s = 1.0 / s;
    double const s1 = q1 * (0.5 * inv_s);
    v3<double> G, Gp;
    for (int k = 0; k < 3; ++k)
    {
        double const vi = (&r.x)[k];
        double const dvi = (&dphi.x)[k];
        double const xi = vi * inv_s;
        (&G.x)[k] = xi;
        (&Gp.x)[k] = (dvi - xi * s1) * inv_s;
    }
    double const a = dot(x0, G);
    double const ap = dot(x0, Gp);
    v3<double> const X = sub(x0, v3<double>{G.x * a, G.y * a, G.z * a});
    v3<double> const Xp = sub(v3<double>{G.x * -ap, G.y * -ap, G.z * -ap}, v3<double>{Gp.x * a, Gp.y * a, Gp.z * a});
    double const d_eta = dot(G, cross(X, Xp)) / dot(X, X);
    double const b = dot(x1, G);
    double const bp = dot(x1, Gp);
    v3<double> const v = sub(G, v3<double>{x1.x * b, x1.y * b, x1.z * b});
    v3<double> const vp = sub(Gp, v3<double>{x1.x * bp, x1.y * bp, x1.z * bp});
    double const w = dot(x1, cross(v, vp)) / dot(v, v);
    return w - d_eta;
}

template <class T>
inline v3<T> ld3i(T const* p, int64_t i)
{
    return ld3(p + 3 * i);
}
} // namespace orc

using namespace orc;

// ---------------------------------------------------------------------------------------------------------------
// C ABI (ctypes)
// ---------------------------------------------------------------------------------------------------------------

static int nthreads(int t)
{
    return t > 0 ? t : omp_get_max_threads();
}

extern "C"
{
int orc_abi_version()
{
    return 3;
}

double orc_vos_half_f64(double const* x1, double const* v0, double const* v1)
{
    return vos_half(ld3(x1), ld3(v0), ld3(v1));
}
float orc_vos_half_f32(float const* x1, float const* v0, float const* v1)
{
    return vos_half(ld3(x1), ld3(v0), ld3(v1));
}

#define ORC_FRAC(SUF, T)                                                                                     \
    void orc_frac_batch_##SUF(T const* pos, int64_t n, T* out, T const* x0, T const* seg, int64_t n_seg,      \
                              int threads)                                                                   \
    {                                                                                                        \
        v3<T> const x = ld3(x0);                                                                             \
        _Pragma("omp parallel for schedule(dynamic, 256) num_threads(nthreads(threads))")                     \
        for (int64_t i = 0; i < n; ++i)                                                                      \
            out[i] = frac_single(ld3i(pos, i), x, seg, n_seg);                                               \
    }                                                                                                        \
    void orc_int_naive_##SUF(T const* pos, int64_t n, int32_t* out, T const* dir, T const* verts, int64_t nv,  \
                             int32_t const* idx, int64_t n_idx, int threads)                                 \
    {                                                                                                        \
        (void)nv;                                                                                            \
        v3<T> const d = ld3(dir);                                                                            \
        _Pragma("omp parallel for schedule(dynamic, 256) num_threads(nthreads(threads))")                     \
        for (int64_t i = 0; i < n; ++i)                                                                      \
            out[i] = naive_count(ld3i(pos, i), d, verts, idx, n_idx / 3);                                    \
    }                                                                                                        \
    void orc_full_naive_##SUF(T const* pos, int64_t n, T* out, T const* x0, T const* verts, int64_t nv,       \
                              int32_t const* idx, int64_t n_idx, T const* seg, int64_t n_seg, int threads)   \
    {                                                                                                        \
        (void)nv;                                                                                            \
        v3<T> const x = ld3(x0);                                                                             \
        _Pragma("omp parallel for schedule(dynamic, 256) num_threads(nthreads(threads))")                     \
        for (int64_t i = 0; i < n; ++i)                                                                      \
        {                                                                                                    \
            v3<T> const p = ld3i(pos, i);                                                                    \
            T const fr = frac_single(p, x, seg, n_seg);                                                      \
            int const ic = naive_count(p, x, verts, idx, n_idx / 3);                                         \
            out[i] = fr + T(ic);                                                                             \
        }                                                                                                    \
    }                                                                                                        \
    void orc_gwn_baseline_##SUF(T const* pos, int64_t n, T* out, T const* verts, int64_t nv,                  \
                                int32_t const* idx, int64_t n_idx, int threads)                              \
    {                                                                                                        \
        (void)nv;                                                                                            \
        _Pragma("omp parallel for schedule(dynamic, 256) num_threads(nthreads(threads))")                     \
        for (int64_t i = 0; i < n; ++i)                                                                      \
            out[i] = gwn_baseline(ld3i(pos, i), verts, idx, n_idx / 3);                                      \
    }                                                                                                        \
    int64_t orc_boundary_##SUF(T const* verts, int64_t nv, int32_t const* idx, int64_t n_idx, T* out,         \
                               int64_t cap)                                                                  \
    {                                                                                                        \
        (void)nv;                                                                                            \
        std::vector<T> const s = boundary_segments(verts, idx, n_idx / 3);                                   \
        int64_t const cnt = int64_t(s.size() / 7);                                                           \
        if (out)                                                                                             \
            std::memcpy(out, s.data(), sizeof(T) * size_t(7 * std::min(cnt, cap)));                          \
        return cnt;                                                                                          \
    }

ORC_FRAC(f64, double)
ORC_FRAC(f32, float)
} // extern "C"

// Robust evaluator.  scalar_bytes: 4 (float queries/geometry) or 8 (double).  policy: 0 int64_grid,
// 1 int128_grid, 2 exact_float (robust_predicates.hh:186-215).  Writes the full GWN, and optionally the
// integer count and the fractional term, per query.
template <class T, class C, int BITS>
static void robust_run(void const* verts, int64_t nv, int32_t const* idx, int64_t n_idx, void const* seg,
                       int64_t n_seg, void const* pos, int64_t n, void* out, int32_t* out_count, void* out_frac,
                       int threads)
{
    robust_mesh<T, C, BITS> const m(static_cast<T const*>(verts), nv, idx, n_idx / 3, static_cast<T const*>(seg),
                                    n_seg);
    T const* p = static_cast<T const*>(pos);
    T* o = static_cast<T*>(out);
    T* of = static_cast<T*>(out_frac);
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads(threads))
    for (int64_t i = 0; i < n; ++i)
    {
        v3<C> const qi = m.quantize(v3<double>{double(p[3 * i]), double(p[3 * i + 1]), double(p[3 * i + 2])});
        T const fr = m.fractional(qi);
        int const c = m.count(qi);
        if (o)
            o[i] = fr + static_cast<T>(c);
        if (out_count)
            out_count[i] = c;
        if (of)
            of[i] = fr;
    }
}

extern "C"
{
int orc_robust_eval(int scalar_bytes, int policy, void const* verts, int64_t nv, int32_t const* idx, int64_t n_idx,
                    void const* seg, int64_t n_seg, void const* pos, int64_t n, void* out, int32_t* out_count,
                    void* out_frac, int threads)
{
#define ORC_ROBUST(T)                                                                                          \
    switch (policy)                                                                                            \
    {                                                                                                          \
    case 0:                                                                                                    \
        robust_run<T, int32_t, 20>(verts, nv, idx, n_idx, seg, n_seg, pos, n, out, out_count, out_frac, threads); \
        return 0;                                                                                              \
    case 1:                                                                                                    \
        robust_run<T, int64_t, 50>(verts, nv, idx, n_idx, seg, n_seg, pos, n, out, out_count, out_frac, threads); \
        return 0;                                                                                              \
    case 2:                                                                                                    \
        robust_run<T, double, 0>(verts, nv, idx, n_idx, seg, n_seg, pos, n, out, out_count, out_frac, threads);  \
        return 0;                                                                                              \
    default:                                                                                                   \
        return 1;                                                                                              \
    }
    if (scalar_bytes == 4)
    {
        ORC_ROBUST(float)
    }
    if (scalar_bytes == 8)
    {
        ORC_ROBUST(double)
    }
    return 1;
#undef ORC_ROBUST
}

// Predicates over batches, for pinning against the reference's predicate tests.  policy 0: int32 coords,
// 1: int64 coords, 2: double coords.  q, q0, q1, q2 hold n points each (3 values per point).
// Outputs: edge_sign(q,q0,q1), atan2_num(q,q0,q1) as a double, project_into_tri(q,q0,q1,q2).sign.
int orc_predicates(int policy, void const* q, void const* q0, void const* q1, void const* q2, int64_t n,
                   int32_t* out_edge_sign, double* out_num, int32_t* out_inside)
{
    auto run = [&](auto tag)
    {
        using C = decltype(tag);
        C const* a = static_cast<C const*>(q);
        C const* b = static_cast<C const*>(q0);
        C const* c = static_cast<C const*>(q1);
        C const* d = static_cast<C const*>(q2);
        for (int64_t i = 0; i < n; ++i)
        {
            v3<C> const qq = ld3i(a, i), p0 = ld3i(b, i), p1 = ld3i(c, i), p2 = ld3i(d, i);
            out_edge_sign[i] = edge_sign(qq, p0, p1);
            out_num[i] = double(atan2_num(qq, p0, p1));
            out_inside[i] = project_into_tri(qq, p0, p1, p2).sign;
        }
    };
    if (policy == 0)
        run(int32_t{});
    else if (policy == 1)
        run(int64_t{});
    else if (policy == 2)
        run(double{});
    else
        return 1;
    return 0;
}

// project_into_tri(q, q0, q1, q2) weights w0, w1, w2 per row (robust_predicates.hh:391-402).
int orc_predicate_weights(int policy, void const* q, void const* q0, void const* q1, void const* q2, int64_t n,
                          double* out_weights)
{
    auto run = [&](auto tag)
    {
        using C = decltype(tag);
        C const* a = static_cast<C const*>(q);
        C const* b = static_cast<C const*>(q0);
        C const* c = static_cast<C const*>(q1);
        C const* d = static_cast<C const*>(q2);
        for (int64_t i = 0; i < n; ++i)
        {
            tri_proj const h = project_into_tri(ld3i(a, i), ld3i(b, i), ld3i(c, i), ld3i(d, i));
            out_weights[3 * i] = h.w0;
            out_weights[3 * i + 1] = h.w1;
            out_weights[3 * i + 2] = h.w2;
        }
    };
    if (policy == 0)
        run(int32_t{});
    else if (policy == 1)
        run(int64_t{});
    else if (policy == 2)
        run(double{});
    else
        return 1;
    return 0;
}

// Parametric fractional GWN over cubic Bezier boundary curves (12 doubles per curve: 4 control points).
// Follows eval_gwnr_parametric_single_fractional / _batch_fractional, src/antipodal/gwn_parametric.hh:130-186,
// with IntegratorGK15.  Optional per-(query, curve) outputs, row-major [n][n_curves]: accepted leaves and the
// deepest accepted level.
void orc_param_frac_bezier3_f64(double const* pos, int64_t n, double* out, double const* x0, double const* ctrl,
                                int64_t n_curves, int min_depth, int max_depth, double tol, int32_t* out_leaves,
                                int32_t* out_depth, int threads)
{
    v3<double> const x = ld3(x0);
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads(threads))
    for (int64_t i = 0; i < n; ++i)
    {
        v3<double> const p = ld3i(pos, i);
        double sum = 0.0;
        for (int64_t c = 0; c < n_curves; ++c)
        {
            double const* cc = ctrl + 12 * c;
            integ_stats st;
            sum += gk15([&](double t) { return param_integrand(cc, p, x, t); }, 0.0, 1.0, min_depth, max_depth, tol,
                        st);
            if (out_leaves)
                out_leaves[i * n_curves + c] = st.leaves;
            if (out_depth)
                out_depth[i * n_curves + c] = st.max_depth;
        }
        out[i] = sum / (4.0 * kPi<double>);
    }
}

// The integrand alone, for point checks.
double orc_param_integrand_bezier3(double const* ctrl, double const* p, double const* x0, double t)
{
    return param_integrand(ctrl, ld3(p), ld3(x0), t);
}

// GK15 on closed-form integrands (for the known-answer tests of src/antipodal/math/integrate_gk15.hh):
// fn 0: sin t, 1: t^2, 2: exp t, 3: t, 4: sin(30 t).
double orc_gk15_known(int fn, double a, double b, int min_depth, int max_depth, double tol, double* err, int* leaves)
{
    integ_stats st;
    auto f = [fn](double t)
    {
        switch (fn)
        {
        case 0:
            return std::sin(t);
        case 1:
            return t * t;
        case 2:
            return std::exp(t);
        case 3:
            return t;
        default:
            return std::sin(t * 30.0);
        }
    };
    double const r = gk15(f, a, b, min_depth, max_depth, tol, st);
    if (err)
        *err = st.err;
    if (leaves)
        *leaves = st.leaves;
    return r;
}
} // extern "C"

// ---------------------------------------------------------------------------------------------------------------
// Learned GK15 depth proposal: features and the MLP's loss and gradient (no reference counterpart).  The checker
// for the device training kernels: the same network in double precision, rounding to BF16 exactly where the
// device feeds a tensor-core product (inputs, weights, hidden activations, output gradients) and nowhere else.
// ---------------------------------------------------------------------------------------------------------------
namespace orc
{
namespace mlp
{
constexpr int F = 12, FP = 16, H = 64, C = 16;
constexpr int oW1 = 0, oB1 = oW1 + H * FP, oW2 = oB1 + H, oB2 = oW2 + H * H, oW3 = oB2 + H, oB3 = oW3 + C * H,
              n_params = oB3 + C;

// float -> bfloat16 -> float, round to nearest even
inline double bf16(double v)
{
    float f = float(v);
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u)
        return f;
    u += 0x7fffu + ((u >> 16) & 1u);
    u &= 0xffff0000u;
    std::memcpy(&f, &u, 4);
    return f;
}

struct d3
{
    double x, y, z;
};
inline d3 sub3(d3 a, d3 b)
{
    return {a.x - b.x, a.y - b.y, a.z - b.z};
}
inline double dot3(d3 a, d3 b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
inline double len3(d3 a)
{
    return std::sqrt(dot3(a, a));
}
inline double angle3(d3 a, d3 b)
{
    d3 const c{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return std::atan2(len3(c), dot3(a, b));
}
inline double seg_dist0(d3 a, d3 b, double* tpar)
{
    d3 const e = sub3(b, a);
    double const ee = dot3(e, e);
    double t = ee > 0 ? -dot3(a, e) / ee : 0.0;
    t = std::min(std::max(t, 0.0), 1.0);
    *tpar = t;
    return len3({a.x + t * e.x, a.y + t * e.y, a.z + t * e.z});
}
inline double lg(double v)
{
    return std::log2(std::max(v, 1e-30)) * 0.125;
}

// The 12 pair features (the device computes the same formulas in float).
void features(double const* c, double const* p, double const* x0in, double tol_feat, float* f)
{
    d3 r[4];
    for (int i = 0; i < 4; ++i)
        r[i] = {double(float(c[3 * i] - p[0])), double(float(c[3 * i + 1] - p[1])), double(float(c[3 * i + 2] - p[2]))};
    d3 const x0{double(float(x0in[0])), double(float(x0in[1])), double(float(x0in[2]))};
    double L = 0;
    d3 e[3];
    for (int i = 0; i < 3; ++i)
    {
        e[i] = sub3(r[i + 1], r[i]);
        L += len3(e[i]);
    }
    L = std::max(L, 1e-30);
    double dpoly = 3e38, t;
    for (int i = 0; i < 3; ++i)
        dpoly = std::min(dpoly, seg_dist0(r[i], r[i + 1], &t));
    double nmin = 3e38, nmax = 0;
    for (int i = 0; i < 4; ++i)
    {
        nmin = std::min(nmin, len3(r[i]));
        nmax = std::max(nmax, len3(r[i]));
    }
    double const chord = len3(sub3(r[3], r[0]));
    double flat = 0;
    for (int i = 1; i <= 2; ++i)
        flat = std::max(flat, seg_dist0(sub3(r[0], r[i]), sub3(r[3], r[i]), &t));
    double const turning = angle3(e[0], e[1]) + angle3(e[1], e[2]);
    double const subt = angle3(r[0], r[1]) + angle3(r[1], r[2]) + angle3(r[2], r[3]);
    d3 u[4];
    for (int i = 0; i < 4; ++i)
    {
        double const a = dot3(r[i], x0);
        u[i] = {r[i].x - a * x0.x, r[i].y - a * x0.y, r[i].z - a * x0.z};
    }
    double dline = 3e38, axial = 0;
    for (int i = 0; i < 3; ++i)
    {
        double const d = seg_dist0(u[i], u[i + 1], &t);
        if (d < dline)
        {
            dline = d;
            d3 const q{r[i].x + t * e[i].x, r[i].y + t * e[i].y, r[i].z + t * e[i].z};
            axial = dot3(q, x0) / std::max(len3(q), 1e-30);
        }
    }
    double v[F] = {lg(dpoly / L),
                   lg(nmin / L),
                   lg(nmax / L),
                   lg(L),
                   chord / L,
                   flat / L,
                   turning / kPi<double>,
                   subt / kPi<double>,
                   lg(dline / L),
                   lg(std::max(dline, 1e-30) / std::max(dpoly, 1e-30)),
                   axial,
                   tol_feat};
    for (int i = 0; i < F; ++i)
        f[i] = float(std::min(std::max(v[i], -8.0), 8.0));
}

// Forward pass of one sample; returns the logits and keeps the pre-activations and BF16 activations.
struct Acts
{
    double x[FP], z1[H], h1[H], z2[H], h2[H], z3[C];
};
void forward(float const* prm, float const* feat, Acts& a)
{
    for (int k = 0; k < FP; ++k)
        a.x[k] = k < F ? bf16(feat[k]) : 0.0;
    for (int o = 0; o < H; ++o)
    {
        double s = 0;
        for (int k = 0; k < FP; ++k)
            s += bf16(prm[oW1 + o * FP + k]) * a.x[k];
        a.z1[o] = double(float(s + prm[oB1 + o]));
        a.h1[o] = bf16(std::max(a.z1[o], 0.0));
    }
    for (int o = 0; o < H; ++o)
    {
        double s = 0;
        for (int k = 0; k < H; ++k)
            s += bf16(prm[oW2 + o * H + k]) * a.h1[k];
        a.z2[o] = double(float(s + prm[oB2 + o]));
        a.h2[o] = bf16(std::max(a.z2[o], 0.0));
    }
    for (int c = 0; c < C; ++c)
    {
        double s = 0;
        for (int k = 0; k < H; ++k)
            s += bf16(prm[oW3 + c * H + k]) * a.h2[k];
        a.z3[c] = s + prm[oB3 + c];
    }
}
} // namespace mlp
} // namespace orc

extern "C"
{
int orc_mlp_param_count()
{
    return orc::mlp::n_params;
}

void orc_param_features_bezier3(double const* pos, int64_t n, double const* x0, double const* curves, int64_t n_curves,
                                double tol, float* out)
{
    double const tf = std::log10(tol) / 10.0;
    for (int64_t q = 0; q < n; ++q)
        for (int64_t c = 0; c < n_curves; ++c)
            orc::mlp::features(curves + 12 * c, pos + 3 * q, x0, double(float(tf)), out + (q * n_curves + c) * 12);
}

void orc_mlp_logits(float const* params, float const* feats, int64_t n, double* logits)
{
    using namespace orc::mlp;
    for (int64_t i = 0; i < n; ++i)
    {
        Acts a;
        forward(params, feats + F * i, a);
        for (int c = 0; c < C; ++c)
            logits[i * C + c] = a.z3[c];
    }
}

// Mean softmax cross-entropy over the first n_classes logits and its gradient, laid out like the parameters.
void orc_mlp_loss_grad(float const* params, float const* feats, uint8_t const* labels, int64_t n, int n_classes,
                       double* grads, double* loss)
{
    using namespace orc::mlp;
    std::fill(grads, grads + n_params, 0.0);
    double total = 0;
    double const inv_n = 1.0 / double(n);
    for (int64_t i = 0; i < n; ++i)
    {
        Acts a;
        forward(params, feats + F * i, a);
        int const lab = std::min(int(labels[i]), n_classes - 1);
        double m = -1e300;
        for (int c = 0; c < n_classes; ++c)
            m = std::max(m, a.z3[c]);
        double sum = 0, ex[C] = {};
        for (int c = 0; c < n_classes; ++c)
            sum += (ex[c] = std::exp(a.z3[c] - m));
        total += std::log(sum) + m - a.z3[lab];
        double dz3[C] = {}, dz3b[C] = {};
        for (int c = 0; c < n_classes; ++c)
        {
            dz3[c] = (ex[c] / sum - (c == lab ? 1.0 : 0.0)) * inv_n;
            dz3b[c] = bf16(dz3[c]);
            grads[oB3 + c] += dz3[c];
            for (int k = 0; k < H; ++k)
                grads[oW3 + c * H + k] += dz3b[c] * a.h2[k];
        }
        double dz2[H], dz2b[H];
        for (int k = 0; k < H; ++k)
        {
            double s = 0;
            for (int c = 0; c < C; ++c)
                s += dz3b[c] * bf16(params[oW3 + c * H + k]);
            dz2[k] = a.z2[k] > 0 ? s : 0.0;
            dz2b[k] = bf16(dz2[k]);
            grads[oB2 + k] += dz2[k];
            for (int j = 0; j < H; ++j)
                grads[oW2 + k * H + j] += dz2b[k] * a.h1[j];
        }
        for (int j = 0; j < H; ++j)
        {
            double s = 0;
            for (int k = 0; k < H; ++k)
                s += dz2b[k] * bf16(params[oW2 + k * H + j]);
            double const dz1 = a.z1[j] > 0 ? s : 0.0;
            double const dz1b = bf16(dz1);
            grads[oB1 + j] += dz1;
            for (int f = 0; f < FP; ++f)
                grads[oW1 + j * FP + f] += dz1b * a.x[f];
        }
    }
    *loss = total * inv_n;
}
} // extern "C"

// ---- parametric integer term: bicubic Bezier patches --------------------------------------------------------
// The Intersector that eval_gwnr_parametric_batch_integer / eval_gwnr_parametric_batch forward to
// (src/antipodal/gwn_parametric.hh:204-284).  The reference ships none for parametric surfaces (README.md, TODO),
// so this restates the project's own rule (the device's, antipodal_gb300/csrc/patch.cu) in plain FP64: every
// crossing of the ray p + lambda dir (lambda > 0) with a patch S(u, v) = sum B_i(v) B_j(u) P[i][j] counts
// sign((S_u x S_v) . dir).
//
// Method: in a right-handed frame whose third axis is dir, the patch relative to p is a map F(u, v) = (x, y) of the
// parameter square with a depth w.  The signed crossings inside a parameter cell whose depth is positive
// throughout are the topological degree of F over the cell at the origin, which is the winding number of the image
// of the cell's boundary (4 cubics) about the origin.  Cells are split in four while their control net's box holds
// the origin and their depth range holds 0; a boundary cubic is split in two while its control points' box holds
// the origin, and a piece whose box does not contributes the crossing of its chord with the positive x axis.  Every
// box test keeps a margin of 2^-42 of the coordinates' scale, far above the rounding of the blossoms, so each
// decision holds for the exact map: the count is exact unless the ray passes within that margin of a cell's
// boundary image or the query lies within it of the surface (the degenerate cases, counted in `degenerate`).
// This is written as plain recursion; the device walks the same trees without a stack.
// Parity of this term is unpinned: no reference implementation exists.
namespace orc
{
// The ray frame: rows e1, e2, e3 = dir / |dir|, right-handed (the helper axis is the unit axis least aligned
// with dir).
inline std::array<double, 9> patch_frame(double const* dir)
{
    double const nn = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    double const z[3] = {dir[0] / nn, dir[1] / nn, dir[2] / nn};
    int m = 0;
    for (int k = 1; k < 3; ++k)
        if (std::fabs(z[k]) < std::fabs(z[m]))
            m = k;
    double a[3] = {0, 0, 0};
    a[m] = 1.0;
    double x[3] = {a[1] * z[2] - a[2] * z[1], a[2] * z[0] - a[0] * z[2], a[0] * z[1] - a[1] * z[0]};
    double const xn = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    for (double& c : x)
        c /= xn;
    double const y[3] = {z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2], z[0] * x[1] - z[1] * x[0]};
    return {x[0], x[1], x[2], y[0], y[1], y[2], z[0], z[1], z[2]};
}

// Control values of the cubic with control values c over [a, b], by blossoming: B(a,a,a), B(a,a,b), B(a,b,b),
// B(b,b,b).  B(t,t,t) is computed by the same steps whichever end t is, so neighbouring pieces share their
// end points exactly.
inline std::array<double, 4> cubic_on(std::array<double, 4> const& c, double a, double b)
{
    auto lerp = [](double p, double q, double t) { return p + t * (q - p); };
    auto blossom = [&](double t1, double t2, double t3)
    {
        double const l0 = lerp(c[0], c[1], t1), l1 = lerp(c[1], c[2], t1), l2 = lerp(c[2], c[3], t1);
        double const m0 = lerp(l0, l1, t2), m1 = lerp(l1, l2, t2);
        return lerp(m0, m1, t3);
    };
    return {blossom(a, a, a), blossom(a, a, b), blossom(a, b, b), blossom(b, b, b)};
}

struct patch_job
{
    double c[16][3]; // [4 iv + iu][x, y across the ray; w along it], relative to the query
    double margin;
    int degenerate = 0;
};

// The crossing of the chord a -> b with the positive x axis: +1 upwards with the origin on its left, -1 downwards
// with the origin on its right (half-open in y, so chords that meet on the axis count once).
inline int chord_crossing(double ax, double ay, double bx, double by)
{
    double const cross = ax * by - ay * bx;
    if (ay <= 0.0)
        return (by > 0.0 && cross > 0.0) ? 1 : 0;
    return (by <= 0.0 && cross < 0.0) ? -1 : 0;
}

// Winding number about the origin of the cubic (x, y) over [t0, t1], with its end points given.
int cubic_winding(patch_job& job, std::array<double, 4> const& x, std::array<double, 4> const& y, double t0,
                  double t1, int level, double ax, double ay, double bx, double by)
{
    std::array<double, 4> const px = cubic_on(x, t0, t1), py = cubic_on(y, t0, t1);
    double const m = job.margin;
    auto [xlo, xhi] = std::minmax({px[0], px[1], px[2], px[3]});
    auto [ylo, yhi] = std::minmax({py[0], py[1], py[2], py[3]});
    if (!(xlo > m || xhi < -m || ylo > m || yhi < -m))
    {
        if (level < 50 && std::max(xhi - xlo, yhi - ylo) >= 4.0 * m)
        {
            double const tm = 0.5 * (t0 + t1);
            std::array<double, 4> const mx = cubic_on(x, tm, tm), my = cubic_on(y, tm, tm);
            return cubic_winding(job, x, y, t0, tm, level + 1, ax, ay, mx[0], my[0]) +
                   cubic_winding(job, x, y, tm, t1, level + 1, mx[0], my[0], bx, by);
        }
        ++job.degenerate; // the curve passes within the margin of the origin
    }
    return chord_crossing(ax, ay, bx, by);
}

// Winding number about the origin of a cell net's boundary, counter-clockwise in (u, v).
int net_winding(patch_job& job, double const (&x)[16], double const (&y)[16])
{
    static constexpr int kEdge[4][4] = {{0, 1, 2, 3}, {3, 7, 11, 15}, {15, 14, 13, 12}, {12, 8, 4, 0}};
    int w = 0;
    for (auto const& e : kEdge)
    {
        std::array<double, 4> const ex = {x[e[0]], x[e[1]], x[e[2]], x[e[3]]};
        std::array<double, 4> const ey = {y[e[0]], y[e[1]], y[e[2]], y[e[3]]};
        w += cubic_winding(job, ex, ey, 0.0, 1.0, 0, ex[0], ey[0], ex[3], ey[3]);
    }
    return w;
}

// Signed crossings in front of the query within the cell [u0, u0 + h] x [v0, v0 + h].
int cell_crossings(patch_job& job, double u0, double v0, double h, int level)
{
    double net[3][16];
    for (int k = 0; k < 3; ++k)
    {
        std::array<double, 4> rows[4];
        for (int r = 0; r < 4; ++r)
            rows[r] = cubic_on({job.c[4 * r][k], job.c[4 * r + 1][k], job.c[4 * r + 2][k], job.c[4 * r + 3][k]}, u0,
                               u0 + h);
        for (int q = 0; q < 4; ++q)
        {
            std::array<double, 4> const col = cubic_on({rows[0][q], rows[1][q], rows[2][q], rows[3][q]}, v0, v0 + h);
            for (int r = 0; r < 4; ++r)
                net[k][4 * r + q] = col[r];
        }
    }
    double const m = job.margin;
    auto [xlo, xhi] = std::minmax_element(net[0], net[0] + 16);
    auto [ylo, yhi] = std::minmax_element(net[1], net[1] + 16);
    auto [wlo, whi] = std::minmax_element(net[2], net[2] + 16);
    if (*xlo > m || *xhi < -m || *ylo > m || *yhi < -m || *whi < -m)
        return 0; // the ray misses the cell, or the cell lies behind the query
    if (*wlo >= m)
        return net_winding(job, net[0], net[1]); // in front throughout: the degree over the cell
    if (level < 45 && *whi - *wlo >= 4.0 * m)
    {
        double const g = 0.5 * h;
        return cell_crossings(job, u0, v0, g, level + 1) + cell_crossings(job, u0 + g, v0, g, level + 1) +
               cell_crossings(job, u0, v0 + g, g, level + 1) + cell_crossings(job, u0 + g, v0 + g, g, level + 1);
    }
    ++job.degenerate; // the query lies within the margin of the surface
    return *wlo + *whi >= 0.0 ? net_winding(job, net[0], net[1]) : 0;
}
} // namespace orc

extern "C"
{
// Signed crossing counts of the rays pos[i] + lambda dir with the bicubic patches ctrl ([n_patches][4][4][3], row
// index v, column index u); degenerate (nullable): per query, the number of unresolved decisions (see above).
void orc_patch_count_bezier3x3_f64(double const* pos, int64_t n, double const* dir, double const* ctrl,
                                   int64_t n_patches, int32_t* out_counts, int32_t* degenerate, int threads)
{
    std::array<double, 9> const f = orc::patch_frame(dir);
    std::vector<double> net(size_t(48) * size_t(n_patches));
    std::vector<double> scale(size_t(n_patches), 0.0);
    for (int64_t k = 0; k < n_patches; ++k)
        for (int j = 0; j < 16; ++j)
            for (int r = 0; r < 3; ++r)
            {
                double const* p = ctrl + 48 * k + 3 * j;
                double const x = f[3 * r] * p[0] + f[3 * r + 1] * p[1] + f[3 * r + 2] * p[2];
                net[48 * k + 3 * j + r] = x;
                scale[k] = std::max(scale[k], std::fabs(x));
            }
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads(threads))
    for (int64_t i = 0; i < n; ++i)
    {
        double q[3];
        for (int r = 0; r < 3; ++r)
            q[r] = f[3 * r] * pos[3 * i] + f[3 * r + 1] * pos[3 * i + 1] + f[3 * r + 2] * pos[3 * i + 2];
        double const qs = std::max(std::max(std::fabs(q[0]), std::fabs(q[1])), std::fabs(q[2]));
        int sum = 0, deg = 0;
        for (int64_t k = 0; k < n_patches; ++k)
        {
            orc::patch_job job;
            for (int j = 0; j < 16; ++j)
                for (int r = 0; r < 3; ++r)
                    job.c[j][r] = net[48 * k + 3 * j + r] - q[r];
            job.margin = std::ldexp(qs + scale[k], -42);
            sum += orc::cell_crossings(job, 0.0, 0.0, 1.0, 0);
            deg += job.degenerate;
        }
        out_counts[i] = sum;
        if (degenerate)
            degenerate[i] = deg;
    }
}
} // extern "C"
