// C ABI over the antipodal reference itself, compiled from the reference's own headers (oracle/Makefile builds
// this into oracle/_ref/libref_gwn.so with the reference's src/ on the include path).
//
// TEST INFRASTRUCTURE ONLY.  It pins the restatement in oracle/gwn_oracle.cc (same entry points with the
// prefix ref_ instead of orc_) and generates the golden fixtures under tests/golden/.  Batch calls go
// through the reference's own PoolDispatcher, NaiveIntersector, RobustMeshGwn and IntegratorGK15.
// RobustMeshGwn needs Embree; oracle/fake_embree provides the subset of its API that the reference uses.

#include <antipodal/dispatcher/dispatcher.hh>
#include <antipodal/dispatcher/dispatcher_threadpool.hh>
#include <antipodal/gwn_mesh.hh>
#include <antipodal/gwn_mesh_robust.hh>
#include <antipodal/gwn_parametric.hh>
#include <antipodal/intersector/intersector.hh>
#include <antipodal/math/common.hh>
#include <antipodal/math/integrate_gk15.hh>
#include <antipodal/math/robust_predicates.hh>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <span>
#include <thread>
#include <vector>

using namespace antipodal;

namespace
{
template <class T>
std::span<vec3<T> const> pts(T const* p, int64_t n)
{
    return {reinterpret_cast<vec3<T> const*>(p), size_t(n)};
}
template <class T>
std::span<weighted_segment3<T> const> segs(T const* p, int64_t n)
{
    static_assert(sizeof(weighted_segment3<T>) == 7 * sizeof(T));
    return {reinterpret_cast<weighted_segment3<T> const*>(p), size_t(n)};
}
int pool_threads(int t)
{
    return t > 0 ? t : int(std::max(1u, std::thread::hardware_concurrency()));
}

// The project's cubic Bezier boundary curve, callable with fwd_diff<T> like the test suite's LineCurve
// (test/test_gwn_parametric.cc:86-97).  Bernstein basis in dual numbers.
struct Bezier3
{
    dvec3 c0, c1, c2, c3;
    template <class S>
    vec3<S> operator()(S t) const
    {
        S const u = 1.0 - t;
        S const b0 = u * u * u;
        S const b1 = 3.0 * u * u * t;
        S const b2 = 3.0 * u * t * t;
        S const b3 = t * t * t;
        return c0 * b0 + c1 * b1 + c2 * b2 + c3 * b3;
    }
};
struct Bezier3Boundary
{
    std::vector<Bezier3> const* curves;
    template <class Visit>
    void operator()(Visit&& visit) const
    {
        for (auto const& c : *curves)
            visit(c);
    }
};
} // namespace

extern "C"
{
double ref_vos_half_f64(double const* x1, double const* v0, double const* v1)
{
    return signed_spherical_tri_area_half_unorm<double>({x1[0], x1[1], x1[2]}, {v0[0], v0[1], v0[2]},
                                                        {v1[0], v1[1], v1[2]});
}
float ref_vos_half_f32(float const* x1, float const* v0, float const* v1)
{
    return signed_spherical_tri_area_half_unorm<float>({x1[0], x1[1], x1[2]}, {v0[0], v0[1], v0[2]},
                                                       {v1[0], v1[1], v1[2]});
}

#define REF_MESH(SUF, T)                                                                                      \
    void ref_frac_batch_##SUF(T const* pos, int64_t n, T* out, T const* x0, T const* seg, int64_t n_seg,       \
                              int threads)                                                                    \
    {                                                                                                         \
        PoolDispatcher disp{pool_threads(threads)};                                                           \
        eval_gwnr_mesh_batch_fractional(disp, pts(pos, n), std::span<T>{out, size_t(n)},                      \
                                        vec3<T>{x0[0], x0[1], x0[2]}, segs(seg, n_seg));                      \
    }                                                                                                         \
    void ref_int_naive_##SUF(T const* pos, int64_t n, int32_t* out, T const* dir, T const* verts, int64_t nv,   \
                             int32_t const* idx, int64_t n_idx, int threads)                                  \
    {                                                                                                         \
        PoolDispatcher disp{pool_threads(threads)};                                                           \
        NaiveIntersector<T> isect{pts(verts, nv), std::span<int const>{idx, size_t(n_idx)}};                  \
        eval_gwnr_mesh_batch_integer(disp, isect, pts(pos, n), std::span<int>{out, size_t(n)},                \
                                     vec3<T>{dir[0], dir[1], dir[2]});                                        \
    }                                                                                                         \
    void ref_full_naive_##SUF(T const* pos, int64_t n, T* out, T const* x0, T const* verts, int64_t nv,        \
                              int32_t const* idx, int64_t n_idx, T const* seg, int64_t n_seg, int threads)    \
    {                                                                                                         \
        PoolDispatcher disp{pool_threads(threads)};                                                           \
        NaiveIntersector<T> isect{pts(verts, nv), std::span<int const>{idx, size_t(n_idx)}};                  \
        eval_gwnr_mesh_batch(disp, isect, pts(pos, n), std::span<T>{out, size_t(n)},                          \
                             vec3<T>{x0[0], x0[1], x0[2]}, segs(seg, n_seg));                                 \
    }                                                                                                         \
    int64_t ref_boundary_##SUF(T const* verts, int64_t nv, int32_t const* idx, int64_t n_idx, T* out,          \
                               int64_t cap)                                                                   \
    {                                                                                                         \
        auto const b = build_boundary_segments<T>(pts(verts, nv), std::span<int const>{idx, size_t(n_idx)});  \
        int64_t const cnt = int64_t(b.size());                                                                \
        if (out)                                                                                              \
            std::memcpy(out, b.data(), sizeof(T) * 7 * size_t(std::min(cnt, cap)));                           \
        return cnt;                                                                                           \
    }

REF_MESH(f64, double)
REF_MESH(f32, float)

int ref_robust_eval(int scalar_bytes, int policy, void const* verts, int64_t nv, int32_t const* idx, int64_t n_idx,
                    void const* seg, int64_t n_seg, void const* pos, int64_t n, void* out, int32_t* out_count,
                    void* out_frac, int threads)
{
    auto run = [&](auto scalar_tag, auto policy_tag)
    {
        using T = decltype(scalar_tag);
        using P = decltype(policy_tag);
        RobustMeshGwn<T, P> const m{pts(static_cast<T const*>(verts), nv), std::span<int const>{idx, size_t(n_idx)},
                                    segs(static_cast<T const*>(seg), n_seg)};
        auto const q = pts(static_cast<T const*>(pos), n);
        if (out)
        {
            PoolDispatcher disp{pool_threads(threads)};
            eval_gwnr_mesh_batch_robust(disp, m, q, std::span<T>{static_cast<T*>(out), size_t(n)});
        }
        for (int64_t i = 0; i < n; ++i)
        {
            if (out_count)
                out_count[i] = m.signed_intersection_count(q[i]);
            if (out_frac)
                static_cast<T*>(out_frac)[i] = m.fractional(q[i]);
        }
    };
    auto by_policy = [&](auto scalar_tag)
    {
        switch (policy)
        {
        case 0:
            run(scalar_tag, robust::int64_grid{});
            return 0;
        case 1:
            run(scalar_tag, robust::int128_grid{});
            return 0;
        case 2:
            run(scalar_tag, robust::exact_float{});
            return 0;
        default:
            return 1;
        }
    };
    if (scalar_bytes == 4)
        return by_policy(float{});
    if (scalar_bytes == 8)
        return by_policy(double{});
    return 1;
}

int ref_predicates(int policy, void const* q, void const* q0, void const* q1, void const* q2, int64_t n,
                   int32_t* out_edge_sign, double* out_num, int32_t* out_inside)
{
    auto run = [&](auto tag)
    {
        using C = decltype(tag);
        auto const* a = static_cast<vec3<C> const*>(q);
        auto const* b = static_cast<vec3<C> const*>(q0);
        auto const* c = static_cast<vec3<C> const*>(q1);
        auto const* d = static_cast<vec3<C> const*>(q2);
        for (int64_t i = 0; i < n; ++i)
        {
            out_edge_sign[i] = robust::edge_sign(a[i], b[i], c[i]);
            out_num[i] = double(robust::atan2_num(a[i], b[i], c[i]));
            out_inside[i] = robust::inside_tri_sign(a[i], b[i], c[i], d[i]);
        }
    };
    if (policy == 0)
        run(std::int32_t{});
    else if (policy == 1)
        run(std::int64_t{});
    else if (policy == 2)
        run(double{});
    else
        return 1;
    return 0;
}

// project_into_tri(q, q0, q1, q2) weights w0, w1, w2 per row (robust_predicates.hh:391-402).
int ref_predicate_weights(int policy, void const* q, void const* q0, void const* q1, void const* q2, int64_t n,
                          double* out_weights)
{
    auto run = [&](auto tag)
    {
        using C = decltype(tag);
        auto const* a = static_cast<vec3<C> const*>(q);
        auto const* b = static_cast<vec3<C> const*>(q0);
        auto const* c = static_cast<vec3<C> const*>(q1);
        auto const* d = static_cast<vec3<C> const*>(q2);
        for (int64_t i = 0; i < n; ++i)
        {
            auto const h = robust::project_into_tri(a[i], b[i], c[i], d[i]);
            out_weights[3 * i] = h.w0;
            out_weights[3 * i + 1] = h.w1;
            out_weights[3 * i + 2] = h.w2;
        }
    };
    if (policy == 0)
        run(std::int32_t{});
    else if (policy == 1)
        run(std::int64_t{});
    else if (policy == 2)
        run(double{});
    else
        return 1;
    return 0;
}

void ref_param_frac_bezier3_f64(double const* pos, int64_t n, double* out, double const* x0, double const* ctrl,
                                int64_t n_curves, int min_depth, int max_depth, double tol, int32_t*, int32_t*,
                                int threads)
{
    std::vector<Bezier3> curves;
    for (int64_t c = 0; c < n_curves; ++c)
    {
        double const* k = ctrl + 12 * c;
        curves.push_back({{k[0], k[1], k[2]}, {k[3], k[4], k[5]}, {k[6], k[7], k[8]}, {k[9], k[10], k[11]}});
    }
    Bezier3Boundary const boundary{&curves};
    integrate_config const cfg{min_depth, max_depth, tol};
    PoolDispatcher disp{pool_threads(threads)};
    eval_gwnr_parametric_batch_fractional(disp, pts(pos, n), std::span<double>{out, size_t(n)},
                                          dvec3{x0[0], x0[1], x0[2]}, boundary, cfg, IntegratorGK15{});
}

double ref_gk15_known(int fn, double a, double b, int min_depth, int max_depth, double tol, double* err, int* leaves)
{
    integrate_config const cfg{min_depth, max_depth, tol};
    auto f = [fn](int, double t)
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
    return integrate_gk15(f, a, b, cfg, err, leaves);
}
} // extern "C"
