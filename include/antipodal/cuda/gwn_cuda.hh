#pragma once

// Header-only C++20 front end of the GB300 batch GWN library: the antipodal library's batch API, with its
// Dispatcher and Intersector roles filled by the GPU.
//
//   antipodal::cuda::CudaDispatcher disp;                              // device 0, own stream
//   antipodal::cuda::CudaIntersector<double> isect{disp, vertices, indices};
//   antipodal::eval_gwnr_mesh_batch(disp, isect, positions, out, x0, boundary);
//
// The overloads below take CudaDispatcher by reference and are more specialised than the reference's
// templates (src/antipodal/gwn_mesh.hh:67-219), so overload resolution picks them.  Every other call with a
// CudaDispatcher fails to compile at parallel_for (there is no CPU fallback).  Include after the reference's own
// headers, or let this header include them: it needs antipodal::vec3 and antipodal::weighted_segment3
// (src/antipodal/math/common.hh).  Link with libantipodal_gb300.so; the C ABI is include/antipodal_gb300.h.
//
// Errors: a non-zero status from the library becomes antipodal::cuda::Error (a std::runtime_error) carrying the
// status and the library's message.  Size mismatches, which the reference asserts, throw std::invalid_argument.

#include <antipodal/math/common.hh>
#include <antipodal/math/integrate.hh>

#include <antipodal_gb300.h>

#include <array>
#include <cstdint>
#include <mutex>
#include <span>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace antipodal::cuda
{
class Error : public std::runtime_error
{
public:
    Error(int status, std::string const& what) : std::runtime_error(what), m_status(status) {}
    [[nodiscard]] int status() const noexcept { return m_status; }

private:
    int m_status;
};

inline void check(int status, char const* where)
{
    if (status != AGWN_OK)
        throw Error(status, std::string(where) + ": " + agwn_status_string(status) + ": " + agwn_last_error_message());
}

enum class precision
{
    exact = AGWN_FRAC_EXACT, // the reference's arithmetic in the input precision (default)
    mixed = AGWN_FRAC_MIXED  // FP32 pairs + FP64 for near / ill-conditioned / branch pairs (double inputs)
};

// The Dispatcher role (src/antipodal/dispatcher/dispatcher.hh:3-36) on one GPU: a device, a stream, scratch
// memory and the fractional-term options.  Runs one job at a time, like PoolDispatcher.
class CudaDispatcher
{
public:
    explicit CudaDispatcher(int device = 0, void* stream = nullptr, precision p = precision::exact)
    {
        check(agwn_context_create(device, stream, &m_ctx), "agwn_context_create");
        set_precision(p);
    }
    ~CudaDispatcher()
    {
        if (m_ctx)
            agwn_context_destroy(m_ctx);
    }
    CudaDispatcher(CudaDispatcher const&) = delete;
    CudaDispatcher& operator=(CudaDispatcher const&) = delete;
    CudaDispatcher(CudaDispatcher&& o) noexcept : m_ctx(std::exchange(o.m_ctx, nullptr)) {}
    CudaDispatcher& operator=(CudaDispatcher&& o) noexcept
    {
        if (this != &o)
        {
            if (m_ctx)
                agwn_context_destroy(m_ctx);
            m_ctx = std::exchange(o.m_ctx, nullptr);
        }
        return *this;
    }

    void set_precision(precision p) { set_option(AGWN_OPT_FRAC_MODE, double(int(p))); }
    // Robust evaluator's fractional term: exact (the reference's FP64 arithmetic, default) or mixed (int64_grid:
    // FP32 pairs under a first-order error bound; exact_float with double queries: the mesh functions' mixed kernel
    // along -x; the other pairs by the evaluator's own FP64 rule); integer counts are the same either way.
    void set_robust_precision(precision p)
    {
        set_option(AGWN_OPT_ROBUST_MODE, p == precision::mixed ? AGWN_ROBUST_MIXED : AGWN_ROBUST_EXACT);
    }
    // The parametric integrator's arithmetic: exact (FP64, bit for bit the reference; default) or mixed
    // (double-float panels on the FP32 pipe, the same tree rule).
    void set_param_precision(precision p)
    {
        set_option(AGWN_OPT_PARAM_MODE, p == precision::mixed ? AGWN_PARAM_MIXED : AGWN_PARAM_EXACT);
    }
    void set_option(int option, double value) { check(agwn_context_set_option(m_ctx, option, value), "set_option"); }
    [[nodiscard]] double option(int option) const
    {
        double v = 0;
        check(agwn_context_get_option(m_ctx, option, &v), "get_option");
        return v;
    }
    void synchronize() { check(agwn_context_synchronize(m_ctx), "agwn_context_synchronize"); }
    [[nodiscard]] agwn_context* handle() const noexcept { return m_ctx; }

    // The reference's parallel_for runs arbitrary host callables; the GPU library has no form for them and no
    // CPU fallback, so a generic batch function instantiated with this dispatcher does not compile.
    template <class F>
    void parallel_for(int, int, F&&)
    {
        static_assert(sizeof(F) == 0, "CudaDispatcher runs the library's GWN kernels only: use a batch function "
                                      "overloaded for CudaDispatcher, or a CPU dispatcher for other callables");
    }

private:
    agwn_context* m_ctx = nullptr;
};

// The Intersector role (src/antipodal/intersector/intersector.hh:3-40) over a device LBVH.  Counts equal
// NaiveIntersector<T>'s bit for bit.  The mesh is copied to the device, so the caller's arrays need not outlive
// the intersector.  signed_intersection_count() is the concept member: thread-safe, but one GPU round trip per
// point -- use the batch functions for throughput.
template <class T>
class CudaIntersector
{
    static_assert(std::is_same_v<T, float> || std::is_same_v<T, double>, "float or double geometry");

public:
    CudaIntersector(CudaDispatcher& disp, std::span<vec3<T> const> vertices, std::span<int const> indices)
      : m_disp(&disp)
    {
        static_assert(sizeof(vec3<T>) == 3 * sizeof(T) && sizeof(int) == sizeof(std::int32_t));
        auto const* v = reinterpret_cast<T const*>(vertices.data());
        auto const* i = reinterpret_cast<std::int32_t const*>(indices.data());
        if constexpr (std::is_same_v<T, double>)
            check(agwn_bvh_create_f64(disp.handle(), v, std::int64_t(vertices.size()), i, std::int64_t(indices.size()),
                                      &m_bvh),
                  "agwn_bvh_create_f64");
        else
            check(agwn_bvh_create_f32(disp.handle(), v, std::int64_t(vertices.size()), i, std::int64_t(indices.size()),
                                      &m_bvh),
                  "agwn_bvh_create_f32");
    }
    ~CudaIntersector()
    {
        if (m_bvh)
            agwn_bvh_destroy(m_bvh);
    }
    CudaIntersector(CudaIntersector const&) = delete;
    CudaIntersector& operator=(CudaIntersector const&) = delete;

    [[nodiscard]] int signed_intersection_count(vec3<T> p, vec3<T> dir) const
    {
        std::lock_guard<std::mutex> lock(m_mutex);
        std::int32_t out = 0;
        T const d[3] = {dir.x, dir.y, dir.z};
        if constexpr (std::is_same_v<T, double>)
            check(agwn_mesh_batch_integer_f64(m_disp->handle(), m_bvh, &p.x, 1, &out, d), "signed_intersection_count");
        else
            check(agwn_mesh_batch_integer_f32(m_disp->handle(), m_bvh, &p.x, 1, &out, d), "signed_intersection_count");
        return out;
    }

    [[nodiscard]] agwn_bvh const* handle() const noexcept { return m_bvh; }
    [[nodiscard]] CudaDispatcher& dispatcher() const noexcept { return *m_disp; }

private:
    CudaDispatcher* m_disp;
    agwn_bvh* m_bvh = nullptr;
    mutable std::mutex m_mutex;
};

// Precision policies of the robust evaluator.  The reference's tags (src/antipodal/math/robust_predicates.hh:
// robust::int64_grid, int128_grid, exact_float) work as well: a policy is recognised by its coord type.
struct int64_grid
{
    using coord = std::int32_t;
};
struct int128_grid
{
    using coord = std::int64_t;
};
struct exact_float
{
    using coord = double;
};
template <class T>
using default_precision = std::conditional_t<std::is_same_v<T, float>, int64_grid, exact_float>;

namespace detail
{
template <class P>
constexpr int policy_of()
{
    using C = typename P::coord;
    static_assert(std::is_same_v<C, std::int32_t> || std::is_same_v<C, std::int64_t> || std::is_same_v<C, double>,
                  "precision policy: coord must be int32_t (int64_grid), int64_t (int128_grid) or double (exact_float)");
    return std::is_same_v<C, std::int32_t> ? AGWN_ROBUST_INT64_GRID
                                           : (std::is_same_v<C, std::int64_t> ? AGWN_ROBUST_INT128_GRID
                                                                              : AGWN_ROBUST_EXACT_FLOAT);
}
} // namespace detail

// RobustMeshGwn<T, Precision> (src/antipodal/gwn_mesh_robust.hh:170-424) on the device: the mesh is quantised and
// its ray-frame hierarchy built on the GPU.  Counts equal the reference's bit for bit under every policy.
// eval / fractional / signed_intersection_count are the concept members (one GPU round trip per point); use
// eval_gwnr_mesh_batch_robust or evaluate() for throughput.
template <class T, class Precision = default_precision<T>>
class CudaRobustMeshGwn
{
    static_assert(std::is_same_v<T, float> || std::is_same_v<T, double>, "float or double geometry");

public:
    using precision = Precision;

    CudaRobustMeshGwn(CudaDispatcher& disp, std::span<vec3<T> const> vertices, std::span<int const> indices,
                      std::span<weighted_segment3<T> const> boundary)
      : m_disp(&disp)
    {
        static_assert(sizeof(vec3<T>) == 3 * sizeof(T) && sizeof(weighted_segment3<T>) == 7 * sizeof(T));
        auto const* v = reinterpret_cast<T const*>(vertices.data());
        auto const* i = reinterpret_cast<std::int32_t const*>(indices.data());
        auto const* b = reinterpret_cast<T const*>(boundary.data());
        constexpr int pol = detail::policy_of<Precision>();
        if constexpr (std::is_same_v<T, double>)
            check(agwn_robust_create_f64(disp.handle(), pol, v, std::int64_t(vertices.size()), i,
                                         std::int64_t(indices.size()), b, std::int64_t(boundary.size()), &m_r),
                  "agwn_robust_create_f64");
        else
            check(agwn_robust_create_f32(disp.handle(), pol, v, std::int64_t(vertices.size()), i,
                                         std::int64_t(indices.size()), b, std::int64_t(boundary.size()), &m_r),
                  "agwn_robust_create_f32");
    }
    ~CudaRobustMeshGwn()
    {
        if (m_r)
            agwn_robust_destroy(m_r);
    }
    CudaRobustMeshGwn(CudaRobustMeshGwn const&) = delete;
    CudaRobustMeshGwn& operator=(CudaRobustMeshGwn const&) = delete;

    // Full GWN (and optionally the integer and fractional terms) of a batch; spans may be host or device memory.
    void evaluate(std::span<vec3<T> const> positions, std::span<T> out, std::span<int> counts = {},
                  std::span<T> fractional = {}) const
    {
        if (out.size() != positions.size() || (!counts.empty() && counts.size() != positions.size()) ||
            (!fractional.empty() && fractional.size() != positions.size()))
            throw std::invalid_argument("CudaRobustMeshGwn::evaluate: positions and outputs differ in size");
        auto const* p = reinterpret_cast<T const*>(positions.data());
        auto* c = counts.empty() ? nullptr : reinterpret_cast<std::int32_t*>(counts.data());
        T* f = fractional.empty() ? nullptr : fractional.data();
        if constexpr (std::is_same_v<T, double>)
            check(agwn_robust_eval_f64(m_disp->handle(), m_r, p, std::int64_t(positions.size()), out.data(), c, f),
                  "agwn_robust_eval_f64");
        else
            check(agwn_robust_eval_f32(m_disp->handle(), m_r, p, std::int64_t(positions.size()), out.data(), c, f),
                  "agwn_robust_eval_f32");
    }

    [[nodiscard]] T eval(vec3<T> p) const
    {
        T out{};
        evaluate(std::span<vec3<T> const>{&p, 1}, std::span<T>{&out, 1});
        return out;
    }
    [[nodiscard]] T fractional(vec3<T> p) const
    {
        T out{}, fr{};
        int c = 0;
        evaluate(std::span<vec3<T> const>{&p, 1}, std::span<T>{&out, 1}, std::span<int>{&c, 1}, std::span<T>{&fr, 1});
        return fr;
    }
    [[nodiscard]] int signed_intersection_count(vec3<T> p) const
    {
        T out{};
        int c = 0;
        evaluate(std::span<vec3<T> const>{&p, 1}, std::span<T>{&out, 1}, std::span<int>{&c, 1});
        return c;
    }

    [[nodiscard]] agwn_robust const* handle() const noexcept { return m_r; }

private:
    CudaDispatcher* m_disp;
    agwn_robust* m_r = nullptr;
};

// Many CudaRobustMeshGwn meshes, each with its own device arrays of queries and results, evaluated in one
// persistent launch over a device work queue (no reference counterpart; the values equal
// eval_gwnr_mesh_batch_robust per mesh bit for bit).  tune() times the launch configurations on a sample and
// keeps the fastest; run() replays a CUDA graph after the first call.  Meshes and arrays must outlive the batch.
template <class T, class Precision = default_precision<T>>
class CudaRobustBatch
{
public:
    struct Job
    {
        CudaRobustMeshGwn<T, Precision> const* mesh;
        vec3<T> const* positions; // device
        std::int64_t n;
        T* out;                   // device
        int* counts = nullptr;    // device, optional
    };

    CudaRobustBatch(CudaDispatcher& disp, std::span<Job const> jobs) : m_disp(&disp)
    {
        std::vector<agwn_robust const*> m;
        std::vector<void const*> p;
        std::vector<std::int64_t> n;
        std::vector<void*> o;
        std::vector<std::int32_t*> c;
        for (auto const& j : jobs)
        {
            m.push_back(j.mesh->handle());
            p.push_back(j.positions);
            n.push_back(j.n);
            o.push_back(j.out);
            c.push_back(reinterpret_cast<std::int32_t*>(j.counts));
        }
        check(agwn_batch_create(disp.handle(), m.data(), std::int32_t(m.size()), p.data(), n.data(), o.data(),
                                c.data(), &m_b),
              "agwn_batch_create");
    }
    ~CudaRobustBatch()
    {
        if (m_b)
            agwn_batch_destroy(m_b);
    }
    CudaRobustBatch(CudaRobustBatch const&) = delete;
    CudaRobustBatch& operator=(CudaRobustBatch const&) = delete;

    void tune(int repeats = 2) { check(agwn_batch_tune(m_disp->handle(), m_b, repeats), "agwn_batch_tune"); }
    void run(bool graph = true) { check(agwn_batch_run(m_disp->handle(), m_b, graph ? 1 : 0), "agwn_batch_run"); }
    // {threads per CTA, queries per thread, segment tile, traversal stack}
    [[nodiscard]] std::array<std::int32_t, 4> config() const
    {
        std::array<std::int32_t, 4> c{};
        check(agwn_batch_info(m_b, c.data(), nullptr, nullptr, nullptr, nullptr, nullptr), "agwn_batch_info");
        return c;
    }

private:
    CudaDispatcher* m_disp;
    agwn_batch* m_b = nullptr;
};

// Boundary of a parametric surface made of cubic Bezier curves (control points c0..c3 per curve), in the order the
// reference's for_each_boundary would visit them: the device-representable form of ForEachBoundary
// (src/antipodal/gwn_parametric.hh:34-41).
struct CubicBezierBoundary
{
    std::span<std::array<vec3<double>, 4> const> curves;
};

// The Intersector role for parametric surfaces of bicubic Bezier patches (the reference ships none: its
// eval_gwnr_parametric_batch_integer / eval_gwnr_parametric_batch, src/antipodal/gwn_parametric.hh:204-284, take
// any Intersector).  A crossing of the ray p + lambda x0 (lambda >= 0) counts sign(N . x0), N = S_u x S_v, with
// S(u, v) = sum B_i(v) B_j(u) P[i][j] and each patch given as its 16 control points P[i][j] at index 4 i + j.  The
// patches are copied to the device.  signed_intersection_count() is the concept member (one GPU round trip per
// point).
class CudaBezierPatchIntersector
{
public:
    CudaBezierPatchIntersector(CudaDispatcher& disp, std::span<std::array<vec3<double>, 16> const> patches)
      : m_disp(&disp)
    {
        static_assert(sizeof(std::array<vec3<double>, 16>) == 48 * sizeof(double));
        check(agwn_patches_create_f64(disp.handle(), reinterpret_cast<double const*>(patches.data()),
                                      std::int64_t(patches.size()), &m_patches),
              "agwn_patches_create_f64");
    }
    ~CudaBezierPatchIntersector()
    {
        if (m_patches)
            agwn_patches_destroy(m_patches);
    }
    CudaBezierPatchIntersector(CudaBezierPatchIntersector const&) = delete;
    CudaBezierPatchIntersector& operator=(CudaBezierPatchIntersector const&) = delete;

    [[nodiscard]] int signed_intersection_count(vec3<double> p, vec3<double> dir) const
    {
        std::int32_t out = 0;
        double const d[3] = {dir.x, dir.y, dir.z};
        check(agwn_param_batch_integer_bezier3x3_f64(m_disp->handle(), m_patches, &p.x, 1, &out, d),
              "signed_intersection_count");
        return out;
    }

    [[nodiscard]] agwn_patches* handle() const noexcept { return m_patches; }

private:
    CudaDispatcher* m_disp;
    agwn_patches* m_patches = nullptr;
};

// Learned start depths for the plain GK15 integrator (no reference counterpart): a 12 -> 64 -> 64 -> 16 MLP on
// the tensor cores, trained on the plain integrator's depths.  Passed as the integrator of the parametric batch
// function; every evaluated panel is still accepted or refined by the plain error test.
class LearnedGK15Proposal
{
public:
    explicit LearnedGK15Proposal(CudaDispatcher& disp, std::uint64_t seed = 0, int n_classes = 11,
                                 float alpha = 0.02f)
      : m_disp(&disp), m_classes(n_classes), m_alpha(alpha)
    {
        check(agwn_mlp_create(disp.handle(), seed, &m_mlp), "agwn_mlp_create");
    }
    ~LearnedGK15Proposal()
    {
        if (m_mlp)
            agwn_mlp_destroy(m_mlp);
    }
    LearnedGK15Proposal(LearnedGK15Proposal const&) = delete;
    LearnedGK15Proposal& operator=(LearnedGK15Proposal const&) = delete;

    [[nodiscard]] std::vector<float> params() const
    {
        std::vector<float> p(static_cast<std::size_t>(agwn_mlp_param_count()));
        check(agwn_mlp_get_params(m_disp->handle(), m_mlp, p.data()), "agwn_mlp_get_params");
        return p;
    }
    void set_params(std::span<float const> p)
    {
        if (p.size() != std::size_t(agwn_mlp_param_count()))
            throw std::invalid_argument("LearnedGK15Proposal::set_params: wrong parameter count");
        check(agwn_mlp_set_params(m_disp->handle(), m_mlp, p.data()), "agwn_mlp_set_params");
    }
    // features: rows of 12 floats from agwn_param_features_bezier3_f64; labels: the plain integrator's shallowest
    // accepted depth per row.  Returns each step's mean loss.
    std::vector<float> train(std::span<float const> features, std::span<std::uint8_t const> labels, int steps,
                             int batch = 8192, float lr = 2e-3f, std::uint64_t seed = 1)
    {
        if (features.size() != 12 * labels.size())
            throw std::invalid_argument("LearnedGK15Proposal::train: 12 features per label");
        std::vector<float> loss(std::size_t(steps > 0 ? steps : 0));
        check(agwn_mlp_train(m_disp->handle(), m_mlp, features.data(), labels.data(), std::int64_t(labels.size()),
                             m_classes, steps, batch, lr, seed, loss.empty() ? nullptr : loss.data()),
              "agwn_mlp_train");
        return loss;
    }

    [[nodiscard]] agwn_mlp const* handle() const noexcept { return m_mlp; }
    [[nodiscard]] int n_classes() const noexcept { return m_classes; }
    [[nodiscard]] float alpha() const noexcept { return m_alpha; }

private:
    CudaDispatcher* m_disp;
    agwn_mlp* m_mlp = nullptr;
    int m_classes;
    float m_alpha;
};

namespace detail
{
template <class T>
T const* raw(std::span<vec3<T> const> s)
{
    static_assert(sizeof(vec3<T>) == 3 * sizeof(T));
    return reinterpret_cast<T const*>(s.data());
}
template <class T>
T const* raw(std::span<weighted_segment3<T> const> s)
{
    static_assert(sizeof(weighted_segment3<T>) == 7 * sizeof(T));
    return reinterpret_cast<T const*>(s.data());
}
inline void same_size(std::size_t a, std::size_t b, char const* what)
{
    if (a != b)
        throw std::invalid_argument(std::string(what) + ": positions and outputs differ in size");
}
} // namespace detail
} // namespace antipodal::cuda

namespace antipodal
{
// gwn_mesh.hh:67-83 on the GPU.
template <class T>
void eval_gwnr_mesh_batch_fractional(cuda::CudaDispatcher& dispatcher, std::span<vec3<T> const> positions,
                                     std::span<T> out_wnrs, vec3<T> x0, std::span<weighted_segment3<T> const> boundary)
{
    cuda::detail::same_size(positions.size(), out_wnrs.size(), "eval_gwnr_mesh_batch_fractional");
    T const x[3] = {x0.x, x0.y, x0.z};
    if constexpr (std::is_same_v<T, double>)
        cuda::check(agwn_mesh_batch_fractional_f64(dispatcher.handle(), cuda::detail::raw(positions),
                                                   std::int64_t(positions.size()), out_wnrs.data(), x,
                                                   cuda::detail::raw(boundary), std::int64_t(boundary.size())),
                    "eval_gwnr_mesh_batch_fractional");
    else
        cuda::check(agwn_mesh_batch_fractional_f32(dispatcher.handle(), cuda::detail::raw(positions),
                                                   std::int64_t(positions.size()), out_wnrs.data(), x,
                                                   cuda::detail::raw(boundary), std::int64_t(boundary.size())),
                    "eval_gwnr_mesh_batch_fractional");
}

// gwn_mesh.hh:127-143 on the GPU.
template <class T>
void eval_gwnr_mesh_batch_integer(cuda::CudaDispatcher& dispatcher, cuda::CudaIntersector<T> const& intersector,
                                  std::span<vec3<T> const> positions, std::span<int> out_counts, vec3<T> x0)
{
    cuda::detail::same_size(positions.size(), out_counts.size(), "eval_gwnr_mesh_batch_integer");
    T const x[3] = {x0.x, x0.y, x0.z};
    auto* o = reinterpret_cast<std::int32_t*>(out_counts.data());
    if constexpr (std::is_same_v<T, double>)
        cuda::check(agwn_mesh_batch_integer_f64(dispatcher.handle(), intersector.handle(), cuda::detail::raw(positions),
                                                std::int64_t(positions.size()), o, x),
                    "eval_gwnr_mesh_batch_integer");
    else
        cuda::check(agwn_mesh_batch_integer_f32(dispatcher.handle(), intersector.handle(), cuda::detail::raw(positions),
                                                std::int64_t(positions.size()), o, x),
                    "eval_gwnr_mesh_batch_integer");
}

// gwn_mesh.hh:201-219 on the GPU: fractional + integer, fused per query.
template <class T>
void eval_gwnr_mesh_batch(cuda::CudaDispatcher& dispatcher, cuda::CudaIntersector<T> const& intersector,
                          std::span<vec3<T> const> positions, std::span<T> out_wnrs, vec3<T> x0,
                          std::span<weighted_segment3<T> const> boundary)
{
    cuda::detail::same_size(positions.size(), out_wnrs.size(), "eval_gwnr_mesh_batch");
    T const x[3] = {x0.x, x0.y, x0.z};
    if constexpr (std::is_same_v<T, double>)
        cuda::check(agwn_mesh_batch_f64(dispatcher.handle(), intersector.handle(), cuda::detail::raw(positions),
                                        std::int64_t(positions.size()), out_wnrs.data(), x,
                                        cuda::detail::raw(boundary), std::int64_t(boundary.size())),
                    "eval_gwnr_mesh_batch");
    else
        cuda::check(agwn_mesh_batch_f32(dispatcher.handle(), intersector.handle(), cuda::detail::raw(positions),
                                        std::int64_t(positions.size()), out_wnrs.data(), x,
                                        cuda::detail::raw(boundary), std::int64_t(boundary.size())),
                    "eval_gwnr_mesh_batch");
}

// common.hh:123-174 on the GPU: the open boundary, rows in ascending (lo, hi) vertex order (the reference emits
// the same rows in hash-map order).
template <class T>
[[nodiscard]] std::vector<weighted_segment3<T>> build_boundary_segments(cuda::CudaDispatcher& dispatcher,
                                                                        std::span<vec3<T> const> vertices,
                                                                        std::span<int const> indices)
{
    static_assert(sizeof(weighted_segment3<T>) == 7 * sizeof(T));
    auto const* v = cuda::detail::raw(vertices);
    auto const* i = reinterpret_cast<std::int32_t const*>(indices.data());
    auto run = [&](weighted_segment3<T>* out, std::int64_t cap, std::int64_t* n)
    {
        if constexpr (std::is_same_v<T, double>)
            cuda::check(agwn_build_boundary_segments_f64(dispatcher.handle(), v, std::int64_t(vertices.size()), i,
                                                         std::int64_t(indices.size()),
                                                         reinterpret_cast<double*>(out), cap, n),
                        "build_boundary_segments");
        else
            cuda::check(agwn_build_boundary_segments_f32(dispatcher.handle(), v, std::int64_t(vertices.size()), i,
                                                         std::int64_t(indices.size()),
                                                         reinterpret_cast<float*>(out), cap, n),
                        "build_boundary_segments");
    };
    std::int64_t n = 0;
    run(nullptr, 0, &n);
    std::vector<weighted_segment3<T>> out(static_cast<std::size_t>(n));
    if (n > 0)
        run(out.data(), n, &n);
    return out;
}

// gwn_mesh_robust.hh:441-456 on the GPU: out_wnrs[i] = robust.eval(positions[i]).
template <class T, class Precision>
void eval_gwnr_mesh_batch_robust(cuda::CudaDispatcher&, cuda::CudaRobustMeshGwn<T, Precision> const& robust,
                                 std::span<vec3<T> const> positions, std::span<T> out_wnrs)
{
    cuda::detail::same_size(positions.size(), out_wnrs.size(), "eval_gwnr_mesh_batch_robust");
    robust.evaluate(positions, out_wnrs);
}

// gwn_parametric.hh:168-186 on the GPU, for cubic Bezier boundaries and the default IntegratorGK15: the same
// value bit for bit.  A non-template function, so it is preferred over the reference's template.
inline void eval_gwnr_parametric_batch_fractional(cuda::CudaDispatcher& dispatcher,
                                                  std::span<vec3<double> const> positions, std::span<double> out_wnrs,
                                                  vec3<double> x0, cuda::CubicBezierBoundary const& boundary,
                                                  integrate_config const& cfg = {})
{
    cuda::detail::same_size(positions.size(), out_wnrs.size(), "eval_gwnr_parametric_batch_fractional");
    static_assert(sizeof(std::array<vec3<double>, 4>) == 12 * sizeof(double));
    double const x[3] = {x0.x, x0.y, x0.z};
    cuda::check(agwn_param_batch_fractional_bezier3_f64(
                    dispatcher.handle(), cuda::detail::raw(positions), std::int64_t(positions.size()),
                    out_wnrs.data(), x, reinterpret_cast<double const*>(boundary.curves.data()),
                    std::int64_t(boundary.curves.size()), cfg.min_depth, cfg.max_depth, cfg.tol, nullptr, nullptr,
                    nullptr),
                "eval_gwnr_parametric_batch_fractional");
}

// The same with the learned start-depth proposal as the integrator.
inline void eval_gwnr_parametric_batch_fractional(cuda::CudaDispatcher& dispatcher,
                                                  std::span<vec3<double> const> positions, std::span<double> out_wnrs,
                                                  vec3<double> x0, cuda::CubicBezierBoundary const& boundary,
                                                  integrate_config const& cfg,
                                                  cuda::LearnedGK15Proposal const& integrator)
{
    cuda::detail::same_size(positions.size(), out_wnrs.size(), "eval_gwnr_parametric_batch_fractional");
    double const x[3] = {x0.x, x0.y, x0.z};
    cuda::check(agwn_param_batch_fractional_learned_bezier3_f64(
                    dispatcher.handle(), integrator.handle(), cuda::detail::raw(positions),
                    std::int64_t(positions.size()), out_wnrs.data(), x,
                    reinterpret_cast<double const*>(boundary.curves.data()), std::int64_t(boundary.curves.size()),
                    integrator.n_classes(), cfg.min_depth, cfg.max_depth, cfg.tol, integrator.alpha(), nullptr,
                    nullptr),
                "eval_gwnr_parametric_batch_fractional");
}
// gwn_parametric.hh:210-226 on the GPU with the Bezier-patch intersector.
inline void eval_gwnr_parametric_batch_integer(cuda::CudaDispatcher& dispatcher,
                                               cuda::CudaBezierPatchIntersector const& intersector,
                                               std::span<vec3<double> const> positions, std::span<int> out_counts,
                                               vec3<double> x0)
{
    cuda::detail::same_size(positions.size(), out_counts.size(), "eval_gwnr_parametric_batch_integer");
    static_assert(sizeof(int) == sizeof(std::int32_t));
    double const x[3] = {x0.x, x0.y, x0.z};
    cuda::check(agwn_param_batch_integer_bezier3x3_f64(dispatcher.handle(), intersector.handle(),
                                                       cuda::detail::raw(positions), std::int64_t(positions.size()),
                                                       reinterpret_cast<std::int32_t*>(out_counts.data()), x),
                "eval_gwnr_parametric_batch_integer");
}

// gwn_parametric.hh:259-284 on the GPU: the fractional term over the cubic Bezier boundary (plain GK15) plus the
// patches' crossing count, per point.
inline void eval_gwnr_parametric_batch(cuda::CudaDispatcher& dispatcher,
                                       cuda::CudaBezierPatchIntersector const& intersector,
                                       std::span<vec3<double> const> positions, std::span<double> out_wnrs,
                                       vec3<double> x0, cuda::CubicBezierBoundary const& boundary,
                                       integrate_config const& cfg = {})
{
    eval_gwnr_parametric_batch_fractional(dispatcher, positions, out_wnrs, x0, boundary, cfg);
    double const x[3] = {x0.x, x0.y, x0.z};
    cuda::check(agwn_param_add_integer_bezier3x3_f64(dispatcher.handle(), intersector.handle(),
                                                     cuda::detail::raw(positions), std::int64_t(positions.size()),
                                                     out_wnrs.data(), x),
                "eval_gwnr_parametric_batch");
}

// The same with the learned start-depth proposal as the integrator.
inline void eval_gwnr_parametric_batch(cuda::CudaDispatcher& dispatcher,
                                       cuda::CudaBezierPatchIntersector const& intersector,
                                       std::span<vec3<double> const> positions, std::span<double> out_wnrs,
                                       vec3<double> x0, cuda::CubicBezierBoundary const& boundary,
                                       integrate_config const& cfg, cuda::LearnedGK15Proposal const& integrator)
{
    eval_gwnr_parametric_batch_fractional(dispatcher, positions, out_wnrs, x0, boundary, cfg, integrator);
    double const x[3] = {x0.x, x0.y, x0.z};
    cuda::check(agwn_param_add_integer_bezier3x3_f64(dispatcher.handle(), intersector.handle(),
                                                     cuda::detail::raw(positions), std::int64_t(positions.size()),
                                                     out_wnrs.data(), x),
                "eval_gwnr_parametric_batch");
}
} // namespace antipodal
