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

#include <antipodal_gb300.h>

#include <cstdint>
#include <mutex>
#include <span>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>

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
} // namespace antipodal
