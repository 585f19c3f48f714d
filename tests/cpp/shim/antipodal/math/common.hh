// Test stand-in for the antipodal reference's value types (src/antipodal/math/common.hh of that project), for
// building tests/cpp/frontend_run.cc where the reference's headers are not installed.  Same member layout: the
// front end passes spans of these straight to the C ABI.  Only what the front-end test uses is defined.
#pragma once

#include <cmath>
#include <numbers>
#include <span>

namespace antipodal
{
template <class T>
struct vec3
{
    T x{}, y{}, z{};
    friend constexpr vec3 operator/(vec3 a, T s) { return {a.x / s, a.y / s, a.z / s}; }
};
using fvec3 = vec3<float>;
using dvec3 = vec3<double>;

template <class T>
struct segment3
{
    vec3<T> pos0, pos1;
};
template <class T>
struct weighted_segment3
{
    segment3<T> segment;
    T weight;
};
using weighted_fsegment3 = weighted_segment3<float>;
using weighted_dsegment3 = weighted_segment3<double>;

template <class T>
vec3<T> normalize(vec3<T> a)
{
    return a / std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
}
} // namespace antipodal
