// Double-float arithmetic: a value is hi + lo, two floats with |lo| <= ulp(hi) / 2, about 44 significant bits,
// computed on the FP32 pipe (64x the FP64 rate of this GPU).  Built from the error-free transformations TwoSum
// (Knuth), FastTwoSum (Dekker, |a| >= |b|) and TwoProduct by FMA; add is the "sloppy" variant (error relative to
// |a| + |b|), multiply folds the cross terms into the FMA error term, divide takes two Newton-style corrections of
// a float estimate and sqrt one.  Every step is written with explicit round-to-nearest intrinsics so the compiler
// cannot reassociate or contract them.
#pragma once

#include <cuda_runtime.h>

#include "approx.cuh"

namespace agwn
{
struct df
{
    float hi, lo;
};

__device__ __forceinline__ df df_from(double d)
{
    float const h = __double2float_rn(d);
    return {h, __double2float_rn(d - double(h))};
}
__device__ __forceinline__ double df_to(df a)
{
    return double(a.hi) + double(a.lo);
}
__device__ __forceinline__ df df_make(float hi)
{
    return {hi, 0.f};
}

__device__ __forceinline__ df fast_two_sum(float a, float b)
{
    float const s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df two_sum(float a, float b)
{
    float const s = __fadd_rn(a, b);
    float const bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ df two_prod(float a, float b)
{
    float const p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ df df_neg(df a)
{
    return {-a.hi, -a.lo};
}
__device__ __forceinline__ df operator+(df a, df b)
{
    df const s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ df operator-(df a, df b)
{
    return a + df_neg(b);
}
__device__ __forceinline__ df operator*(df a, df b)
{
    df const p = two_prod(a.hi, b.hi);
    float const e = __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.lo, p.lo));
    return fast_two_sum(p.hi, e);
}
// exact scaling by a power of two
__device__ __forceinline__ df df_scale(df a, float p2)
{
    return {__fmul_rn(a.hi, p2), __fmul_rn(a.lo, p2)};
}
__device__ __forceinline__ df operator/(df a, df b)
{
    float const rb = rcp_approx(b.hi); // one reciprocal for the three float quotients
    float const q1 = __fmul_rn(a.hi, rb);
    df const r = a - b * df_make(q1);
    float const q2 = __fmul_rn(r.hi, rb);
    df const q = fast_two_sum(q1, q2);
    df const r2 = a - b * q; // a second correction brings the quotient to double-float accuracy
    return q + df_make(__fmul_rn(r2.hi, rb));
}
__device__ __forceinline__ df df_sqrt(df a)
{
    if (!(a.hi > 0.f))
        return {sqrtf(a.hi), 0.f};
    float const ri = rsqrt_approx(a.hi);
    float const y = __fmul_rn(a.hi, ri);
    df const e = a - two_prod(y, y);
    return fast_two_sum(y, __fmul_rn(__fmul_rn(e.hi, ri), 0.5f));
}

struct df3
{
    df x, y, z;
};
__device__ __forceinline__ df3 operator-(df3 a, df3 b)
{
    return {a.x - b.x, a.y - b.y, a.z - b.z};
}
__device__ __forceinline__ df3 operator*(df3 a, df s)
{
    return {a.x * s, a.y * s, a.z * s};
}
__device__ __forceinline__ df dot(df3 a, df3 b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
__device__ __forceinline__ df3 cross(df3 a, df3 b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
} // namespace agwn
