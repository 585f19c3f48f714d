// The FP32 reciprocal and reciprocal square root as single approximate instructions (inline PTX, rcp.approx and
// rsqrt.approx with subnormal inputs flushed to zero): one MUFU operation each, without the subnormal handling that
// the library's __fdividef and rsqrtf carry, and the same rounding in every inlined copy of the code that calls
// them.  A flushed (or zero) input gives an infinite result; the callers' error bounds and range checks turn that
// into a NaN or a rejected pair.
#pragma once

#include <cuda_runtime.h>

namespace agwn
{
__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rsqrt_approx(float x)
{
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
} // namespace agwn
