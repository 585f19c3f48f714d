// Shared device side of the learned GK15 proposal: the network's layout and its tensor-core forward pass
// (mma.sync m16n8k16, BF16 operands, FP32 accumulation), and the geometric features of a (query, curve) pair or of
// one panel of it.  Used by mlp.cu (training and the per-pair start depth) and param.cu (the per-panel decision
// inside the integrator).
#pragma once

#include "agwn_internal.cuh"

#include <cuda_bf16.h>

namespace agwn
{
namespace
{
constexpr int kF = 12;  // features
constexpr int kFP = 16; // padded input width
constexpr int kH = 64;  // hidden width
constexpr int kC = 16;  // output width (classes, <= 16)

// FP32 parameter blob: W1t[kH][kFP], b1[kH], W2t[kH][kH], b2[kH], W3t[kC][kH], b3[kC] (W*t = [out][in])
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kH * kFP;
constexpr int kOffW2 = kOffB1 + kH;
constexpr int kOffB2 = kOffW2 + kH * kH;
constexpr int kOffW3 = kOffB2 + kH;
constexpr int kOffB3 = kOffW3 + kC * kH;
constexpr int kParams = kOffB3 + kC;

// BF16 weight copies: the forward layouts ([out][in], pairs along `in`) and the backward ones ([in][out], pairs
// along `out`), in this order.
constexpr int kBW1t = 0;
constexpr int kBW2t = kBW1t + kH * kFP;
constexpr int kBW3t = kBW2t + kH * kH;
constexpr int kBW2n = kBW3t + kC * kH;
constexpr int kBW3n = kBW2n + kH * kH;
constexpr int kBWCount = kBW3n + kH * kC;

// Shared-memory row strides in 32-bit words, padded so that a fragment load (8 rows x 4 words) hits 32 banks.
constexpr int kS16 = 12; // rows of 16 bf16
constexpr int kS64 = 36; // rows of 64 bf16

constexpr int kChunk = 128;           // training samples per block pass (8 warps x 16)
constexpr int kSA = kChunk / 2 + 4;   // words per transposed activation row (128 bf16 + padding)
constexpr int kActRows = kFP + 4 * kH + kC; // X, H1, H2, dZ1, dZ2, dZ3

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 const v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Shared-memory copy of the BF16 forward weights (padded rows) and the FP32 biases; the backward layouts are a
// separate block that only training needs.
struct WeightsSmem
{
    uint32_t w1t[kH * kS16];
    uint32_t w2t[kH * kS64];
    uint32_t w3t[kC * kS64];
    float b1[kH], b2[kH], b3[kC];
};
struct BackWeightsSmem
{
    uint32_t w2n[kH * kS64];
    uint32_t w3n[kH * kS16];
};

__device__ __forceinline__ void smem_copy_rows(uint32_t* dst, const __nv_bfloat16* wb, int off, int rows, int cols,
                                               int stride)
{
    const uint32_t* src = reinterpret_cast<const uint32_t*>(wb + off);
    int const wpr = cols / 2;
    for (int e = threadIdx.x; e < rows * wpr; e += blockDim.x)
        dst[(e / wpr) * stride + e % wpr] = src[e];
}

__device__ void load_weights(WeightsSmem& s, const __nv_bfloat16* wb, const float* params)
{
    smem_copy_rows(s.w1t, wb, kBW1t, kH, kFP, kS16);
    smem_copy_rows(s.w2t, wb, kBW2t, kH, kH, kS64);
    smem_copy_rows(s.w3t, wb, kBW3t, kC, kH, kS64);
    for (int e = threadIdx.x; e < kH; e += blockDim.x)
    {
        s.b1[e] = params[kOffB1 + e];
        s.b2[e] = params[kOffB2 + e];
    }
    for (int e = threadIdx.x; e < kC; e += blockDim.x)
        s.b3[e] = params[kOffB3 + e];
}

__device__ void load_back_weights(BackWeightsSmem& s, const __nv_bfloat16* wb)
{
    smem_copy_rows(s.w2n, wb, kBW2n, kH, kH, kS64);
    smem_copy_rows(s.w3n, wb, kBW3n, kH, kC, kS16);
}

// Forward pass of one m16 tile of samples; a0 is the input fragment (16 samples x 16 features).
// z1, z2: pre-activations of the hidden layers, z3: logits, all as m16n8 accumulator fragments.
__device__ __forceinline__ void mlp_forward(const WeightsSmem& s, const uint32_t (&a0)[4], float (&z1)[8][4],
                                            float (&z2)[8][4], float (&z3)[2][4])
{
    int const lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
    {
        int const n0 = nt * 8 + tig * 2;
        z1[nt][0] = z1[nt][2] = s.b1[n0];
        z1[nt][1] = z1[nt][3] = s.b1[n0 + 1];
        uint32_t const* w = s.w1t + (nt * 8 + g) * kS16;
        mma_bf16(z1[nt], a0[0], a0[1], a0[2], a0[3], w[tig], w[4 + tig]);
    }
    uint32_t a1[4][4];
#pragma unroll
    for (int kt = 0; kt < 4; ++kt)
    {
        a1[kt][0] = pack_bf16(fmaxf(z1[2 * kt][0], 0.f), fmaxf(z1[2 * kt][1], 0.f));
        a1[kt][1] = pack_bf16(fmaxf(z1[2 * kt][2], 0.f), fmaxf(z1[2 * kt][3], 0.f));
        a1[kt][2] = pack_bf16(fmaxf(z1[2 * kt + 1][0], 0.f), fmaxf(z1[2 * kt + 1][1], 0.f));
        a1[kt][3] = pack_bf16(fmaxf(z1[2 * kt + 1][2], 0.f), fmaxf(z1[2 * kt + 1][3], 0.f));
    }
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
    {
        int const n0 = nt * 8 + tig * 2;
        z2[nt][0] = z2[nt][2] = s.b2[n0];
        z2[nt][1] = z2[nt][3] = s.b2[n0 + 1];
        uint32_t const* w = s.w2t + (nt * 8 + g) * kS64;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt)
            mma_bf16(z2[nt], a1[kt][0], a1[kt][1], a1[kt][2], a1[kt][3], w[kt * 8 + tig], w[kt * 8 + 4 + tig]);
    }
    uint32_t a2[4][4];
#pragma unroll
    for (int kt = 0; kt < 4; ++kt)
    {
        a2[kt][0] = pack_bf16(fmaxf(z2[2 * kt][0], 0.f), fmaxf(z2[2 * kt][1], 0.f));
        a2[kt][1] = pack_bf16(fmaxf(z2[2 * kt][2], 0.f), fmaxf(z2[2 * kt][3], 0.f));
        a2[kt][2] = pack_bf16(fmaxf(z2[2 * kt + 1][0], 0.f), fmaxf(z2[2 * kt + 1][1], 0.f));
        a2[kt][3] = pack_bf16(fmaxf(z2[2 * kt + 1][2], 0.f), fmaxf(z2[2 * kt + 1][3], 0.f));
    }
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
    {
        int const n0 = nt * 8 + tig * 2;
        z3[nt][0] = z3[nt][2] = s.b3[n0];
        z3[nt][1] = z3[nt][3] = s.b3[n0 + 1];
        uint32_t const* w = s.w3t + (nt * 8 + g) * kS64;
#pragma unroll
        for (int kt = 0; kt < 4; ++kt)
            mma_bf16(z3[nt], a2[kt][0], a2[kt][1], a2[kt][2], a2[kt][3], w[kt * 8 + tig], w[kt * 8 + 4 + tig]);
    }
}

// ---- features ------------------------------------------------------------------------------------------------

__device__ __forceinline__ float3 f3sub(float3 a, float3 b)
{
    return make_float3(a.x - b.x, a.y - b.y, a.z - b.z);
}
__device__ __forceinline__ float f3dot(float3 a, float3 b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
__device__ __forceinline__ float f3len(float3 a)
{
    return sqrtf(f3dot(a, a));
}
__device__ __forceinline__ float f3angle(float3 a, float3 b)
{
    float3 const c = make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
    return atan2f(f3len(c), f3dot(a, b));
}
// distance from the origin to segment [a, b], and the segment parameter of the nearest point
__device__ __forceinline__ float seg_dist0(float3 a, float3 b, float* tpar)
{
    float3 const e = f3sub(b, a);
    float const ee = f3dot(e, e);
    float t = ee > 0.f ? -f3dot(a, e) / ee : 0.f;
    t = fminf(fmaxf(t, 0.f), 1.f);
    *tpar = t;
    return f3len(make_float3(a.x + t * e.x, a.y + t * e.y, a.z + t * e.z));
}
__device__ __forceinline__ float flog2(float v)
{
    return log2f(fmaxf(v, 1e-30f)) * 0.125f;
}

// The 12 features of a (query, curve) pair, from the control polygon r_i = c_i - p (relative to the query):
//  0 log2(polygon distance / L)   1 log2(nearest control point / L)   2 log2(farthest control point / L)
//  3 log2(L)                      4 chord / L                         5 control-point offset from the chord / L
//  6 polygon turning / pi         7 angle the polygon subtends at p / pi
//  8 log2(distance of the polygon from the line p + t x0, / L)   9 log2(that distance / polygon distance)
// 10 axial cosine of the polygon point nearest that line      11 log10(tol) / 10
// (logs are /8; L = polygon length).  The integrand is steep where the curve passes close to p and where it
// passes close to the line through p along x0, where w and d_eta change fast.
__device__ __forceinline__ void rel_features(const float3 (&r)[4], float3 x0, float tol_feat, float* f)
{
    float L = 0.f;
    float3 e[3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
    {
        e[i] = f3sub(r[i + 1], r[i]);
        L += f3len(e[i]);
    }
    L = fmaxf(L, 1e-30f);
    float dpoly = 3e38f, t;
#pragma unroll
    for (int i = 0; i < 3; ++i)
        dpoly = fminf(dpoly, seg_dist0(r[i], r[i + 1], &t));
    float nmin = 3e38f, nmax = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i)
    {
        float const n = f3len(r[i]);
        nmin = fminf(nmin, n);
        nmax = fmaxf(nmax, n);
    }
    float3 const ch = f3sub(r[3], r[0]);
    float const chord = f3len(ch);
    float flat = 0.f;
#pragma unroll
    for (int i = 1; i <= 2; ++i)
    {
        float3 const a = f3sub(r[0], r[i]), b = f3sub(r[3], r[i]);
        flat = fmaxf(flat, seg_dist0(a, b, &t));
    }
    float const turning = f3angle(e[0], e[1]) + f3angle(e[1], e[2]);
    float const subt = f3angle(r[0], r[1]) + f3angle(r[1], r[2]) + f3angle(r[2], r[3]);
    float3 u[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
    {
        float const a = f3dot(r[i], x0);
        u[i] = make_float3(r[i].x - a * x0.x, r[i].y - a * x0.y, r[i].z - a * x0.z);
    }
    float dline = 3e38f, axial = 0.f;
#pragma unroll
    for (int i = 0; i < 3; ++i)
    {
        float const d = seg_dist0(u[i], u[i + 1], &t);
        if (d < dline)
        {
            dline = d;
            float3 const q = make_float3(r[i].x + t * e[i].x, r[i].y + t * e[i].y, r[i].z + t * e[i].z);
            axial = f3dot(q, x0) / fmaxf(f3len(q), 1e-30f);
        }
    }
    float const kInvPi = 0.31830988618379067f;
    f[0] = flog2(dpoly / L);
    f[1] = flog2(nmin / L);
    f[2] = flog2(nmax / L);
    f[3] = flog2(L);
    f[4] = chord / L;
    f[5] = flat / L;
    f[6] = turning * kInvPi;
    f[7] = subt * kInvPi;
    f[8] = flog2(dline / L);
    f[9] = flog2(fmaxf(dline, 1e-30f) / fmaxf(dpoly, 1e-30f));
    f[10] = axial;
    f[11] = tol_feat;
#pragma unroll
    for (int i = 0; i < kF; ++i)
        f[i] = fminf(fmaxf(f[i], -8.f), 8.f);
}

__device__ __forceinline__ void pair_features(const double* c, double px, double py, double pz, float3 x0,
                                              float tol_feat, float* f)
{
    float3 r[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        r[i] = make_float3(float(c[3 * i] - px), float(c[3 * i + 1] - py), float(c[3 * i + 2] - pz));
    rel_features(r, x0, tol_feat, f);
}

// The control points of the piece [a, b] of the cubic with control points cp (relative to the query, xyz per
// point): the ends B(a), B(b) and the inner points B(a) + (b - a)/3 B'(a), B(b) - (b - a)/3 B'(b).
__device__ __forceinline__ void subcurve(const float (&cp)[12], float a, float b, float3 (&r)[4])
{
    float ba[4], bb[4], da[4], db[4];
    auto basis = [](float t, float* B, float* D)
    {
        float const u = 1.f - t;
        B[0] = u * u * u;
        B[1] = 3.f * u * u * t;
        B[2] = 3.f * u * t * t;
        B[3] = t * t * t;
        D[0] = -3.f * u * u;
        D[1] = 3.f * u * u - 6.f * u * t;
        D[2] = 6.f * u * t - 3.f * t * t;
        D[3] = 3.f * t * t;
    };
    basis(a, ba, da);
    basis(b, bb, db);
    float const k = (b - a) * (1.f / 3.f);
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
        float pa = 0.f, pb = 0.f, ta = 0.f, tb = 0.f;
#pragma unroll
        for (int i = 0; i < 4; ++i)
        {
            pa = fmaf(ba[i], cp[3 * i + c], pa);
            pb = fmaf(bb[i], cp[3 * i + c], pb);
            ta = fmaf(da[i], cp[3 * i + c], ta);
            tb = fmaf(db[i], cp[3 * i + c], tb);
        }
        float* const r0 = &r[0].x;
        float* const r1 = &r[1].x;
        float* const r2 = &r[2].x;
        float* const r3 = &r[3].x;
        r0[c] = pa;
        r1[c] = fmaf(k, ta, pa);
        r2[c] = fmaf(-k, tb, pb);
        r3[c] = pb;
    }
}

// Features of the panel [j 2^-d, (j + 1) 2^-d] of a pair: the pair features of that piece of the curve, with the
// panel's own tolerance (tol 2^-d) in place of tol.
__device__ __forceinline__ void panel_features(const float (&cp)[12], int d, uint32_t j, float3 x0, float log10_tol,
                                               float* f)
{
    float const scale = ldexpf(1.f, -d);
    float3 r[4];
    subcurve(cp, float(j) * scale, float(j + 1) * scale, r);
    rel_features(r, x0, (log10_tol - 0.30103f * float(d)) * 0.1f, f);
}

} // namespace
} // namespace agwn
