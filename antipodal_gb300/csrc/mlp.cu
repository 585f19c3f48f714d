// Learned GK15 depth proposal for the parametric path: a 12 -> 64 -> 64 -> 16 MLP that predicts, for each
// (query, boundary curve) pair, the shallowest depth at which the plain adaptive integrator
// (src/antipodal/math/integrate_gk15.hh:63-290) accepts a panel.  The proposal only says where the integrator
// starts evaluating: panels above the proposed depth are split unevaluated, every evaluated panel is accepted or
// split by the plain |Ik - Ig| <= tol 2^-depth test, so the plain method decides every panel (param.cu).  No
// counterpart in the reference.
//
// All three layers run on the tensor cores (mma.sync m16n8k16, BF16 operands, FP32 accumulation): inference,
// the training forward pass, the backward pass (dH = dZ W^T) and the weight gradients (dW = dZ^T H over the
// batch).  Activations stay in registers between layers (an m16n8 accumulator fragment is, two n-tiles at a
// time, the next layer's m16k16 operand fragment); the weight-gradient products read the batch's activations
// and output gradients transposed through shared memory.  Training is Adam on FP32 master weights; each step's
// two launches are captured once in a CUDA graph and replayed.

#include "mlp.cuh"

#include <cuda_bf16.h>

#include <cmath>
#include <vector>

namespace agwn
{
namespace
{
// Features and labels of logged panels: entry = (pair index, (depth << 25) | (j << 1) | accepted).
__global__ void k_panel_features(const double* __restrict__ pos, float x0x, float x0y, float x0z,
                                 const double* __restrict__ curves, int64_t n_curves, float log10_tol,
                                 const uint32_t* __restrict__ log, int64_t n_entries, float* __restrict__ feats,
                                 uint8_t* __restrict__ labels)
{
    float3 const x0 = make_float3(x0x, x0y, x0z);
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < n_entries;
         e += int64_t(gridDim.x) * blockDim.x)
    {
        int64_t const pair = log[2 * e];
        uint32_t const w = log[2 * e + 1];
        int const d = int(w >> 25);
        uint32_t const j = (w >> 1) & 0xffffffu;
        int64_t const q = pair / n_curves, c = pair - q * n_curves;
        float cp[12];
#pragma unroll
        for (int i = 0; i < 12; ++i)
            cp[i] = float(curves[12 * c + i] - pos[3 * q + i % 3]);
        float f[kF];
        panel_features(cp, d, j, x0, log10_tol, f);
#pragma unroll
        for (int i = 0; i < kF; ++i)
            feats[e * kF + i] = f[i];
        if (labels)
            labels[e] = uint8_t(w & 1u);
    }
}

__global__ void k_features(const double* __restrict__ pos, int64_t n, float x0x, float x0y, float x0z,
                           const double* __restrict__ curves, int64_t n_curves, float tol_feat,
                           float* __restrict__ feats)
{
    float3 const x0 = make_float3(x0x, x0y, x0z);
    int64_t const total = n * n_curves;
    for (int64_t pair = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; pair < total;
         pair += int64_t(gridDim.x) * blockDim.x)
    {
        int64_t const q = pair / n_curves, c = pair - q * n_curves;
        float f[kF];
        pair_features(curves + 12 * c, pos[3 * q], pos[3 * q + 1], pos[3 * q + 2], x0, tol_feat, f);
#pragma unroll
        for (int i = 0; i < kF; ++i)
            feats[pair * kF + i] = f[i];
    }
}

// ---- inference: features -> logits -> start depth ---------------------------------------------------------------

// The largest start depth s whose predicted probability of a shallower first leaf, P(label < s), is <= alpha;
// then at least min_depth (no leaf is accepted above it) and at most max_depth.
__device__ __forceinline__ int decide_depth(const float* logits, int n_classes, float alpha, int min_depth,
                                            int max_depth)
{
    float m = -3e38f;
    for (int c = 0; c < n_classes; ++c)
        m = fmaxf(m, logits[c]);
    float e[kC], sum = 0.f;
    for (int c = 0; c < n_classes; ++c)
    {
        e[c] = __expf(logits[c] - m);
        sum += e[c];
    }
    float const lim = alpha * sum;
    float cdf = 0.f;
    int s = 0;
    for (int c = 0; c < n_classes - 1; ++c)
    {
        cdf += e[c];
        if (cdf > lim)
            break;
        s = c + 1;
    }
    return min(max(s, min_depth), max_depth);
}

constexpr int kInferWarps = 8;
struct InferSmem
{
    WeightsSmem w;
    uint32_t feat[kInferWarps][32][kS16 - 4 + 1]; // 16 bf16 per row (8 words) + 1 word padding
    float logit[kInferWarps][32][kC + 1];
};

__global__ void __launch_bounds__(kInferWarps * 32) k_propose(const __nv_bfloat16* __restrict__ wb,
                                                              const float* __restrict__ params,
                                                              const double* __restrict__ pos, int64_t n, float x0x,
                                                              float x0y, float x0z, const double* __restrict__ curves,
                                                              int64_t n_curves, float tol_feat, int n_classes,
                                                              float alpha, int min_depth, int max_depth,
                                                              uint8_t* __restrict__ start_depth,
                                                              float* __restrict__ logits_out)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    InferSmem& s = *reinterpret_cast<InferSmem*>(smem_raw);
    load_weights(s.w, wb, params);
    __syncthreads();
    int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
    float3 const x0 = make_float3(x0x, x0y, x0z);
    int64_t const total = n * n_curves;
    int64_t const n_groups = (total + 31) / 32;
    for (int64_t grp = blockIdx.x * int64_t(kInferWarps) + warp; grp < n_groups;
         grp += int64_t(gridDim.x) * kInferWarps)
    {
        int64_t const pair = grp * 32 + lane;
        float f[kF];
        if (pair < total)
        {
            int64_t const q = pair / n_curves, c = pair - q * n_curves;
            pair_features(curves + 12 * c, pos[3 * q], pos[3 * q + 1], pos[3 * q + 2], x0, tol_feat, f);
        }
        else
        {
#pragma unroll
            for (int i = 0; i < kF; ++i)
                f[i] = 0.f;
        }
        uint32_t* const row = s.feat[warp][lane];
#pragma unroll
        for (int i = 0; i < kF / 2; ++i)
            row[i] = pack_bf16(f[2 * i], f[2 * i + 1]);
        row[6] = 0u;
        row[7] = 0u;
        __syncwarp();
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
        {
            uint32_t a0[4];
            a0[0] = s.feat[warp][mt * 16 + g][tig];
            a0[1] = s.feat[warp][mt * 16 + g + 8][tig];
            a0[2] = s.feat[warp][mt * 16 + g][4 + tig];
            a0[3] = s.feat[warp][mt * 16 + g + 8][4 + tig];
            float z1[8][4], z2[8][4], z3[2][4];
            mlp_forward(s.w, a0, z1, z2, z3);
#pragma unroll
            for (int nt = 0; nt < 2; ++nt)
            {
                int const c0 = nt * 8 + tig * 2;
                s.logit[warp][mt * 16 + g][c0] = z3[nt][0];
                s.logit[warp][mt * 16 + g][c0 + 1] = z3[nt][1];
                s.logit[warp][mt * 16 + g + 8][c0] = z3[nt][2];
                s.logit[warp][mt * 16 + g + 8][c0 + 1] = z3[nt][3];
            }
        }
        __syncwarp();
        if (pair < total)
        {
            const float* lg = s.logit[warp][lane];
            if (start_depth)
                start_depth[pair] = uint8_t(decide_depth(lg, n_classes, alpha, min_depth, max_depth));
            if (logits_out)
                for (int c = 0; c < kC; ++c)
                    logits_out[pair * kC + c] = lg[c];
        }
        __syncwarp();
    }
}

// ---- training: loss and gradients over a batch ------------------------------------------------------------------

struct TrainSmem
{
    WeightsSmem w;
    BackWeightsSmem wback;
    uint32_t act[kActRows][kSA]; // transposed BF16 tiles [feature][sample] of X, H1, H2, dZ1, dZ2, dZ3
    float db[kH + kH + kC];
    float loss;
};
constexpr int kRowX = 0, kRowH1 = kFP, kRowH2 = kFP + kH, kRowDZ1 = kFP + 2 * kH, kRowDZ2 = kFP + 3 * kH,
              kRowDZ3 = kFP + 4 * kH;

__device__ __forceinline__ void put_bf16(uint32_t (*act)[kSA], int row, int col, float v)
{
    reinterpret_cast<__nv_bfloat16*>(act[row])[col] = __float2bfloat16_rn(v);
}

__device__ __forceinline__ uint64_t mix64(uint64_t x)
{
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

// One block pass covers kChunk samples (16 per warp).  Sample s of the batch is data row s (d_step == NULL) or a
// row drawn by hashing (seed, step, s).  Gradients of the mean cross-entropy are added to `grads`; the mean loss
// to loss_hist[step] (or loss_hist[0]).
__global__ void __launch_bounds__(256, 1) k_mlp_grad(const __nv_bfloat16* __restrict__ wb,
                                                     const float* __restrict__ params,
                                                     const float* __restrict__ feats,
                                                     const uint8_t* __restrict__ labels, int64_t n_data, int batch,
                                                     int n_classes, unsigned long long seed,
                                                     const int* __restrict__ d_step, int step_base,
                                                     float* __restrict__ grads, float* __restrict__ loss_hist)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem& s = *reinterpret_cast<TrainSmem*>(smem_raw);
    load_weights(s.w, wb, params);
    load_back_weights(s.wback, wb);
    for (int e = threadIdx.x; e < kH + kH + kC; e += blockDim.x)
        s.db[e] = 0.f;
    if (threadIdx.x == 0)
        s.loss = 0.f;
    int const step = d_step ? *d_step : 0;
    __syncthreads();
    int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
    float const inv_b = 1.f / float(batch);

    // weight-gradient tiles owned by this warp: 48 m16n8 tiles (dW1t 4x2, dW2t 4x8, dW3t 1x8), 6 per warp
    float acc[6][4];
#pragma unroll
    for (int u = 0; u < 6; ++u)
        acc[u][0] = acc[u][1] = acc[u][2] = acc[u][3] = 0.f;

    int const n_chunks = (batch + kChunk - 1) / kChunk;
    for (int ch = blockIdx.x; ch < n_chunks; ch += gridDim.x)
    {
        // ---- forward + backward of this warp's 16 samples, in registers
        int const r0 = ch * kChunk + warp * 16 + g, r1 = r0 + 8; // batch rows of this lane's two sample rows
        bool const v0 = r0 < batch, v1 = r1 < batch;
        auto data_row = [&](int r) -> int64_t
        {
            if (!d_step)
                return r;
            return int64_t(mix64(seed ^ (uint64_t(step) << 32) ^ uint64_t(r)) % uint64_t(n_data));
        };
        int64_t const d0 = v0 ? data_row(r0) : 0, d1 = v1 ? data_row(r1) : 0;
        float x[2][4]; // rows g, g+8: features tig*2, tig*2+1, tig*2+8, tig*2+9
#pragma unroll
        for (int h = 0; h < 2; ++h)
        {
            bool const v = h ? v1 : v0;
            int64_t const d = h ? d1 : d0;
            int const cols[4] = {tig * 2, tig * 2 + 1, tig * 2 + 8, tig * 2 + 9};
#pragma unroll
            for (int e = 0; e < 4; ++e)
                x[h][e] = (v && cols[e] < kF) ? feats[d * kF + cols[e]] : 0.f;
        }
        uint32_t a0[4] = {pack_bf16(x[0][0], x[0][1]), pack_bf16(x[1][0], x[1][1]), pack_bf16(x[0][2], x[0][3]),
                          pack_bf16(x[1][2], x[1][3])};
        float z1[8][4], z2[8][4], z3[2][4];
        mlp_forward(s.w, a0, z1, z2, z3);

        // softmax cross-entropy over the n_classes first logits; each row's 16 logits live in one lane quad
        int const lab0 = v0 ? min(int(labels[d0]), n_classes - 1) : -1;
        int const lab1 = v1 ? min(int(labels[d1]), n_classes - 1) : -1;
        float dz3[2][4];
        float loss_part = 0.f;
#pragma unroll
        for (int h = 0; h < 2; ++h)
        {
            int const lab = h ? lab1 : lab0;
            bool const v = h ? v1 : v0;
            float l[4] = {z3[0][2 * h], z3[0][2 * h + 1], z3[1][2 * h], z3[1][2 * h + 1]};
            int const col[4] = {tig * 2, tig * 2 + 1, 8 + tig * 2, 8 + tig * 2 + 1};
            float m = -3e38f;
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (col[e] < n_classes)
                    m = fmaxf(m, l[e]);
            m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 1));
            m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 2));
            float ex[4], sum = 0.f, zlab = 0.f;
#pragma unroll
            for (int e = 0; e < 4; ++e)
            {
                ex[e] = col[e] < n_classes ? expf(l[e] - m) : 0.f;
                sum += ex[e];
                if (col[e] == lab)
                    zlab = l[e];
            }
            sum += __shfl_xor_sync(0xffffffffu, sum, 1);
            sum += __shfl_xor_sync(0xffffffffu, sum, 2);
            zlab += __shfl_xor_sync(0xffffffffu, zlab, 1);
            zlab += __shfl_xor_sync(0xffffffffu, zlab, 2);
            if (v && tig == 0)
                loss_part += (logf(sum) + m - zlab);
#pragma unroll
            for (int e = 0; e < 4; ++e)
            {
                float const p = ex[e] / sum;
                float const d = v ? (p - (col[e] == lab ? 1.f : 0.f)) * inv_b : 0.f;
                dz3[e >> 1][2 * h + (e & 1)] = d;
            }
        }
        // dH2 = dZ3 W3^T, masked by ReLU'
        float dz2[8][4];
        {
            uint32_t const b0 = pack_bf16(dz3[0][0], dz3[0][1]), b1 = pack_bf16(dz3[0][2], dz3[0][3]),
                           b2 = pack_bf16(dz3[1][0], dz3[1][1]), b3 = pack_bf16(dz3[1][2], dz3[1][3]);
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
            {
                dz2[nt][0] = dz2[nt][1] = dz2[nt][2] = dz2[nt][3] = 0.f;
                uint32_t const* w = s.wback.w3n + (nt * 8 + g) * kS16;
                mma_bf16(dz2[nt], b0, b1, b2, b3, w[tig], w[4 + tig]);
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    dz2[nt][e] = z2[nt][e] > 0.f ? dz2[nt][e] : 0.f;
            }
        }
        // dH1 = dZ2 W2^T, masked by ReLU'
        float dz1[8][4];
        {
            uint32_t a[4][4];
#pragma unroll
            for (int kt = 0; kt < 4; ++kt)
            {
                a[kt][0] = pack_bf16(dz2[2 * kt][0], dz2[2 * kt][1]);
                a[kt][1] = pack_bf16(dz2[2 * kt][2], dz2[2 * kt][3]);
                a[kt][2] = pack_bf16(dz2[2 * kt + 1][0], dz2[2 * kt + 1][1]);
                a[kt][3] = pack_bf16(dz2[2 * kt + 1][2], dz2[2 * kt + 1][3]);
            }
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
            {
                dz1[nt][0] = dz1[nt][1] = dz1[nt][2] = dz1[nt][3] = 0.f;
                uint32_t const* w = s.wback.w2n + (nt * 8 + g) * kS64;
#pragma unroll
                for (int kt = 0; kt < 4; ++kt)
                    mma_bf16(dz1[nt], a[kt][0], a[kt][1], a[kt][2], a[kt][3], w[kt * 8 + tig], w[kt * 8 + 4 + tig]);
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    dz1[nt][e] = z1[nt][e] > 0.f ? dz1[nt][e] : 0.f;
            }
        }

        // ---- stage the transposed BF16 tiles and add the bias gradients
        int const c0 = warp * 16 + g, c1 = c0 + 8; // sample columns of this lane's rows within the chunk
        __syncthreads(); // the previous chunk's weight-gradient products are done with `act`
        {
            int const cols[4] = {tig * 2, tig * 2 + 1, tig * 2 + 8, tig * 2 + 9};
#pragma unroll
            for (int e = 0; e < 4; ++e)
            {
                put_bf16(s.act, kRowX + cols[e], c0, x[0][e]);
                put_bf16(s.act, kRowX + cols[e], c1, x[1][e]);
            }
        }
        auto stage = [&](int row0, const float(*t)[4], int n_tiles, bool relu, float* db)
        {
            for (int nt = 0; nt < n_tiles; ++nt)
            {
                int const n0 = nt * 8 + tig * 2;
                float v[4];
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    v[e] = relu ? fmaxf(t[nt][e], 0.f) : t[nt][e];
                put_bf16(s.act, row0 + n0, c0, v[0]);
                put_bf16(s.act, row0 + n0 + 1, c0, v[1]);
                put_bf16(s.act, row0 + n0, c1, v[2]);
                put_bf16(s.act, row0 + n0 + 1, c1, v[3]);
                if (db)
                {
                    float s0 = v[0] + v[2], s1 = v[1] + v[3];
#pragma unroll
                    for (int o = 4; o < 32; o <<= 1)
                    {
                        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
                        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
                    }
                    if (g == 0)
                    {
                        atomicAdd(db + n0, s0);
                        atomicAdd(db + n0 + 1, s1);
                    }
                }
            }
        };
        stage(kRowH1, z1, 8, true, nullptr);
        stage(kRowH2, z2, 8, true, nullptr);
        stage(kRowDZ1, dz1, 8, false, s.db);
        stage(kRowDZ2, dz2, 8, false, s.db + kH);
        stage(kRowDZ3, dz3, 2, false, s.db + 2 * kH);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
            loss_part += __shfl_xor_sync(0xffffffffu, loss_part, o);
        if (lane == 0)
            atomicAdd(&s.loss, loss_part * inv_b);
        __syncthreads();

        // ---- weight gradients dW^T[out][in] += dZ^T[out][samples] H[samples][in] over the chunk
#pragma unroll
        for (int u = 0; u < 6; ++u)
        {
            int const t = warp + 8 * u;
            int arow, brow;
            if (t < 8)
            {
                arow = kRowDZ1 + (t >> 1) * 16;
                brow = kRowX + (t & 1) * 8;
            }
            else if (t < 40)
            {
                arow = kRowDZ2 + ((t - 8) >> 3) * 16;
                brow = kRowH1 + ((t - 8) & 7) * 8;
            }
            else
            {
                arow = kRowDZ3;
                brow = kRowH2 + (t - 40) * 8;
            }
#pragma unroll
            for (int kt = 0; kt < kChunk / 16; ++kt)
            {
                int const kw = kt * 8 + tig;
                mma_bf16(acc[u], s.act[arow + g][kw], s.act[arow + g + 8][kw], s.act[arow + g][kw + 4],
                         s.act[arow + g + 8][kw + 4], s.act[brow + g][kw], s.act[brow + g][kw + 4]);
            }
        }
    }
    // ---- flush: this block's weight-gradient tiles, bias gradients and loss
#pragma unroll
    for (int u = 0; u < 6; ++u)
    {
        int const t = warp + 8 * u;
        int base, ld, mt, nt;
        if (t < 8)
        {
            base = kOffW1, ld = kFP, mt = t >> 1, nt = t & 1;
        }
        else if (t < 40)
        {
            base = kOffW2, ld = kH, mt = (t - 8) >> 3, nt = (t - 8) & 7;
        }
        else
        {
            base = kOffW3, ld = kH, mt = 0, nt = t - 40;
        }
        int const row = mt * 16 + g, col = nt * 8 + tig * 2;
        atomicAdd(grads + base + row * ld + col, acc[u][0]);
        atomicAdd(grads + base + row * ld + col + 1, acc[u][1]);
        atomicAdd(grads + base + (row + 8) * ld + col, acc[u][2]);
        atomicAdd(grads + base + (row + 8) * ld + col + 1, acc[u][3]);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kH; e += blockDim.x)
    {
        atomicAdd(grads + kOffB1 + e, s.db[e]);
        atomicAdd(grads + kOffB2 + e, s.db[kH + e]);
    }
    for (int e = threadIdx.x; e < kC; e += blockDim.x)
        atomicAdd(grads + kOffB3 + e, s.db[2 * kH + e]);
    if (threadIdx.x == 0)
        atomicAdd(loss_hist + (d_step ? step - step_base : 0), s.loss);
}

// BF16 copies of the FP32 weights in the forward and backward layouts.
__device__ __forceinline__ void write_bf16(__nv_bfloat16* wb, int i, float v)
{
    __nv_bfloat16 const b = __float2bfloat16_rn(v);
    if (i < kOffB1)
    {
        int const o = i / kFP, k = i % kFP;
        wb[kBW1t + o * kFP + k] = b;
    }
    else if (i >= kOffW2 && i < kOffB2)
    {
        int const o = (i - kOffW2) / kH, k = (i - kOffW2) % kH;
        wb[kBW2t + o * kH + k] = b;
        wb[kBW2n + k * kH + o] = b;
    }
    else if (i >= kOffW3 && i < kOffB3)
    {
        int const c = (i - kOffW3) / kH, k = (i - kOffW3) % kH;
        wb[kBW3t + c * kH + k] = b;
        wb[kBW3n + k * kC + c] = b;
    }
}

__global__ void k_mlp_sync_bf16(const float* __restrict__ params, __nv_bfloat16* __restrict__ wb)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kParams; i += gridDim.x * blockDim.x)
        write_bf16(wb, i, params[i]);
}

// Adam on the FP32 master weights (bias-corrected, step t = *d_step + 1), refreshes the BF16 copies, clears the
// gradients; the last block to finish advances *d_step.
__global__ void k_mlp_adam(float* __restrict__ params, float* __restrict__ m1, float* __restrict__ m2,
                           float* __restrict__ grads, __nv_bfloat16* __restrict__ wb, int* d_step,
                           unsigned* d_done, float lr, float beta1, float beta2, float eps)
{
    int const t = *d_step + 1;
    float const c1 = 1.f - powf(beta1, float(t)), c2 = 1.f - powf(beta2, float(t));
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kParams; i += gridDim.x * blockDim.x)
    {
        float const gr = grads[i];
        grads[i] = 0.f;
        float const a = beta1 * m1[i] + (1.f - beta1) * gr;
        float const b = beta2 * m2[i] + (1.f - beta2) * gr * gr;
        m1[i] = a;
        m2[i] = b;
        float const p = params[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
        params[i] = p;
        write_bf16(wb, i, p);
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        __threadfence();
        if (atomicAdd(d_done, 1u) == gridDim.x - 1)
        {
            *d_done = 0u;
            *d_step = t;
        }
    }
}
} // namespace
} // namespace agwn

// ---- C ABI ------------------------------------------------------------------------------------------------------

struct agwn_mlp
{
    int device = 0;
    agwn::DevBuf params, m1, m2, grads, wb, step, loss;
};

using namespace agwn;

namespace
{
int mlp_smem_setup()
{
    AGWN_TRY_CUDA(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(TrainSmem))));
    AGWN_TRY_CUDA(cudaFuncSetAttribute(k_propose, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(InferSmem))));
    return AGWN_OK;
}

int check_mlp(agwn_context* ctx, const agwn_mlp* mlp)
{
    AGWN_CHECK_ARG(ctx && mlp, "null context/network");
    AGWN_CHECK_ARG(ctx->device == mlp->device, "the network lives on device %d, the context on %d", mlp->device,
                   ctx->device);
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    return mlp_smem_setup();
}
} // namespace

extern "C" int agwn_mlp_param_count(void)
{
    return kParams;
}

extern "C" int agwn_mlp_create(agwn_context* ctx, uint64_t seed, agwn_mlp** out)
{
    AGWN_CHECK_ARG(ctx && out, "null argument");
    clear_message();
    *out = nullptr;
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    auto* m = new agwn_mlp;
    m->device = ctx->device;
    int st = AGWN_OK;
    auto fail_free = [&](int s)
    {
        m->params.release(), m->m1.release(), m->m2.release(), m->grads.release(), m->wb.release();
        m->step.release(), m->loss.release();
        delete m;
        return s;
    };
    for (DevBuf* b : {&m->params, &m->m1, &m->m2, &m->grads})
        if ((st = b->reserve(sizeof(float) * kParams)) != AGWN_OK)
            return fail_free(st);
    if ((st = m->wb.reserve(sizeof(__nv_bfloat16) * kBWCount)) != AGWN_OK ||
        (st = m->step.reserve(2 * sizeof(int))) != AGWN_OK)
        return fail_free(st);
    // He-uniform initial weights from a splitmix64 stream, zero biases; the padded input columns stay zero
    std::vector<float> h(kParams, 0.f);
    uint64_t state = seed;
    auto uni = [&]()
    {
        state += 0x9e3779b97f4a7c15ull;
        uint64_t z = state;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        z ^= z >> 31;
        return double(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
    };
    for (int o = 0; o < kH; ++o)
        for (int k = 0; k < kF; ++k)
            h[kOffW1 + o * kFP + k] = float(uni() * std::sqrt(6.0 / kF));
    for (int i = 0; i < kH * kH; ++i)
        h[kOffW2 + i] = float(uni() * std::sqrt(6.0 / kH));
    for (int i = 0; i < kC * kH; ++i)
        h[kOffW3 + i] = float(uni() * std::sqrt(6.0 / kH));
    *out = m;
    return agwn_mlp_set_params(ctx, m, h.data());
}

extern "C" int agwn_mlp_destroy(agwn_mlp* mlp)
{
    if (!mlp)
        return AGWN_OK;
    cudaSetDevice(mlp->device);
    cudaDeviceSynchronize();
    mlp->params.release(), mlp->m1.release(), mlp->m2.release(), mlp->grads.release(), mlp->wb.release();
    mlp->step.release(), mlp->loss.release();
    delete mlp;
    return AGWN_OK;
}

extern "C" int agwn_mlp_set_params(agwn_context* ctx, agwn_mlp* mlp, const float* params)
{
    AGWN_CHECK_ARG(params, "null parameters");
    AGWN_TRY(check_mlp(ctx, mlp));
    clear_message();
    for (int i = 0; i < kParams; ++i)
        AGWN_CHECK_ARG(std::isfinite(params[i]), "parameter %d is not finite", i);
    AGWN_TRY_CUDA(cudaMemcpyAsync(mlp->params.ptr, params, sizeof(float) * kParams, cudaMemcpyHostToDevice,
                                  ctx->stream));
    // the padded input columns of W1 carry no feature: keep them zero
    for (int o = 0; o < kH; ++o)
        AGWN_TRY_CUDA(cudaMemsetAsync(static_cast<float*>(mlp->params.ptr) + kOffW1 + o * kFP + kF, 0,
                                      sizeof(float) * (kFP - kF), ctx->stream));
    AGWN_TRY_CUDA(cudaMemsetAsync(mlp->m1.ptr, 0, sizeof(float) * kParams, ctx->stream));
    AGWN_TRY_CUDA(cudaMemsetAsync(mlp->m2.ptr, 0, sizeof(float) * kParams, ctx->stream));
    AGWN_TRY_CUDA(cudaMemsetAsync(mlp->grads.ptr, 0, sizeof(float) * kParams, ctx->stream));
    AGWN_TRY_CUDA(cudaMemsetAsync(mlp->wb.ptr, 0, sizeof(__nv_bfloat16) * kBWCount, ctx->stream));
    AGWN_TRY_CUDA(cudaMemsetAsync(mlp->step.ptr, 0, 2 * sizeof(int), ctx->stream));
    k_mlp_sync_bf16<<<div_up(kParams, 256), 256, 0, ctx->stream>>>(static_cast<const float*>(mlp->params.ptr),
                                                                 static_cast<__nv_bfloat16*>(mlp->wb.ptr));
    AGWN_TRY_CUDA(cudaGetLastError());
    AGWN_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
    return AGWN_OK;
}

extern "C" int agwn_mlp_get_params(agwn_context* ctx, const agwn_mlp* mlp, float* params)
{
    AGWN_CHECK_ARG(params, "null parameters");
    AGWN_TRY(check_mlp(ctx, mlp));
    clear_message();
    AGWN_TRY_CUDA(cudaMemcpyAsync(params, mlp->params.ptr, sizeof(float) * kParams, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    AGWN_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
    return AGWN_OK;
}

extern "C" int agwn_param_features_bezier3_f64(agwn_context* ctx, const double* positions, int64_t n,
                                               const double* x0, const double* curves, int64_t n_curves, double tol,
                                               float* features)
{
    AGWN_CHECK_ARG(ctx && x0 && n >= 0 && n_curves >= 0, "bad arguments");
    AGWN_CHECK_ARG((n == 0 || n_curves == 0) || (positions && curves && features), "null array");
    AGWN_CHECK_ARG(std::isfinite(tol) && tol > 0, "tol must be finite and > 0");
    clear_message();
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    int64_t const total = n * n_curves;
    if (total == 0)
        return AGWN_OK;
    const void *dpos = nullptr, *dcur = nullptr;
    void* dfeat = nullptr;
    bool h_feat = false;
    AGWN_TRY(stage_in(*ctx, positions, sizeof(double) * 3 * n, S_QUERIES, &dpos));
    AGWN_TRY(stage_in(*ctx, curves, sizeof(double) * 12 * n_curves, S_MISC0, &dcur));
    AGWN_TRY(stage_out(*ctx, features, sizeof(float) * kF * total, S_MISC1, &dfeat, &h_feat));
    AGWN_TRY(ctx->launch_begin(AGWN_K_OTHER));
    k_features<<<int(std::min<int64_t>(div_up(total, 256), 8 * ctx->sm_count)), 256, 0, ctx->stream>>>(
        static_cast<const double*>(dpos), n, float(x0[0]), float(x0[1]), float(x0[2]),
        static_cast<const double*>(dcur), n_curves, float(std::log10(tol) / 10.0), static_cast<float*>(dfeat));
    AGWN_TRY(ctx->launch_end(AGWN_K_OTHER));
    if (h_feat)
        AGWN_TRY_CUDA(cudaMemcpyAsync(features, dfeat, sizeof(float) * kF * total, cudaMemcpyDeviceToHost,
                                      ctx->stream));
    bool const sync = h_feat || dpos != positions || dcur != curves;
    return sync ? ctx->check_flags() : AGWN_OK;
}

extern "C" int agwn_mlp_loss_grad(agwn_context* ctx, const agwn_mlp* mlp, const float* features,
                                  const uint8_t* labels, int64_t n, int n_classes, float* grads, double* loss)
{
    AGWN_TRY(check_mlp(ctx, mlp));
    AGWN_CHECK_ARG(n > 0 && n <= (int64_t(1) << 30) && features && labels && grads && loss, "bad arguments");
    AGWN_CHECK_ARG(n_classes >= 2 && n_classes <= kC, "n_classes must be in [2, %d]", kC);
    clear_message();
    const void *dfeat = nullptr, *dlab = nullptr;
    AGWN_TRY(stage_in(*ctx, features, sizeof(float) * kF * n, S_MISC0, &dfeat));
    AGWN_TRY(stage_in(*ctx, labels, size_t(n), S_MISC1, &dlab));
    void* work = nullptr; // gradient accumulator + loss
    AGWN_TRY(ctx->scratch_reserve(S_MISC2, sizeof(float) * (kParams + 1), &work));
    float* const g = static_cast<float*>(work);
    AGWN_TRY_CUDA(cudaMemsetAsync(g, 0, sizeof(float) * (kParams + 1), ctx->stream));
    int const n_chunks = int(div_up(n, kChunk));
    AGWN_TRY(ctx->launch_begin(AGWN_K_OTHER));
    k_mlp_grad<<<std::min(n_chunks, ctx->sm_count), 256, sizeof(TrainSmem), ctx->stream>>>(
        static_cast<const __nv_bfloat16*>(mlp->wb.ptr), static_cast<const float*>(mlp->params.ptr),
        static_cast<const float*>(dfeat), static_cast<const uint8_t*>(dlab), n, int(n), n_classes, 0ull, nullptr, 0,
        g, g + kParams);
    AGWN_TRY(ctx->launch_end(AGWN_K_OTHER));
    std::vector<float> h(kParams + 1);
    AGWN_TRY_CUDA(cudaMemcpyAsync(h.data(), g, sizeof(float) * (kParams + 1), cudaMemcpyDeviceToHost, ctx->stream));
    AGWN_TRY(ctx->check_flags());
    std::copy(h.begin(), h.begin() + kParams, grads);
    *loss = h[kParams];
    return AGWN_OK;
}

extern "C" int agwn_mlp_train(agwn_context* ctx, agwn_mlp* mlp, const float* features, const uint8_t* labels,
                              int64_t n, int n_classes, int steps, int batch, float lr, uint64_t seed,
                              float* loss_per_step)
{
    AGWN_TRY(check_mlp(ctx, mlp));
    AGWN_CHECK_ARG(n > 0 && features && labels, "bad arguments");
    AGWN_CHECK_ARG(n_classes >= 2 && n_classes <= kC, "n_classes must be in [2, %d]", kC);
    AGWN_CHECK_ARG(steps >= 0 && batch > 0 && batch % kChunk == 0, "batch must be a positive multiple of %d",
                   kChunk);
    AGWN_CHECK_ARG(std::isfinite(lr) && lr > 0, "lr must be > 0");
    clear_message();
    if (steps == 0)
        return AGWN_OK;
    const void *dfeat = nullptr, *dlab = nullptr;
    AGWN_TRY(stage_in(*ctx, features, sizeof(float) * kF * n, S_MISC0, &dfeat));
    AGWN_TRY(stage_in(*ctx, labels, size_t(n), S_MISC1, &dlab));
    AGWN_TRY(mlp->loss.reserve(sizeof(float) * size_t(steps)));
    float* const dloss = static_cast<float*>(mlp->loss.ptr);
    AGWN_TRY_CUDA(cudaMemsetAsync(dloss, 0, sizeof(float) * size_t(steps), ctx->stream));
    int* const dstep = static_cast<int*>(mlp->step.ptr);
    // the loss history is indexed from this call's first step
    int step0 = 0;
    AGWN_TRY_CUDA(cudaMemcpyAsync(&step0, dstep, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    AGWN_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
    int const grid_grad = std::min(batch / kChunk, ctx->sm_count);
    int const grid_adam = div_up(kParams, 256);

    // one training step = gradient launch + Adam launch, captured once and replayed `steps` times
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cap = nullptr;
    AGWN_TRY_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    int st = AGWN_OK;
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess)
    {
        k_mlp_grad<<<grid_grad, 256, sizeof(TrainSmem), cap>>>(
            static_cast<const __nv_bfloat16*>(mlp->wb.ptr), static_cast<const float*>(mlp->params.ptr),
            static_cast<const float*>(dfeat), static_cast<const uint8_t*>(dlab), n, batch, n_classes,
            (unsigned long long)seed, dstep, step0, static_cast<float*>(mlp->grads.ptr), dloss);
        k_mlp_adam<<<grid_adam, 256, 0, cap>>>(static_cast<float*>(mlp->params.ptr), static_cast<float*>(mlp->m1.ptr),
                                               static_cast<float*>(mlp->m2.ptr), static_cast<float*>(mlp->grads.ptr),
                                               static_cast<__nv_bfloat16*>(mlp->wb.ptr), dstep,
                                               reinterpret_cast<unsigned*>(dstep + 1), lr, 0.9f, 0.999f, 1e-8f);
        e = cudaStreamEndCapture(cap, &graph);
    }
    if (e == cudaSuccess)
        e = cudaGraphInstantiate(&exec, graph, 0);
    // the capture stream waits for the staging copies on the context stream, and the context stream for the steps
    cudaEvent_t ev = nullptr;
    if (e == cudaSuccess)
        e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess)
        e = cudaEventRecord(ev, ctx->stream);
    if (e == cudaSuccess)
        e = cudaStreamWaitEvent(cap, ev, 0);
    for (int i = 0; e == cudaSuccess && i < steps; ++i)
        e = cudaGraphLaunch(exec, cap);
    if (e == cudaSuccess)
        e = cudaEventRecord(ev, cap);
    if (e == cudaSuccess)
        e = cudaStreamWaitEvent(ctx->stream, ev, 0);
    if (e == cudaSuccess)
        ctx->launches[AGWN_K_OTHER] += 2 * int64_t(steps);
    if (e == cudaSuccess && loss_per_step)
        e = cudaMemcpyAsync(loss_per_step, dloss, sizeof(float) * size_t(steps), cudaMemcpyDeviceToHost,
                            ctx->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess)
        st = fail(AGWN_ERR_CUDA, "training: %s", cudaGetErrorString(e));
    if (ev)
        cudaEventDestroy(ev);
    if (exec)
        cudaGraphExecDestroy(exec);
    if (graph)
        cudaGraphDestroy(graph);
    cudaStreamDestroy(cap);
    return st != AGWN_OK ? st : ctx->check_flags();
}

namespace agwn
{
void mlp_device_weights(const agwn_mlp* mlp, const void** bf16_weights, const float** params)
{
    *bf16_weights = mlp->wb.ptr;
    *params = static_cast<const float*>(mlp->params.ptr);
}

int mlp_propose_run(Context& ctx, const agwn_mlp* mlp, const double* d_pos, int64_t n, const double* x0,
                    const double* d_curves, int64_t n_curves, int n_classes, int min_depth, int max_depth, double tol,
                    float alpha, uint8_t* d_start, float* d_logits)
{
    AGWN_CHECK_ARG(ctx.device == mlp->device, "the network lives on device %d, the context on %d", mlp->device,
                   ctx.device);
    AGWN_CHECK_ARG(n_classes >= 2 && n_classes <= kC, "n_classes must be in [2, %d]", kC);
    AGWN_CHECK_ARG(alpha >= 0.f && alpha < 1.f, "alpha must be in [0, 1)");
    AGWN_TRY(mlp_smem_setup());
    int64_t const total = n * n_curves;
    if (total == 0)
        return AGWN_OK;
    int per_sm = 0;
    AGWN_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_propose, kInferWarps * 32,
                                                               sizeof(InferSmem)));
    int64_t const n_groups = div_up(total, 32);
    int const grid = int(std::max<int64_t>(1, std::min<int64_t>(div_up(n_groups, kInferWarps),
                                                                int64_t(std::max(per_sm, 1)) * ctx.sm_count)));
    AGWN_TRY(ctx.launch_begin(AGWN_K_PARAMETRIC));
    k_propose<<<grid, kInferWarps * 32, sizeof(InferSmem), ctx.stream>>>(
        static_cast<const __nv_bfloat16*>(mlp->wb.ptr), static_cast<const float*>(mlp->params.ptr), d_pos, n,
        float(x0[0]), float(x0[1]), float(x0[2]), d_curves, n_curves, float(std::log10(tol) / 10.0), n_classes, alpha,
        min_depth, max_depth, d_start, d_logits);
    return ctx.launch_end(AGWN_K_PARAMETRIC);
}
} // namespace agwn

extern "C" int agwn_param_propose_depth_bezier3_f64(agwn_context* ctx, const agwn_mlp* mlp, const double* positions,
                                                    int64_t n, const double* x0, const double* curves,
                                                    int64_t n_curves, int n_classes, int min_depth, int max_depth,
                                                    double tol, float alpha, uint8_t* start_depth, float* logits)
{
    AGWN_TRY(check_mlp(ctx, mlp));
    AGWN_CHECK_ARG(x0 && n >= 0 && n_curves >= 0, "bad arguments");
    AGWN_CHECK_ARG((n == 0 || n_curves == 0) || (positions && curves && (start_depth || logits)), "null array");
    AGWN_CHECK_ARG(min_depth >= 0 && max_depth >= 0 && max_depth <= 255, "bad depths");
    AGWN_CHECK_ARG(std::isfinite(tol) && tol > 0, "bad tol");
    clear_message();
    int64_t const total = n * n_curves;
    if (total == 0)
        return AGWN_OK;
    const void *dpos = nullptr, *dcur = nullptr;
    void *dsd = nullptr, *dlog = nullptr;
    bool h_sd = false, h_log = false;
    AGWN_TRY(stage_in(*ctx, positions, sizeof(double) * 3 * n, S_QUERIES, &dpos));
    AGWN_TRY(stage_in(*ctx, curves, sizeof(double) * 12 * n_curves, S_MISC0, &dcur));
    if (start_depth)
        AGWN_TRY(stage_out(*ctx, start_depth, size_t(total), S_MISC1, &dsd, &h_sd));
    if (logits)
        AGWN_TRY(stage_out(*ctx, logits, sizeof(float) * kC * total, S_MISC2, &dlog, &h_log));
    AGWN_TRY(mlp_propose_run(*ctx, mlp, static_cast<const double*>(dpos), n, x0, static_cast<const double*>(dcur),
                             n_curves, n_classes, min_depth, max_depth, tol, alpha, static_cast<uint8_t*>(dsd),
                             static_cast<float*>(dlog)));
    if (h_sd)
        AGWN_TRY_CUDA(cudaMemcpyAsync(start_depth, dsd, size_t(total), cudaMemcpyDeviceToHost, ctx->stream));
    if (h_log)
        AGWN_TRY_CUDA(cudaMemcpyAsync(logits, dlog, sizeof(float) * kC * total, cudaMemcpyDeviceToHost, ctx->stream));
    bool const sync = h_sd || h_log || dpos != positions || dcur != curves;
    return sync ? ctx->check_flags() : AGWN_OK;
}

extern "C" int agwn_param_panel_features_bezier3_f64(agwn_context* ctx, const double* positions, int64_t n,
                                                     const double* x0, const double* curves, int64_t n_curves,
                                                     double tol, const uint32_t* log, int64_t n_entries,
                                                     float* features, uint8_t* labels)
{
    AGWN_CHECK_ARG(ctx && x0 && n >= 0 && n_curves > 0 && n_entries >= 0, "bad arguments");
    AGWN_CHECK_ARG(n_entries == 0 || (positions && curves && log && features), "null array");
    AGWN_CHECK_ARG(std::isfinite(tol) && tol > 0, "tol must be finite and > 0");
    clear_message();
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    if (n_entries == 0)
        return AGWN_OK;
    const void *dpos = nullptr, *dcur = nullptr, *dlog = nullptr;
    void *dfeat = nullptr, *dlab = nullptr;
    bool h_feat = false, h_lab = false;
    AGWN_TRY(stage_in(*ctx, positions, sizeof(double) * 3 * n, S_QUERIES, &dpos));
    AGWN_TRY(stage_in(*ctx, curves, sizeof(double) * 12 * n_curves, S_MISC0, &dcur));
    AGWN_TRY(stage_in(*ctx, log, sizeof(uint32_t) * 2 * size_t(n_entries), S_SEGS, &dlog));
    AGWN_TRY(stage_out(*ctx, features, sizeof(float) * kF * size_t(n_entries), S_MISC1, &dfeat, &h_feat));
    if (labels)
        AGWN_TRY(stage_out(*ctx, labels, size_t(n_entries), S_MISC2, &dlab, &h_lab));
    AGWN_TRY(ctx->launch_begin(AGWN_K_OTHER));
    k_panel_features<<<int(std::min<int64_t>(div_up(n_entries, 256), 8 * ctx->sm_count)), 256, 0, ctx->stream>>>(
        static_cast<const double*>(dpos), float(x0[0]), float(x0[1]), float(x0[2]), static_cast<const double*>(dcur),
        n_curves, float(std::log10(tol)), static_cast<const uint32_t*>(dlog), n_entries, static_cast<float*>(dfeat),
        static_cast<uint8_t*>(dlab));
    AGWN_TRY(ctx->launch_end(AGWN_K_OTHER));
    if (h_feat)
        AGWN_TRY_CUDA(cudaMemcpyAsync(features, dfeat, sizeof(float) * kF * size_t(n_entries), cudaMemcpyDeviceToHost,
                                      ctx->stream));
    if (h_lab)
        AGWN_TRY_CUDA(cudaMemcpyAsync(labels, dlab, size_t(n_entries), cudaMemcpyDeviceToHost, ctx->stream));
    return ctx->check_flags();
}
