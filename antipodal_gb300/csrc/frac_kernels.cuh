// Device code of the fractional kernels (segment layouts, the exact and mixed forms, boundary preparation),
// shared by the translation units that launch them.  Everything here has internal linkage, so each including
// unit owns its instantiations.  The design is described at the top of frac.cu.
#pragma once

#include "agwn_internal.cuh"
#include "approx.cuh"
#include "tma.cuh"

#include <type_traits>

#include <climits>
#include <cmath>

namespace agwn
{
namespace
{
template <class T>
struct alignas(16) SegX
{
    T p0x, p0y, p0z, p1x, p1y, p1z, w, pad;
};
// Mixed-mode boundary entry: a vertex and the segment that ends at it, in chain order (k_prep_mixed).
//   segment entry: a = (P1_hi, w), b = (P1 - P0, near2), c = (P1_lo, segment index as bits);
//   chain start:   a = (P0_hi, 0), b = (0, 0, 0, near2), c = (P0_lo, -1 as bits).
// P0 of a segment entry is the vertex of the entry before it.  near2 = (tau * L)^2 with L the longer of the (one or
// two) segments of the chain that meet at the vertex.
struct alignas(16) SegM
{
    float4 a, b, c;
};
struct Rot
{
    double m[9];
};
struct Frame
{
    double c[3];
    long long n_entries; // boundary entries written by k_prep_mixed
};

template <class T>
constexpr T kPi = T(3.141592653589793238462643383279502884L);

// --------------------------------------------------------------------------------------------------------------
// exact form (reference arithmetic)
// --------------------------------------------------------------------------------------------------------------
template <class S>
__device__ __forceinline__ auto vos_exact(ev3<S> x1, ev3<S> v0, ev3<S> v1)
{
    S const l0 = ex_sqrt(edot(v0, v0));
    S const l1 = ex_sqrt(edot(v1, v1));
    S const num = edot(x1, ecross(v0, v1));
    S const den = l0 * l1 + l1 * edot(x1, v0) + l0 * edot(x1, v1) + edot(v0, v1);
    return ex_atan2(num, den);
}

template <class T>
__global__ void k_prep_exact(const T* __restrict__ raw, int64_t n_seg, SegX<T>* __restrict__ out)
{
    for (int64_t s = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; s < n_seg; s += int64_t(gridDim.x) * blockDim.x)
    {
        const T* w = raw + 7 * s;
        out[s] = SegX<T>{w[0], w[1], w[2], w[3], w[4], w[5], w[6], T(0)};
    }
}

// Shared skeleton of both fractional kernels: persistent CTAs over query tiles, segment tiles in shared memory.
// Policy provides: Seg type, per-thread state init (load), per-segment accumulate, and finish (store).
template <class Seg>
struct TilePipe
{
    Seg* buf[2];
    uint64_t* bar;
    const Seg* gseg;
    int64_t n_seg;
    int tile;
    int n_tiles;
    bool single;

    __device__ __forceinline__ int tile_count(int st) const
    {
        int64_t const rem = n_seg - int64_t(st) * tile;
        return int(rem < tile ? rem : tile);
    }
    // Issued by one thread: item `it` of the flattened (query tile, segment tile) sequence into buffer it & 1.
    __device__ __forceinline__ void issue(int it) const
    {
        int const b = it & 1;
        int const st = it % n_tiles;
        unsigned const bytes = unsigned(tile_count(st)) * unsigned(sizeof(Seg));
        mbar_arrive_expect_tx(&bar[b], bytes);
        bulk_copy_g2s(buf[b], gseg + int64_t(st) * tile, bytes, &bar[b]);
    }
};

template <class T, int K>
__global__ void __launch_bounds__(256) k_frac_exact(const T* __restrict__ pos, int64_t n, T* __restrict__ out,
                                                    const int32_t* __restrict__ counts, T x0x, T x0y, T x0z,
                                                    const SegX<T>* __restrict__ seg, int64_t n_seg, int tile,
                                                    int* flags)
{
    using S = typename exact_of<T>::type;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ int abort_cta;

    TilePipe<SegX<T>> pipe;
    pipe.n_tiles = int((n_seg + tile - 1) / tile);
    pipe.single = pipe.n_tiles == 1;
    pipe.buf[0] = reinterpret_cast<SegX<T>*>(smem);
    pipe.buf[1] = pipe.buf[0] + (pipe.single ? 0 : tile);
    pipe.bar = bars;
    pipe.gseg = seg;
    pipe.n_seg = n_seg;
    pipe.tile = tile;

    int64_t const per_tile = int64_t(blockDim.x) * K;
    int64_t const n_qtiles = (n + per_tile - 1) / per_tile;
    int const my_qtiles = blockIdx.x < n_qtiles ? int((n_qtiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;
    int const n_items = pipe.single ? (my_qtiles > 0 ? 1 : 0) : my_qtiles * pipe.n_tiles;

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

    S const x1x = S(-x0x), x1y = S(-x0y), x1z = S(-x0z);
    ev3<S> const x1{x1x, x1y, x1z};
    T const two_pi = T(2) * kPi<T>;

    int it = 0;
    for (int j = 0; j < my_qtiles; ++j)
    {
        int64_t const base = (blockIdx.x + int64_t(j) * gridDim.x) * per_tile + threadIdx.x;
        ev3<S> p[K];
        S area[K];
#pragma unroll
        for (int k = 0; k < K; ++k)
        {
            int64_t const i = base + int64_t(k) * blockDim.x;
            int64_t const ii = i < n ? i : n - 1;
            p[k] = {S(pos[3 * ii]), S(pos[3 * ii + 1]), S(pos[3 * ii + 2])};
            area[k] = S(T(0));
        }
        for (int st = 0; st < pipe.n_tiles; ++st)
        {
            int const b = it & 1;
            if (!pipe.single || j == 0)
            {
                bool ok = mbar_wait_bounded(&bars[b], unsigned((it >> 1) & 1), flags, 1);
                if (!ok)
                    abort_cta = 1;
            }
            __syncthreads();
            if (abort_cta)
                return;
            SegX<T> const* sb = pipe.buf[b];
            int const cnt = pipe.tile_count(st);
            for (int s = 0; s < cnt; ++s)
            {
                SegX<T> const g = sb[s];
                ev3<S> const a{S(g.p0x), S(g.p0y), S(g.p0z)};
                ev3<S> const c{S(g.p1x), S(g.p1y), S(g.p1z)};
                S const w = S(g.w);
#pragma unroll
                for (int k = 0; k < K; ++k)
                {
                    ev3<S> const v0 = a - p[k];
                    ev3<S> const v1 = c - p[k];
                    area[k] = area[k] + w * S(vos_exact(x1, v0, v1));
                }
            }
            if (!pipe.single)
            {
                __syncthreads();
                if (threadIdx.x == 0 && it + 2 < n_items)
                    pipe.issue(it + 2);
                ++it;
            }
        }
#pragma unroll
        for (int k = 0; k < K; ++k)
        {
            int64_t const i = base + int64_t(k) * blockDim.x;
            if (i < n)
            {
                S v = area[k] / S(two_pi);
                if (counts)
                    v = v + S(T(counts[i]));
                out[i] = v.v;
            }
        }
    }
}

// --------------------------------------------------------------------------------------------------------------
// mixed form
// --------------------------------------------------------------------------------------------------------------

// Boundaries of up to this many segments are put in chain order; larger ones take one chain per segment.
constexpr int kChainMax = 4096;

__host__ __device__ constexpr int chain_table_size(int64_t n_seg)
{
    int t = 64;
    while (t < 2 * n_seg && t < 2 * kChainMax)
        t <<= 1;
    return t;
}
__host__ __device__ constexpr int64_t chain_scratch_ints(int64_t n_seg)
{
    return n_seg <= kChainMax ? 4 * n_seg + chain_table_size(n_seg) : 0;
}

// Hash of a point for the link table; +0.0 folds -0.0 into +0.0, which compares equal to it.
__device__ __forceinline__ uint32_t point_hash(double x, double y, double z)
{
    uint64_t const a = uint64_t(__double_as_longlong(x + 0.0)), b = uint64_t(__double_as_longlong(y + 0.0)),
                   c = uint64_t(__double_as_longlong(z + 0.0));
    uint64_t h = a * 0x9E3779B97F4A7C15ull ^ b * 0xC2B2AE3D27D4EB4Full ^ c * 0x165667B19E3779F9ull;
    h ^= h >> 29;
    return uint32_t(h) ^ uint32_t(h >> 32);
}

__device__ __forceinline__ float seg_length(const double* w)
{
    double const ex = w[3] - w[0], ey = w[4] - w[1], ez = w[5] - w[2];
    return float(sqrt(ex * ex + ey * ey + ez * ez));
}

// Chains of ns <= kChainMax segments by exact endpoint equality, in one block (every thread calls it): segment t
// follows s when start(t) == end(s) (all three coordinates), each t following at most one s (the lowest-numbered),
// so the links form disjoint open chains and closed loops.  Writes order[0..m) -- ~s: a chain start at start(s),
// s: segment s, ending at end(s) -- open chains from their first segment, then closed loops from their
// lowest-numbered segment, and wrap[e]: for the first and last entry of a closed loop the segment that closes it
// at that vertex, else -1.  Returns m in every thread.  start(t), end(s): the endpoints as double3 (exact for the
// callers' coordinates).  table: chain_table_size(ns) ints of global scratch; the s_ arrays: kChainMax each.
template <class Start, class End>
__device__ int block_chains(int ns, Start start, End end, int* __restrict__ order, int* __restrict__ wrap,
                            int* __restrict__ table, int* s_succ, int* s_pred, unsigned char* s_seen, int* s_m)
{
    int const tmask = chain_table_size(ns) - 1;
    for (int t = threadIdx.x; t < ns; t += blockDim.x)
    {
        s_pred[t] = INT_MAX;
        s_seen[t] = 0;
        wrap[2 * t] = -1;
        wrap[2 * t + 1] = -1;
    }
    for (int h = threadIdx.x; ns > 0 && h <= tmask; h += blockDim.x)
        table[h] = -1;
    __syncthreads();
    // segment starts into the table (linear probing; at least half of it stays empty), then every segment looks
    // up the lowest-numbered other segment that starts where it ends
    for (int t = threadIdx.x; t < ns; t += blockDim.x)
    {
        double3 const u = start(t);
        uint32_t h = point_hash(u.x, u.y, u.z) & uint32_t(tmask);
        while (atomicCAS(&table[h], -1, t) != -1)
            h = (h + 1) & uint32_t(tmask);
    }
    __syncthreads();
    for (int si = threadIdx.x; si < ns; si += blockDim.x)
    {
        double3 const e = end(si);
        int next = -1;
        for (uint32_t h = point_hash(e.x, e.y, e.z) & uint32_t(tmask);; h = (h + 1) & uint32_t(tmask))
        {
            int const t = __ldcg(&table[h]); // written by atomics: read from L2
            if (t < 0)
                break;
            double3 const u = start(t);
            if (u.x == e.x && u.y == e.y && u.z == e.z && t != si && (next < 0 || t < next))
                next = t;
        }
        s_succ[si] = next;
        if (next >= 0)
            atomicMin(&s_pred[next], si);
    }
    __syncthreads();
    for (int si = threadIdx.x; si < ns; si += blockDim.x)
    {
        int const t = s_succ[si];
        if (t >= 0 && s_pred[t] != si)
            s_succ[si] = -1; // t follows a lower-numbered segment
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        int m = 0;
        // pass 0: open chains from their heads (no predecessor); pass 1: what is left lies on closed loops
        for (int pass = 0; pass < 2; ++pass)
            for (int si = 0; si < ns; ++si)
            {
                if (s_seen[si] || (pass == 0 && s_pred[si] != INT_MAX))
                    continue;
                int const first = m;
                order[m++] = ~si;
                int last = si;
                for (int cur = si; cur >= 0 && !s_seen[cur]; cur = s_succ[cur])
                {
                    s_seen[cur] = 1;
                    order[m++] = cur;
                    last = cur;
                }
                if (pass == 1)
                {
                    // a closed loop: its last segment ends at the start vertex
                    wrap[first] = last;
                    wrap[m - 1] = si;
                }
            }
        *s_m = m;
    }
    __syncthreads();
    return *s_m;
}

// One block.  (1) The bounding-box centre of all endpoints.  (2) Chains: segment t follows segment s when
// P0(t) == P1(s) exactly (all three doubles), each t following at most one s (the lowest-numbered), so the links form
// disjoint open chains and closed loops.  (3) The entry stream: per chain a start entry (its first segment's P0)
// and then one entry per segment (its P1), open chains from their first segment and closed loops from their
// lowest-numbered segment, each vertex moved into the x1 = +z frame around the centre.  Chained vertices are the
// same doubles, so every segment sees the same P0 and P1 as in a stream of one chain per segment; chaining only
// lets the fractional kernel share the per-vertex work of consecutive segments.  A vertex's near threshold takes
// the longer of the segments that meet it in its chain, the last and first segments of a closed loop included, so
// on a boundary where no more than two segments meet at a vertex it does not depend on the input order.
// order: chain_scratch_ints(n_seg) ints of scratch (the stream order, each entry's loop-closing neighbour, and an
// open-addressing hash table of segment starts that finds the links in O(n_seg)).
__global__ void __launch_bounds__(1024) k_prep_mixed(const double* __restrict__ raw, int64_t n_seg, Rot rot,
                                                     float tau, Frame* __restrict__ frame, SegM* __restrict__ out,
                                                     SegX<double>* __restrict__ out64, int* __restrict__ order)
{
    __shared__ double red[2][3][32];
    __shared__ double centre[3];
    __shared__ int s_succ[kChainMax], s_pred[kChainMax];
    __shared__ unsigned char s_seen[kChainMax];
    __shared__ int s_entries;
    double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t s = threadIdx.x; s < n_seg; s += blockDim.x)
    {
        const double* w = raw + 7 * s;
        for (int k = 0; k < 3; ++k)
        {
            mn[k] = fmin(mn[k], fmin(w[k], w[3 + k]));
            mx[k] = fmax(mx[k], fmax(w[k], w[3 + k]));
        }
    }
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < 3; ++k)
    {
        for (int o = 16; o > 0; o >>= 1)
        {
            mn[k] = fmin(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
            mx[k] = fmax(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
        }
        if (lane == 0)
        {
            red[0][k][warp] = mn[k];
            red[1][k][warp] = mx[k];
        }
    }
    bool const chain = n_seg <= kChainMax;
    int const ns = chain ? int(n_seg) : 0;
    int* const wrap = order + 2 * ns; // per entry: the segment that closes its loop at this vertex, or -1
    int* const table = order + 4 * ns;
    __syncthreads(); // the warps' bounding boxes are in red
    if (threadIdx.x < 3)
    {
        int const k = threadIdx.x;
        double a = INFINITY, b = -INFINITY;
        for (int w = 0; w < int(blockDim.x + 31) / 32; ++w)
        {
            a = fmin(a, red[0][k][w]);
            b = fmax(b, red[1][k][w]);
        }
        centre[k] = (n_seg > 0) ? 0.5 * (a + b) : 0.0;
        frame->c[k] = centre[k];
    }
    // (2) the chains
    int const mc = block_chains(
        ns, [&](int t) { const double* u = raw + 7 * size_t(t); return make_double3(u[0], u[1], u[2]); },
        [&](int t) { const double* u = raw + 7 * size_t(t); return make_double3(u[3], u[4], u[5]); }, order, wrap,
        table, s_succ, s_pred, s_seen, &s_entries);
    int const m = chain ? mc : int(2 * n_seg);
    if (threadIdx.x == 0)
        frame->n_entries = m;
    // the links are done: s_pred now holds each segment's length
    float* const s_len = reinterpret_cast<float*>(s_pred);
    for (int s = threadIdx.x; s < ns; s += blockDim.x)
        s_len[s] = seg_length(raw + 7 * size_t(s));
    __syncthreads();
    auto len_of = [&](int s) { return chain ? s_len[s] : seg_length(raw + 7 * size_t(s)); };
    double const cx = centre[0], cy = centre[1], cz = centre[2];
    auto rotated = [&](const double* pt, double (&P)[3])
    {
        double const dx = pt[0] - cx, dy = pt[1] - cy, dz = pt[2] - cz;
        for (int r = 0; r < 3; ++r)
            P[r] = rot.m[3 * r] * dx + rot.m[3 * r + 1] * dy + rot.m[3 * r + 2] * dz;
    };
    for (int e = threadIdx.x; e < m; e += blockDim.x)
    {
        int s;
        bool start;
        if (chain)
        {
            int const o = order[e];
            start = o < 0;
            s = start ? ~o : o;
        }
        else
        {
            s = e >> 1;
            start = (e & 1) == 0;
        }
        const double* w = raw + 7 * size_t(s);
        double P0[3], P1[3];
        rotated(w, P0);
        rotated(w + 3, P1);
        double const* V = start ? P0 : P1;
        float hi[3], lo[3], dv[3];
        for (int r = 0; r < 3; ++r)
        {
            hi[r] = __double2float_rn(V[r]);
            lo[r] = __double2float_rn(V[r] - double(hi[r]));
            dv[r] = __double2float_rn(P1[r] - P0[r]);
        }
        // the segments meeting at this vertex: the entry's own (unless a start) and the next entry's (unless a start)
        int next = -1;
        if (e + 1 < m)
        {
            if (chain)
                next = order[e + 1];
            else
                next = (e & 1) == 0 ? s : -1;
        }
        int const closing = chain ? wrap[e] : -1;
        float const L = fmaxf(fmaxf(start ? 0.f : len_of(s), next >= 0 ? len_of(next) : 0.f),
                              closing >= 0 ? len_of(closing) : 0.f);
        float const near2 = (tau * L) * (tau * L);
        SegM mm;
        if (start)
        {
            mm.a = make_float4(hi[0], hi[1], hi[2], 0.f);
            mm.b = make_float4(0.f, 0.f, 0.f, near2);
            mm.c = make_float4(lo[0], lo[1], lo[2], __int_as_float(-1));
        }
        else
        {
            mm.a = make_float4(hi[0], hi[1], hi[2], float(w[6]));
            mm.b = make_float4(dv[0], dv[1], dv[2], near2);
            mm.c = make_float4(lo[0], lo[1], lo[2], __int_as_float(s));
        }
        out[e] = mm;
    }
    for (int64_t s = threadIdx.x; s < n_seg; s += blockDim.x)
    {
        const double* w = raw + 7 * s;
        out64[s] = SegX<double>{w[0], w[1], w[2], w[3], w[4], w[5], w[6], 0.0};
    }
}

// atan2 for the FP32 terms, our own: reduce to t = min(|y|, |x|) / max(|y|, |x|) in [0, 1], evaluate
// atan(t) = t * P(t^2) with a degree-8 polynomial P, then unfold the octant.  P's coefficients come from a
// minimax fit of atan(t) / t on [0, 1] by the Remez exchange algorithm (re-derived by tests/test_atan_fit.py;
// relative error 1.5e-8 in exact arithmetic,
// below float's 6e-8; about 3 ulp overall in float with the approximate reciprocal).
__device__ __forceinline__ float atan_unit(float t)
{
    float const s = t * t;
    float p = 0.0028498897585520423f;
    p = fmaf(p, s, -0.01606862951374933f);
    p = fmaf(p, s, 0.04269152017510156f);
    p = fmaf(p, s, -0.07504294615760822f);
    p = fmaf(p, s, 0.10640934061441572f);
    p = fmaf(p, s, -0.1420364447570674f);
    p = fmaf(p, s, 0.1999261939280182f);
    p = fmaf(p, s, -0.3333307334510578f);
    p = fmaf(p, s, 0.9999999847657755f);
    return t * p;
}
// atan2(y, x) given |x| and |y| already divided by max(|x|, |y|) (so the larger is 1).
__device__ __forceinline__ float atan2_scaled(float y, float x, float ax1, float ay1)
{
    float a = atan_unit(fminf(ax1, ay1));
    a = ay1 > ax1 ? 1.5707963267948966f - a : a;
    a = x < 0.f ? 3.141592653589793f - a : a;
    return copysignf(a, y);
}
__device__ __forceinline__ float atan2_fast(float y, float x)
{
    float const ax = fabsf(x), ay = fabsf(y);
    float const inv = __fdividef(1.f, fmaxf(fmaxf(ax, ay), 1e-37f));
    return atan2_scaled(y, x, ax * inv, ay * inv);
}

// Per-warp queue of (query, segment) pairs that go to FP64: packed (segment << 8) | (lane << 3) | k.
// Pairs are appended as the warp meets them and evaluated 32 at a time, one per lane, so the FP64 pipe works
// with full warps instead of one divergent lane per warp step.
template <int K>
struct Fp64Queue
{
    static constexpr unsigned kCap = 128u * K; // > 31 left over + 2 * 32 * K pushed per pair of entries
    uint32_t* e;                              // kCap entries of this warp
    double* res;                              // 32 results of this warp
    unsigned head = 0, tail = 0;              // warp-uniform counters
};

// The FP64 rule of the mesh functions for a pair the FP32 path turns down: the reference formula on the original
// doubles, times the weight.
struct MeshFallback
{
    const SegX<double>* seg64;
    __device__ __forceinline__ double operator()(const double* __restrict__ pos, int64_t i, uint32_t s,
                                                 ev3<rd> x1) const
    {
        SegX<double> const g = seg64[s];
        ev3<rd> const p{rd(pos[3 * i]), rd(pos[3 * i + 1]), rd(pos[3 * i + 2])};
        ev3<rd> const v0 = ev3<rd>{rd(g.p0x), rd(g.p0y), rd(g.p0z)} - p;
        ev3<rd> const v1 = ev3<rd>{rd(g.p1x), rd(g.p1y), rd(g.p1z)} - p;
        return (rd(g.w) * rd(vos_exact(x1, v0, v1))).v;
    }
};

// Evaluates up to 32 queued pairs, one per lane, with the FP64 rule fb(pos, query, segment, x1), and adds each
// result to its owner's accumulator.
template <int K, class FB>
__device__ __forceinline__ void fp64_flush(Fp64Queue<K>& q, unsigned c, int lane, int warp, int64_t tile_base,
                                           const double* __restrict__ pos, int64_t n, FB fb, ev3<rd> x1,
                                           double (&acc64)[K])
{
    __syncwarp();
    if (unsigned(lane) < c)
    {
        uint32_t const e = q.e[(q.head + lane) & (Fp64Queue<K>::kCap - 1)];
        int const owner = (e >> 3) & 31, kk = e & 7;
        int64_t i = tile_base + int64_t(kk) * blockDim.x + warp * 32 + owner;
        i = i < n ? i : n - 1;
        q.res[lane] = fb(pos, i, e >> 8, x1);
    }
    __syncwarp();
    for (unsigned j = 0; j < c; ++j)
    {
        uint32_t const e = q.e[(q.head + j) & (Fp64Queue<K>::kCap - 1)];
        if (int((e >> 3) & 31) == lane)
        {
            double const r = q.res[j];
#pragma unroll
            for (int k = 0; k < K; ++k)
                if (int(e & 7) == k)
                    acc64[k] += r;
        }
    }
    __syncwarp();
    q.head += c;
}

// The same operations on a lane vector: one query (float) or a packed pair of queries (float2, the paired add /
// multiply / FMA instructions of sm_100 and later, one instruction for both).  Each lane is rounded as the scalar
// operation would be, so code written over a lane vector gives bit-identical lanes for one query per thread and
// for two.
__device__ __forceinline__ float lv_add(float a, float b)
{
    return __fadd_rn(a, b);
}
__device__ __forceinline__ float lv_mul(float a, float b)
{
    return __fmul_rn(a, b);
}
__device__ __forceinline__ float lv_fma(float a, float b, float c)
{
    return __fmaf_rn(a, b, c);
}
__device__ __forceinline__ float2 lv_add(float2 a, float2 b)
{
    return __fadd2_rn(a, b);
}
__device__ __forceinline__ float2 lv_mul(float2 a, float2 b)
{
    return __fmul2_rn(a, b);
}
__device__ __forceinline__ float2 lv_fma(float2 a, float2 b, float2 c)
{
    return __ffma2_rn(a, b, c);
}
template <class V>
__device__ __forceinline__ V lv_set(float x)
{
    if constexpr (std::is_same_v<V, float>)
        return x;
    else
        return make_float2(x, x);
}
// a - b, rounded once
template <class V>
__device__ __forceinline__ V lv_sub(V a, V b)
{
    return lv_fma(b, lv_set<V>(-1.f), a);
}
// lane h of a lane vector
__device__ __forceinline__ float& ln(float& v, int)
{
    return v;
}
__device__ __forceinline__ float ln(float const& v, int)
{
    return v;
}
__device__ __forceinline__ float& ln(float2& v, int h)
{
    return h ? v.y : v.x;
}
__device__ __forceinline__ float ln(float2 const& v, int h)
{
    return h ? v.y : v.x;
}
// Compensated accumulation: acc + x by TwoSum (Knuth), its exact rounding error added to comp.  The pair
// (acc, comp) carries the sum to well below float's rounding, independently of the order of the terms.
template <class V>
__device__ __forceinline__ void two_sum_lv(V& acc, V& comp, V x)
{
    V const s = lv_add(acc, x);
    V const bp = lv_sub(s, acc);
    V const ap = lv_sub(s, bp);
    V const e = lv_add(lv_sub(acc, ap), lv_sub(x, bp));
    acc = s;
    comp = lv_add(comp, e);
}
// atan_unit on a lane vector (the same polynomial)
template <class V>
__device__ __forceinline__ V atan_unit_lv(V t)
{
    V const s = lv_mul(t, t);
    V p = lv_set<V>(0.0028498897585520423f);
    p = lv_fma(p, s, lv_set<V>(-0.01606862951374933f));
    p = lv_fma(p, s, lv_set<V>(0.04269152017510156f));
    p = lv_fma(p, s, lv_set<V>(-0.07504294615760822f));
    p = lv_fma(p, s, lv_set<V>(0.10640934061441572f));
    p = lv_fma(p, s, lv_set<V>(-0.1420364447570674f));
    p = lv_fma(p, s, lv_set<V>(0.1999261939280182f));
    p = lv_fma(p, s, lv_set<V>(-0.3333307334510578f));
    p = lv_fma(p, s, lv_set<V>(0.9999999847657755f));
    return lv_mul(t, p);
}

// atan(t) for 0 <= t <= 0.125: t (1 - s / 3 + s^2 / 5 - s^3 / 7), s = t^2, the Taylor series cut after t^7 (its
// relative truncation error is below s^4 / 9 = 6.6e-9 at t = 0.125, under float's 6e-8).
template <class V>
__device__ __forceinline__ V atan_small_lv(V t)
{
    V const s = lv_mul(t, t);
    V p = lv_set<V>(-0.14285714285714285f);
    p = lv_fma(p, s, lv_set<V>(0.2f));
    p = lv_fma(p, s, lv_set<V>(-0.3333333333333333f));
    p = lv_fma(p, s, lv_set<V>(1.f));
    return lv_mul(t, p);
}
// The mixed kernel's atan on [0, 1]: the short series up to t = 0.125 (which holds every pair of a certified
// group), the degree-8 fit above.  Both of the kernel's paths evaluate a small t with atan_small_lv, so they round
// alike.
__device__ __forceinline__ float2 atan_mixed_lv(float2 t)
{
    float2 const a = atan_small_lv(t), b = atan_unit_lv(t);
    return make_float2(t.x <= 0.125f ? a.x : b.x, t.y <= 0.125f ? a.y : b.y);
}

// Per-vertex quantities of one boundary vertex relative to two queries (frame coordinates, one lane each):
// v = vertex - query and the half-angle form (n, d) of l + z, l = |v|; d is NaN at a near vertex.
struct VState2
{
    float2 x, y, z, n, d;
};

// Blocks per SM the mixed kernel is compiled for: registers per thread scale with the queries per thread.
template <int K>
constexpr int mixed_min_blocks()
{
    return K >= 8 ? 1 : (K >= 4 ? 2 : (K >= 2 ? 3 : 4));
}

// Certified groups of the entry stream.  Group g of a tile is its entries [g G, g G + G) with the vertex before
// them.  In the frame (ray along +z) let r be the xy-distance from a query to a segment and L the segment's xy-length.
// With lambda = L / r, the segment subtends at most the angle lambda across the ray, den > 0, |num| / den <=
// lambda / cos(lambda), and the first-order bound the kernel computes per pair is at most
// lambda (1 / cos(lambda) + 1 / cos^2(lambda)) <= 2.02 lambda for lambda <= 0.1.  So r >= kappa L with
// kappa = max(10, 2.25 / te_units) keeps every pair's bound below 0.9 of te_units (the bound's own float rounding
// is a few ulps): no pair goes to FP64, and the angle lies in the first octant (|num| < den), where atan2 needs no
// unfolding.  With r also at least the near distance
// of each vertex (sqrt of its near2), no vertex state is NaN.  A warp tests this once per group and query tile
// against circles: each of its query slots' xy-circle and the group's, of centre (cx, cy) and reach = radius +
// max(kappa L_max, near distance), with a relative and an absolute slack for the float arithmetic of the test.
// Groups holding a chain start, the first group of a tile (its vertex before lies in the previous tile) and a
// tile's last, partial group take the full path.  A certified group's terms are bit-identical to the full path's:
// the same operations minus the selects that the certificate fixes.  Groups of 8 entries with kappa 10 certify 82%
// of the pairs of a 212-segment loop with 256^3 grid queries (16 entries, kappa 11.9: 72%; 3% slower).
constexpr int kCertG = 8;
constexpr int kCertMaxGroups = 256; // tiles of up to 2,048 entries

__device__ __forceinline__ float4 cert_group(SegM const* __restrict__ sb, int g, float kappa)
{
    int const e0 = g * kCertG;
    if (e0 == 0)
        return make_float4(0.f, 0.f, INFINITY, 0.f);
    float xmin = INFINITY, xmax = -INFINITY, ymin = INFINITY, ymax = -INFINITY, l2 = 0.f, near2 = 0.f, amax = 0.f;
    bool start = false;
    for (int e = e0 - 1; e < e0 + kCertG; ++e)
    {
        SegM const& s = sb[e];
        float const x = s.a.x + s.c.x, y = s.a.y + s.c.y;
        xmin = fminf(xmin, x);
        xmax = fmaxf(xmax, x);
        ymin = fminf(ymin, y);
        ymax = fmaxf(ymax, y);
        amax = fmaxf(amax, fmaxf(fmaxf(fabsf(s.a.x), fabsf(s.a.y)), fabsf(s.a.z)));
        near2 = fmaxf(near2, s.b.w);
        if (e >= e0)
        {
            start |= __float_as_int(s.c.w) < 0;
            l2 = fmaxf(l2, s.b.x * s.b.x + s.b.y * s.b.y);
        }
    }
    float const thr = fmaxf(kappa * sqrtf(l2), sqrtf(near2));
    // the range guard: vertices within 2^24 and distances of at least 2^-30 keep every product of the certified
    // path (up to the fourth power of a distance) normal and finite in float
    if (start || !(amax <= 16777216.f) || !(thr >= 9.3132257e-10f))
        return make_float4(0.f, 0.f, INFINITY, 0.f);
    float const cx = 0.5f * (xmin + xmax), cy = 0.5f * (ymin + ymax);
    float const rad = 0.5f * sqrtf((xmax - xmin) * (xmax - xmin) + (ymax - ymin) * (ymax - ymin));
    float const reach = rad + thr;
    float const slack = 1e-5f * (fabsf(cx) + fabsf(cy) + reach);
    return make_float4(cx, cy, 1.01f * reach + slack, 0.f);
}

// fb: the FP64 rule for the pairs the FP32 path turns down (MeshFallback, or the robust evaluator's).  K (even)
// queries per thread, evaluated as K / 2 packed pairs.
template <int K, class FB>
__global__ void __launch_bounds__(256, mixed_min_blocks<K>())
    k_frac_mixed(const double* __restrict__ pos, int64_t n, double* __restrict__ out, const int32_t* __restrict__ counts,
                 double x0x, double x0y, double x0z, Rot rot, const Frame* __restrict__ frame, int certify,
                 float term_err, const SegM* __restrict__ seg, FB fb, int64_t n_seg, int tile, int* flags,
                 long long* counters, int count_pairs)
{
    static_assert(K % 2 == 0, "queries per thread come in packed pairs");
    constexpr int KP = K / 2;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ int abort_cta;
    __shared__ double centre[3];
    __shared__ uint32_t q_entries[8][Fp64Queue<K>::kCap];
    __shared__ double q_results[8][32];
    __shared__ float4 s_grp[kCertMaxGroups];

    // the entry stream (chain starts and segments, k_prep_mixed) is what the tiles walk
    int64_t const n_entries = frame->n_entries;
    TilePipe<SegM> pipe;
    pipe.n_tiles = int((n_entries + tile - 1) / tile);
    pipe.single = pipe.n_tiles == 1;
    pipe.buf[0] = reinterpret_cast<SegM*>(smem);
    pipe.buf[1] = pipe.buf[0] + (pipe.single ? 0 : tile);
    pipe.bar = bars;
    pipe.gseg = seg;
    pipe.n_seg = n_entries;
    pipe.tile = tile;

    int64_t const per_tile = int64_t(blockDim.x) * K;
    int64_t const n_qtiles = (n + per_tile - 1) / per_tile;
    int const my_qtiles = blockIdx.x < n_qtiles ? int((n_qtiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;
    int const n_items = pipe.single ? (my_qtiles > 0 ? 1 : 0) : my_qtiles * pipe.n_tiles;
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned const lt = (1u << lane) - 1u;

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
    if (threadIdx.x < 3)
        centre[threadIdx.x] = frame->c[threadIdx.x];
    __syncthreads();

    // Rounding bound per FP32 operation chain (4 eps32), and the term error bound in its units.
    constexpr float kEpsBound = 4.0f * 5.9604645e-8f;
    float const te_units = term_err / kEpsBound;
    // kappa: the certificate's distance in longest segments (infinite with certify 0: no group certified)
    float const kappa = certify ? fmaxf(10.f, 2.25f / te_units) : INFINITY;
    // the certified groups of the tile in shared memory (every thread calls it; ends with a block barrier)
    auto groups_of = [&](SegM const* sb, int cnt)
    {
        int const ng = min(cnt / kCertG, kCertMaxGroups);
        for (int g = threadIdx.x; g < ng; g += blockDim.x)
            s_grp[g] = cert_group(sb, g, kappa);
        __syncthreads();
    };
    double const two_pi = 2.0 * kPi<double>;
    ev3<rd> const x1{rd(-x0x), rd(-x0y), rd(-x0z)};
    Fp64Queue<K> fq;
    fq.e = q_entries[warp];
    fq.res = q_results[warp];

    int it = 0;
    long long n_cert = 0; // entries of certified groups this warp evaluated (warp-uniform)
    for (int j = 0; j < my_qtiles; ++j)
    {
        int64_t const tile_base = (blockIdx.x + int64_t(j) * gridDim.x) * per_tile;
        int64_t const base = tile_base + threadIdx.x;
        // the queries' frame coordinates as float hi + lo, negated (the vertex difference is then an add), queries
        // 2p and 2p + 1 in the lanes of pair p
        float2 nqhx[KP], nqhy[KP], nqhz[KP], nqlx[KP], nqly[KP], nqlz[KP];
        float2 acc[KP], comp[KP];
        double acc64[K];
        // per-vertex state of the two most recent entries, in alternation (even entries write st0, odd ones st1)
        VState2 st0[KP], st1[KP];
#pragma unroll
        for (int k = 0; k < K; ++k)
        {
            int64_t const i = base + int64_t(k) * blockDim.x;
            int64_t const ii = i < n ? i : n - 1;
            double const dx = pos[3 * ii] - centre[0], dy = pos[3 * ii + 1] - centre[1],
                         dz = pos[3 * ii + 2] - centre[2];
            double const Qx = rot.m[0] * dx + rot.m[1] * dy + rot.m[2] * dz;
            double const Qy = rot.m[3] * dx + rot.m[4] * dy + rot.m[5] * dz;
            double const Qz = rot.m[6] * dx + rot.m[7] * dy + rot.m[8] * dz;
            float const hx = __double2float_rn(Qx), hy = __double2float_rn(Qy), hz = __double2float_rn(Qz);
            float const lx = __double2float_rn(Qx - double(hx)), ly = __double2float_rn(Qy - double(hy)),
                        lz = __double2float_rn(Qz - double(hz));
            auto const set = [&](float2& v, float x) { (k & 1 ? v.y : v.x) = x; };
            set(nqhx[k / 2], -hx);
            set(nqhy[k / 2], -hy);
            set(nqhz[k / 2], -hz);
            set(nqlx[k / 2], -lx);
            set(nqly[k / 2], -ly);
            set(nqlz[k / 2], -lz);
            acc64[k] = 0.0;
        }
#pragma unroll
        for (int p = 0; p < KP; ++p)
        {
            acc[p] = lv_set<float2>(0.f);
            comp[p] = lv_set<float2>(0.f);
            st0[p] = VState2{};
            st1[p] = VState2{};
        }
        // each query slot's xy-circle over the warp's 32 lanes (centre, radius with a slack); a slot with a
        // coordinate beyond 2^24 (or NaN) gets an infinite radius, so none of the warp's groups is certified
        float scx[K], scy[K], srad[K];
#pragma unroll
        for (int k = 0; k < K; ++k)
        {
            float const x = -ln(nqhx[k / 2], k & 1), y = -ln(nqhy[k / 2], k & 1), z = -ln(nqhz[k / 2], k & 1);
            float x0 = x, x1 = x, y0 = y, y1 = y;
            bool sane = fmaxf(fmaxf(fabsf(x), fabsf(y)), fabsf(z)) <= 16777216.f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
            {
                x0 = fminf(x0, __shfl_xor_sync(0xffffffffu, x0, o));
                x1 = fmaxf(x1, __shfl_xor_sync(0xffffffffu, x1, o));
                y0 = fminf(y0, __shfl_xor_sync(0xffffffffu, y0, o));
                y1 = fmaxf(y1, __shfl_xor_sync(0xffffffffu, y1, o));
            }
            sane = __all_sync(0xffffffffu, sane);
            scx[k] = 0.5f * (x0 + x1);
            scy[k] = 0.5f * (y0 + y1);
            float const rad = 0.5f * sqrtf((x1 - x0) * (x1 - x0) + (y1 - y0) * (y1 - y0));
            srad[k] = sane ? 1.01f * rad + 1e-5f * (fabsf(scx[k]) + fabsf(scy[k]) + rad) : INFINITY;
        }
        // Pairs that go to FP64 are marked in a bit mask (bit slot * K + k) while two entries are evaluated, and
        // pushed to the warp's queue afterwards behind one warp-uniform branch that is rarely taken.
        uint32_t nb = 0;
        // One entry: its vertex relative to each query (into cv), then the pair term of the segment from the
        // previous entry's vertex (pv) to this one.  With may_start false (both entries of the pair are segments,
        // the common case) the body has no branches: a term taken to FP64 adds an exact zero to the TwoSum, so the
        // compiler schedules consecutive entries together.  With may_start true a chain start skips the pair term.
        // The arithmetic runs on packed pairs of queries; selects and comparisons per lane.
        // near: the NaN for a vertex within its near distance (a certified group has none, and its states come out
        // the same without the test)
        auto vertex = [&](SegM const& ent, VState2 (&cv)[KP], bool near)
        {
            float4 const A = ent.a, B = ent.b, C = ent.c;
            float2 const ax = lv_set<float2>(A.x), ay = lv_set<float2>(A.y), az = lv_set<float2>(A.z);
            float2 const cx = lv_set<float2>(C.x), cy = lv_set<float2>(C.y), cz = lv_set<float2>(C.z);
#pragma unroll
            for (int p = 0; p < KP; ++p)
            {
                VState2& c = cv[p];
                c.x = lv_add(lv_add(ax, nqhx[p]), lv_add(cx, nqlx[p]));
                c.y = lv_add(lv_add(ay, nqhy[p]), lv_add(cy, nqly[p]));
                c.z = lv_add(lv_add(az, nqhz[p]), lv_add(cz, nqlz[p]));
                float2 const r = lv_fma(c.x, c.x, lv_mul(c.y, c.y));
                float2 const q = lv_fma(c.z, c.z, r);
                float2 const l = lv_mul(q, make_float2(rsqrt_approx(q.x), rsqrt_approx(q.y)));
                // l + z = n / d with (n, d) = (l + z, 1) for z >= 0 and (x^2 + y^2, l - z) for z < 0, free of
                // cancellation.  d > 0, or NaN for a near vertex (|v|^2 < near2): the NaN makes the error bound of
                // both segments at this vertex NaN, which sends them to FP64
                float2 const lpz = lv_add(l, c.z), lmz = lv_sub(l, c.z);
                float const nan = __int_as_float(0x7fffffff);
                c.n = make_float2(c.z.x >= 0.f ? lpz.x : r.x, c.z.y >= 0.f ? lpz.y : r.y);
                float2 const d = make_float2(c.z.x >= 0.f ? 1.f : lmz.x, c.z.y >= 0.f ? 1.f : lmz.y);
                c.d = near ? make_float2(q.x < B.w ? nan : d.x, q.y < B.w ? nan : d.y) : d;
            }
        };
        // a certified pair term: the full path's operations with need = false, |num| <= den and den > 0
        auto fast = [&](SegM const& ent, VState2 (&pv)[KP], VState2 (&cv)[KP])
        {
            vertex(ent, cv, false);
            float4 const A = ent.a, B = ent.b;
            float2 const by = lv_set<float2>(B.y), nbx = lv_set<float2>(-B.x), w = lv_set<float2>(A.w);
#pragma unroll
            for (int p = 0; p < KP; ++p)
            {
                VState2 const& v0 = pv[p];
                VState2 const& v1 = cv[p];
                float2 const num = lv_fma(v0.x, by, lv_mul(v0.y, nbx));
                float2 const D = lv_mul(v0.d, v1.d), nn = lv_mul(v0.n, v1.n);
                float2 const num_s = lv_mul(num, D);
                float2 const den_s = lv_fma(lv_fma(v0.x, v1.x, lv_mul(v0.y, v1.y)), D, nn);
                float2 const an = make_float2(fabsf(num_s.x), fabsf(num_s.y));
                float2 const inv = make_float2(rcp_approx(den_s.x), rcp_approx(den_s.y));
                float2 const a = atan_small_lv(lv_mul(an, inv)); // t <= 0.101 here
                float2 const ang = make_float2(copysignf(a.x, num_s.x), copysignf(a.y, num_s.y));
                two_sum_lv(acc[p], comp[p], lv_mul(w, ang));
            }
        };
        auto step = [&](SegM const& ent, VState2 (&pv)[KP], VState2 (&cv)[KP], bool may_start, int slot)
        {
            vertex(ent, cv, true);
            float4 const A = ent.a, B = ent.b, C = ent.c;
            int const sidx = __float_as_int(C.w);
            if (may_start && sidx < 0)
                return;
            float2 const by = lv_set<float2>(B.y), nbx = lv_set<float2>(-B.x), w = lv_set<float2>(A.w);
#pragma unroll
            for (int p = 0; p < KP; ++p)
            {
                VState2 const& v0 = pv[p];
                VState2 const& v1 = cv[p];
                // num from the segment vector B (accurate on its own, no cancellation for a far segment)
                // num = v0.x * B.y - v0.y * B.x and v0.x * v1.x + v0.y * v1.y as written FMAs (the certified path
                // computes the same); ta and pxy are the products for the error bound
                float2 const ta = lv_mul(v0.x, by), tbn = lv_mul(v0.y, nbx);
                float2 const num = lv_fma(v0.x, by, tbn);
                // scaling num and den by the positive D = d0 * d1 leaves the angle unchanged and removes both
                // divisions: den * D = n0 * n1 + (v0.x*v1.x + v0.y*v1.y) * D
                float2 const D = lv_mul(v0.d, v1.d), nn = lv_mul(v0.n, v1.n);
                float2 const pxy = lv_mul(v0.x, v1.x), pyy = lv_mul(v0.y, v1.y);
                float2 const num_s = lv_mul(num, D);
                float2 const den_s = lv_fma(lv_fma(v0.x, v1.x, pyy), D, nn);
                // first-order rounding bounds: num errs by about eps * sn and den by about eps * sd, so the angle
                // errs by at most eps * (sn * |den| + sd * |num|) / (num^2 + den^2) <= eps * (sn * ad1 + sd * an1) / M
                // with M = max(|num|, |den|) and an1, ad1 the two divided by M: one of them is 1, the other is the
                // ratio t that atan2 takes as well
                float2 const sn =
                    lv_mul(make_float2(fabsf(ta.x) + fabsf(tbn.x), fabsf(ta.y) + fabsf(tbn.y)), D);
                float2 const sd =
                    lv_fma(make_float2(fabsf(pxy.x) + fabsf(pyy.x), fabsf(pxy.y) + fabsf(pyy.y)), D, nn);
                float2 const an = make_float2(fabsf(num_s.x), fabsf(num_s.y));
                float2 const ad = make_float2(fabsf(den_s.x), fabsf(den_s.y));
                bool const sw0 = an.x > ad.x, sw1 = an.y > ad.y;
                // (num = den = 0 gives an infinite reciprocal, a NaN t and a NaN bound: the pair goes to FP64)
                float2 const inv = make_float2(rcp_approx(fmaxf(an.x, ad.x)), rcp_approx(fmaxf(an.y, ad.y)));
                // an1, ad1: |num| and |den| over M, t the smaller; the bound (sn * ad1 + sd * an1) / M as packed
                // products, without per-lane selects
                float2 const an1 = lv_mul(an, inv), ad1 = lv_mul(ad, inv);
                float2 const t = make_float2(fminf(an1.x, ad1.x), fminf(an1.y, ad1.y));
                float2 const bound = lv_mul(lv_fma(sn, ad1, lv_mul(sd, an1)), inv); // in units of kEpsBound
                // a NaN or infinity anywhere (a near vertex, |v| = 0, overflow) makes the bound NaN, which the negated
                // comparison sends to FP64; so does a branch (den <= 0) decided within the rounding of num
                float2 const margin = lv_fma(lv_set<float2>(-kEpsBound), sn, an);
                bool const need0 = !(bound.x <= te_units) || fmaxf(den_s.x, margin.x) <= 0.f;
                bool const need1 = !(bound.y <= te_units) || fmaxf(den_s.y, margin.y) <= 0.f;
                nb |= (need0 ? (1u << (slot * K + 2 * p)) : 0u) | (need1 ? (1u << (slot * K + 2 * p + 1)) : 0u);
                // atan2(num_s, den_s): atan(t) in [0, pi/4], then the octant as |c1 - a| (pi/2 - a when |num| >
                // |den|, else a) and |c2 - a| (pi - a when den < 0, else a), signed like num
                float2 const a = atan_mixed_lv(t);
                float2 const c1 = make_float2(sw0 ? 1.5707963267948966f : 0.f, sw1 ? 1.5707963267948966f : 0.f);
                float2 const a1 = lv_sub(c1, a);
                float2 const c2 = make_float2(den_s.x < 0.f ? 3.141592653589793f : 0.f,
                                              den_s.y < 0.f ? 3.141592653589793f : 0.f);
                float2 const a2 = lv_sub(c2, make_float2(fabsf(a1.x), fabsf(a1.y)));
                float2 const ang = make_float2(copysignf(fabsf(a2.x), num_s.x), copysignf(fabsf(a2.y), num_s.y));
                float2 const term = lv_mul(w, ang);
                two_sum_lv(acc[p], comp[p], make_float2(need0 ? 0.f : term.x, need1 ? 0.f : term.y));
            }
        };
        // the marked pairs of `count` entries from sb[s0] into the queue (the caller then drains full batches: at
        // most 31 + 2 * 32 * K entries stay queued, below the ring's capacity)
        auto push = [&](SegM const* sb, int s0, int count)
        {
#pragma unroll
            for (int e = 0; e < 2; ++e)
            {
                if (e >= count)
                    break;
                uint32_t const sidx = uint32_t(__float_as_int(sb[s0 + e].c.w));
#pragma unroll
                for (int k = 0; k < K; ++k)
                {
                    bool const nd = (nb >> (e * K + k)) & 1u;
                    unsigned const mq = __ballot_sync(0xffffffffu, nd);
                    if (nd)
                        fq.e[(fq.tail + __popc(mq & lt)) & (Fp64Queue<K>::kCap - 1)] =
                            (sidx << 8) | (uint32_t(lane) << 3) | uint32_t(k);
                    fq.tail += __popc(mq);
                }
            }
            nb = 0;
        };
        for (int st = 0; st < pipe.n_tiles; ++st)
        {
            int const b = it & 1;
            // a single tile stays in shared memory for every query tile: only the first waits for it, and the warps
            // then run their query tiles without meeting at a barrier
            if (!pipe.single || j == 0)
            {
                bool ok = mbar_wait_bounded(&bars[b], unsigned((it >> 1) & 1), flags, 2);
                if (!ok)
                    abort_cta = 1;
                __syncthreads();
                if (abort_cta)
                    return;
            }
            SegM const* sb = pipe.buf[b];
            int const cnt = pipe.tile_count(st);
            int const ng = min(cnt / kCertG, kCertMaxGroups);
            if (!pipe.single || j == 0)
                groups_of(sb, cnt);
            // tiles start at even positions of the stream (the tile and the group are even), so the alternation runs
            // across groups and tiles; only the last tile can end on an odd count
            uint32_t cmask = 0;
            for (int s0 = 0; s0 < cnt; s0 += kCertG)
            {
                int const g = s0 / kCertG;
                if ((g & 31) == 0)
                {
                    // lane l tests group g + l against every query slot of the warp
                    int const gl = g + lane;
                    bool ok = gl < ng;
                    if (ok)
                    {
                        float4 const c = s_grp[gl];
#pragma unroll
                        for (int k = 0; k < K; ++k)
                        {
                            float const dx = c.x - scx[k], dy = c.y - scy[k], need = c.z + srad[k];
                            ok = ok && dx * dx + dy * dy >= need * need;
                        }
                    }
                    cmask = __ballot_sync(0xffffffffu, ok);
                }
                if ((cmask >> (g & 31)) & 1u)
                {
                    n_cert += kCertG;
                    for (int s = s0; s < s0 + kCertG; s += 2)
                    {
                        fast(sb[s], st1, st0);
                        fast(sb[s + 1], st0, st1);
                    }
                    continue;
                }
                int const e1 = min(s0 + kCertG, cnt);
                int s = s0;
                for (; s + 1 < e1; s += 2)
                {
                    if ((__float_as_int(sb[s].c.w) | __float_as_int(sb[s + 1].c.w)) >= 0)
                    {
                        step(sb[s], st1, st0, false, 0);
                        step(sb[s + 1], st0, st1, false, 1);
                    }
                    else
                    {
                        step(sb[s], st1, st0, true, 0);
                        step(sb[s + 1], st0, st1, true, 1);
                    }
                    if (__any_sync(0xffffffffu, nb != 0))
                    {
                        push(sb, s, 2);
                        while (fq.tail - fq.head >= 32)
                            fp64_flush<K>(fq, 32, lane, warp, tile_base, pos, n, fb, x1, acc64);
                    }
                }
                if (s < e1)
                {
                    step(sb[s], st1, st0, true, 0);
                    if (__any_sync(0xffffffffu, nb != 0))
                    {
                        push(sb, s, 1);
                        while (fq.tail - fq.head >= 32)
                            fp64_flush<K>(fq, 32, lane, warp, tile_base, pos, n, fb, x1, acc64);
                    }
                }
            }
            if (!pipe.single)
            {
                __syncthreads();
                if (threadIdx.x == 0 && it + 2 < n_items)
                    pipe.issue(it + 2);
                ++it;
            }
        }
        while (fq.tail != fq.head)
        {
            unsigned const c = min(32u, fq.tail - fq.head);
            fp64_flush<K>(fq, c, lane, warp, tile_base, pos, n, fb, x1, acc64);
        }
#pragma unroll
        for (int k = 0; k < K; ++k)
        {
            int64_t const i = base + int64_t(k) * blockDim.x;
            if (i < n)
            {
                float const ak = (k & 1) ? acc[k / 2].y : acc[k / 2].x, ck = (k & 1) ? comp[k / 2].y : comp[k / 2].x;
                double v = ((double(ak) + double(ck)) + acc64[k]) / two_pi;
                if (counts)
                    v += double(counts[i]);
                out[i] = v;
            }
        }
    }
    if (count_pairs && lane == 0)
    {
        // statistics: pairs taken to FP64 (queue entries, valid queries or not) and all pairs of valid queries
        long long tot = 0;
        for (int j = 0; j < my_qtiles; ++j)
        {
            int64_t const b0 = (blockIdx.x + int64_t(j) * gridDim.x) * per_tile + warp * 32;
            for (int k = 0; k < K; ++k)
            {
                int64_t const first = b0 + int64_t(k) * blockDim.x;
                int64_t const valid = first >= n ? 0 : (n - first < 32 ? n - first : 32);
                tot += valid * n_seg;
            }
        }
        atomicAdd(reinterpret_cast<unsigned long long*>(counters), static_cast<unsigned long long>(fq.tail));
        atomicAdd(reinterpret_cast<unsigned long long*>(counters + 3),
                  static_cast<unsigned long long>(n_cert * 32 * K));
        atomicAdd(reinterpret_cast<unsigned long long*>(counters + 1), static_cast<unsigned long long>(tot));
    }
}

template <class T>
__global__ void k_fill_counts(T* out, const int32_t* counts, int64_t n)
{
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        out[i] = counts ? T(counts[i]) : T(0);
}

// Rotation whose third row is x1 = -x0 / |x0|: rows (e1, e2, x1_hat), right-handed.
Rot make_rotation(const double* x0)
{
    double const n = std::sqrt(x0[0] * x0[0] + x0[1] * x0[1] + x0[2] * x0[2]);
    double z[3] = {-x0[0] / n, -x0[1] / n, -x0[2] / n};
    // helper axis least aligned with z
    double a[3] = {0, 0, 0};
    int m = 0;
    for (int k = 1; k < 3; ++k)
        if (std::fabs(z[k]) < std::fabs(z[m]))
            m = k;
    a[m] = 1.0;
    double x[3] = {a[1] * z[2] - a[2] * z[1], a[2] * z[0] - a[0] * z[2], a[0] * z[1] - a[1] * z[0]};
    double const xn = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    for (double& v : x)
        v /= xn;
    double y[3] = {z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2], z[0] * x[1] - z[1] * x[0]};
    Rot r;
    for (int k = 0; k < 3; ++k)
    {
        r.m[k] = x[k];
        r.m[3 + k] = y[k];
        r.m[6 + k] = z[k];
    }
    return r;
}

} // namespace
} // namespace agwn
