// Integer (ray-crossing) term of the mesh GWN, and the CudaIntersector C ABI.
//
// Counting rule: NaiveIntersector::signed_intersection_count (src/antipodal/intersector/intersector.hh:61-100):
// Moller-Trumbore against (p, dir), t >= 0, sign of (e1 x e2) . dir, with its early rejections.  The test is
// written with unfused, correctly rounded operations (rd/rf), so every candidate triangle gets exactly the CPU's
// decision -- including the double count of a ray through an edge shared by two triangles.
//
// Acceleration.  All rays of one batch share the direction dir (the reference passes x0 to every query, and its
// contract fixes x0 per mesh), so the hierarchy is built in the frame (u, v, w) with w along dir: a ray is the
// point (u_q, v_q) plus the half-line w >= w_q.  A node is then hit iff its (u, v) box contains the query's point
// and its largest w is not behind the query -- five float compares, no slab divisions, and boxes that are tight
// around the projected triangles.  The hierarchy is built on the device when a context first queries an
// intersector along a direction and cached in that context: (u, v) centroids -> 2 x 15-bit Morton codes ->
// stable LSD radix sort in four 8-bit passes -> Karras (2012) hierarchy (ties broken by position) -> bottom-up
// boxes with one atomic visit counter per node.  One triangle per leaf; the leaves' world-space vertices are
// stored in leaf order as contiguous 9-scalar records for the exact test.
//
// The hierarchy only culls.  Boxes are rounded outward to float and the comparisons are widened by a tolerance
// far above the float rounding of the rotated query, so a triangle the exact test would count is never culled:
// counts equal the linear scan's.

#include "agwn_internal.cuh"
#include "gwn_kernels.cuh"
#include "hier.cuh"
#include "radix.cuh"

#include <type_traits>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <vector>

namespace agwn
{
namespace
{

std::atomic<unsigned long long> g_generation{1};

__device__ __forceinline__ unsigned expand_bits2(unsigned v)
{
    v &= 0x7fffu;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

__device__ __forceinline__ unsigned float_flip(float f)
{
    unsigned const u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float float_unflip(unsigned u)
{
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Gathers the indexed triangles into 9-scalar records and finds the largest coordinate magnitude.  Raises
// flags[FLAG_COUNT - 1] on an out-of-range index.
template <class T>
__global__ void k_gather(const T* __restrict__ verts, int64_t nv, const int32_t* __restrict__ idx, int64_t n_tri,
                         T* __restrict__ tri, unsigned* __restrict__ scale_bits, int* flags)
{
    float amax = 0.f;
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n_tri; t += int64_t(gridDim.x) * blockDim.x)
    {
        for (int v = 0; v < 3; ++v)
        {
            int32_t const i = idx[3 * t + v];
            bool const ok = i >= 0 && i < nv;
            if (!ok)
                atomicOr(flags + FLAG_COUNT - 1, 1);
            for (int k = 0; k < 3; ++k)
            {
                T const c = ok ? verts[3 * int64_t(i) + k] : T(0);
                tri[9 * t + 3 * v + k] = c;
                amax = fmaxf(amax, fabsf(float(c)));
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1)
        amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    if ((threadIdx.x & 31) == 0)
        atomicMax(scale_bits, __float_as_uint(amax)); // non-negative floats order like their bits
}

// Per triangle: outward-rounded float box in the ray frame and its (u, v) centroid; (u, v) bounds of the
// centroids as flipped-uint atomics.
template <class T>
__global__ void k_ray_boxes(const T* __restrict__ tri, int64_t n_tri, Frame64 f, float* __restrict__ box,
                            float* __restrict__ cen, unsigned* __restrict__ cbounds, unsigned* __restrict__ scale_bits)
{
    float cmn[2] = {INFINITY, INFINITY}, cmx[2] = {-INFINITY, -INFINITY};
    float amax = 0.f;
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n_tri; t += int64_t(gridDim.x) * blockDim.x)
    {
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int v = 0; v < 3; ++v)
        {
            double const x = double(tri[9 * t + 3 * v]), y = double(tri[9 * t + 3 * v + 1]),
                         z = double(tri[9 * t + 3 * v + 2]);
            for (int r = 0; r < 3; ++r)
            {
                double const c = f.r[3 * r] * x + f.r[3 * r + 1] * y + f.r[3 * r + 2] * z;
                lo[r] = fmin(lo[r], c);
                hi[r] = fmax(hi[r], c);
            }
        }
        for (int r = 0; r < 3; ++r)
        {
            box[6 * t + r] = __double2float_rd(lo[r]);
            box[6 * t + 3 + r] = __double2float_ru(hi[r]);
            amax = fmaxf(amax, fmaxf(fabsf(box[6 * t + r]), fabsf(box[6 * t + 3 + r])));
        }
        for (int r = 0; r < 2; ++r)
        {
            float const c = float(0.5 * (lo[r] + hi[r]));
            cen[2 * t + r] = c;
            cmn[r] = fminf(cmn[r], c);
            cmx[r] = fmaxf(cmx[r], c);
        }
    }
    for (int r = 0; r < 2; ++r)
        for (int o = 16; o > 0; o >>= 1)
        {
            cmn[r] = fminf(cmn[r], __shfl_xor_sync(0xffffffffu, cmn[r], o));
            cmx[r] = fmaxf(cmx[r], __shfl_xor_sync(0xffffffffu, cmx[r], o));
        }
    for (int o = 16; o > 0; o >>= 1)
        amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    if ((threadIdx.x & 31) == 0)
    {
        for (int r = 0; r < 2; ++r)
        {
            atomicMin(cbounds + r, float_flip(cmn[r]));
            atomicMax(cbounds + 2 + r, float_flip(cmx[r]));
        }
        atomicMax(scale_bits, __float_as_uint(amax)); // non-negative floats order like their bits
    }
}

__global__ void k_morton2(const float* __restrict__ cen, int64_t n_tri, const unsigned* __restrict__ cbounds,
                          unsigned* __restrict__ keys, unsigned* __restrict__ vals)
{
    float lo[2], ext[2];
    for (int r = 0; r < 2; ++r)
    {
        lo[r] = float_unflip(cbounds[r]);
        ext[r] = float_unflip(cbounds[2 + r]) - lo[r];
    }
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n_tri; t += int64_t(gridDim.x) * blockDim.x)
    {
        unsigned m[2];
        for (int r = 0; r < 2; ++r)
        {
            float const u = ext[r] > 0.f ? (cen[2 * t + r] - lo[r]) / ext[r] : 0.5f;
            m[r] = unsigned(fminf(fmaxf(u * 32768.f, 0.f), 32767.f));
        }
        keys[t] = (expand_bits2(m[0]) << 1) | expand_bits2(m[1]);
        vals[t] = unsigned(t);
    }
}



// ---- Karras hierarchy ---------------------------------------------------------------------------------------
__device__ __forceinline__ int delta(const unsigned* keys, int n, int i, int j)
{
    if (j < 0 || j >= n)
        return -1;
    unsigned const a = keys[i], b = keys[j];
    if (a == b)
        return 32 + __clz(unsigned(i) ^ unsigned(j));
    return __clz(a ^ b);
}

__global__ void k_karras(const unsigned* __restrict__ keys, int n, int* __restrict__ left, int* __restrict__ right,
                         int* __restrict__ parent_node, int* __restrict__ parent_leaf)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1)
        return;
    int const d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    int const dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin)
        lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (delta(keys, n, i, i + (l + t) * d) > dmin)
            l += t;
    int const j = i + l * d;
    int const dnode = delta(keys, n, i, j);
    int s = 0;
    for (int div = 2;; div *= 2)
    {
        int const t = (l + div - 1) / div;
        if (delta(keys, n, i, i + (s + t) * d) > dnode)
            s += t;
        if (t <= 1)
            break;
    }
    int const gamma = i + s * d + min(d, 0);
    int const lo = min(i, j), hi = max(i, j);
    int const lc = (lo == gamma) ? ~gamma : gamma;
    int const rc = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    left[i] = lc;
    right[i] = rc;
    if (lc < 0)
        parent_leaf[~lc] = i;
    else
        parent_node[lc] = i;
    if (rc < 0)
        parent_leaf[~rc] = i;
    else
        parent_node[rc] = i;
    if (i == 0)
        parent_node[0] = -1;
}

// Leaf setup: each sorted triangle's world-space vertices, its ray-frame box and its vertices projected on the
// (u, v) plane (rounded to float; 8 floats per leaf: u0 v0 u1 v1 u2 v2 0 0) into leaf order.
template <class T>
__global__ void k_leaves(const T* __restrict__ tri_in, const unsigned* __restrict__ order,
                         const float* __restrict__ box, int64_t n_tri, Frame64 f, T* __restrict__ tri,
                         float* __restrict__ leaf_box, float* __restrict__ leaf_uv)
{
    for (int64_t l = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; l < n_tri; l += int64_t(gridDim.x) * blockDim.x)
    {
        unsigned const t = order[l];
        for (int k = 0; k < 9; ++k)
            tri[9 * l + k] = tri_in[9 * int64_t(t) + k];
        for (int k = 0; k < 6; ++k)
            leaf_box[6 * l + k] = box[6 * int64_t(t) + k];
        float* const o = leaf_uv + 4 * kLeafF4 * l; // layout: see kLeafF4 (hier.cuh)
        for (int v = 0; v < 3; ++v)
        {
            double const x = double(tri_in[9 * int64_t(t) + 3 * v]), y = double(tri_in[9 * int64_t(t) + 3 * v + 1]),
                         z = double(tri_in[9 * int64_t(t) + 3 * v + 2]);
            o[2 * v] = float(f.r[0] * x + f.r[1] * y + f.r[2] * z);
            o[2 * v + 1] = float(f.r[3] * x + f.r[4] * y + f.r[5] * z);
            o[6 + v] = float(f.r[6] * x + f.r[7] * y + f.r[8] * z);
        }
        o[9] = o[10] = o[11] = 0.f;
    }
}

__global__ void k_refit(int n, const int* __restrict__ left, const int* __restrict__ right,
                        const int* __restrict__ parent_node, const int* __restrict__ parent_leaf,
                        const float* __restrict__ leaf_box, float* node_box, int* visit, BvhNode* __restrict__ nodes)
{
    int const l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= n)
        return;
    int node = parent_leaf[l];
    while (node >= 0)
    {
        __threadfence();
        if (atomicAdd(&visit[node], 1) == 0)
            return; // the sibling subtree is not finished; its last thread continues upward
        float b[2][6];
        int const ch[2] = {left[node], right[node]};
        for (int c = 0; c < 2; ++c)
        {
            const float* src = ch[c] < 0 ? leaf_box + 6 * int64_t(~ch[c]) : node_box + 6 * int64_t(ch[c]);
            for (int k = 0; k < 6; ++k)
                b[c][k] = __ldcg(src + k);
        }
        BvhNode nd;
        nd.lo_l = make_float4(b[0][0], b[0][1], b[0][2], __int_as_float(ch[0]));
        nd.hi_l = make_float4(b[0][3], b[0][4], b[0][5], 0.f);
        nd.lo_r = make_float4(b[1][0], b[1][1], b[1][2], __int_as_float(ch[1]));
        nd.hi_r = make_float4(b[1][3], b[1][4], b[1][5], 0.f);
        nodes[node] = nd;
        for (int k = 0; k < 3; ++k)
        {
            __stcg(node_box + 6 * int64_t(node) + k, fminf(b[0][k], b[1][k]));
            __stcg(node_box + 6 * int64_t(node) + 3 + k, fmaxf(b[0][3 + k], b[1][3 + k]));
        }
        node = parent_node[node];
    }
}

__global__ void k_depth(int n, const int* __restrict__ parent_node, const int* __restrict__ parent_leaf, int* depth)
{
    int const l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= n)
        return;
    int d = 1;
    int node = parent_leaf[l];
    while (node >= 0 && d <= n)
    {
        ++d;
        node = parent_node[node];
    }
    atomicMax(depth, d); // d > n only for a broken parent chain
}

// ---- traversal ----------------------------------------------------------------------------------------------
// Moller-Trumbore sign with NaiveIntersector's arithmetic and early rejections, in unfused precision S.
template <class S>
__device__ __forceinline__ int mt_sign(ev3<S> p, ev3<S> dir, ev3<S> a, ev3<S> b, ev3<S> c, bool* tie = nullptr)
{
    ev3<S> const e1 = b - a;
    ev3<S> const e2 = c - a;
    ev3<S> const h = ecross(dir, e2);
    S const det = edot(e1, h);
    if (det.v == 0)
        return 0;
    S const inv = S(1) / det;
    ev3<S> const s = p - a;
    S const u = inv * edot(s, h);
    if (u.v < 0 || u.v > 1)
        return 0;
    ev3<S> const q = ecross(s, e1);
    S const v = inv * edot(dir, q);
    if (v.v < 0 || (u + v).v > 1)
        return 0;
    S const t = inv * edot(e2, q);
    if (t.v < 0)
        return 0;
    // a counted hit exactly on the triangle's boundary (an edge or a vertex: the neighbour sharing it counts the
    // same crossing again) or at the query itself
    if (tie)
        *tie = u.v == 0 || v.v == 0 || (u + v).v == 1 || t.v == 0;
    ev3<S> const ng = ecross(e1, e2);
    return edot(ng, dir).v > 0 ? 1 : -1;
}

template <class T>
__device__ __forceinline__ int leaf_test(const T* __restrict__ tri, int leaf, ev3<typename exact_of<T>::type> p,
                                         ev3<typename exact_of<T>::type> dir)
{
    using S = typename exact_of<T>::type;
    const T* r = tri + 9 * int64_t(leaf);
    ev3<S> const a{S(r[0]), S(r[1]), S(r[2])};
    ev3<S> const b{S(r[3]), S(r[4]), S(r[5])};
    ev3<S> const c{S(r[6]), S(r[7]), S(r[8])};
    return mt_sign(p, dir, a, b, c);
}

// One query per thread.  The walk itself is float work only; the exact (FP64 for double input) leaf tests are
// the expensive part, so candidate leaves that pass the float pre-test are collected during the walk and tested
// after it: the lanes of a warp then run their j-th exact test together instead of one divergent lane at a time
// in the middle of the walk.  A full candidate list is tested early, so any number of candidates is handled.
constexpr int kTravBlock = 128;
constexpr int kCand = 8;

template <class T>
__global__ void __launch_bounds__(kTravBlock) k_traverse(const BvhNode* __restrict__ nodes, const T* __restrict__ tri,
                                                         const float4* __restrict__ leaf_uv, int64_t n_tri,
                                                         float scene_scale, Frame32 f, const T* __restrict__ pos,
                                                         int64_t n, int32_t* __restrict__ counts, T dx, T dy, T dz,
                                                         int* flags)
{
    using S = typename exact_of<T>::type;
    ev3<S> const dir{S(dx), S(dy), S(dz)};
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    {
        T const px = pos[3 * i], py = pos[3 * i + 1], pz = pos[3 * i + 2];
        ev3<S> const p{S(px), S(py), S(pz)};
        int sum = 0;
        if (n_tri == 1)
        {
            sum = leaf_test<T>(tri, 0, p, dir);
        }
        else if (n_tri > 1)
        {
            float const ox = float(px), oy = float(py), oz = float(pz);
            float const u = f.r[0] * ox + f.r[1] * oy + f.r[2] * oz;
            float const v = f.r[3] * ox + f.r[4] * oy + f.r[5] * oz;
            float const w = f.r[6] * ox + f.r[7] * oy + f.r[8] * oz;
            float const qmax = fmaxf(fmaxf(fabsf(ox), fabsf(oy)), fabsf(oz));
            float const tol = (qmax + scene_scale) * 3.8146973e-6f + 1e-30f; // 2^-18 of the coordinate scale
            float const m8 = margin_rotated(qmax, scene_scale);
            // Double input: most candidates are decided in float by certain_leaf, whose margins are ~1e9 times the
            // FP64 test's rounding; the rest take NaiveIntersector's exact test.  Float input always takes the exact
            // test: its own rounding is not small enough against the margin for very thin triangles.
            auto const decide = [&](int leaf) -> int
            {
                if constexpr (std::is_same_v<T, double>)
                {
                    int const c = certain_leaf(leaf_uv, leaf, u, v, w, m8);
                    if (c != 2)
                        return c;
                }
                return leaf_test<T>(tri, leaf, p, dir);
            };
            int cand[kCand];
            int nc = 0;
            bool const ok = hier_walk(nodes, leaf_uv, u, v, w, tol, m8,
                                      [&](int leaf)
                                      {
                                          if (nc == kCand)
                                          {
                                              for (int j = 0; j < kCand; ++j)
                                                  sum += decide(cand[j]);
                                              nc = 0;
                                          }
                                          cand[nc++] = leaf;
                                      });
            if (!ok)
                atomicOr(flags + FLAG_STACK, 1);
            for (int j = 0; j < nc; ++j)
                sum += decide(cand[j]);
        }
        counts[i] = sum;
    }
}

// ---- integer term through a grid of cells --------------------------------------------------------------------
// Every ray of a batch has the same direction, so in the ray frame a ray is a point (u, v) and a depth w.  A uniform
// grid over (u, v) lists, per cell, the leaves whose (u, v) box widened by `margin` overlaps the cell; a ray reads
// its cell's list instead of walking the hierarchy.  The leaves it then considers are a superset of the walk's (a
// listed leaf whose box the point misses by more than the walk's tolerance is one the exact test answers 0 for),
// and they go through the same conditions -- top of the leaf above the query's depth, may_hit -- and the same
// decision, so the counts are the walk's.  Neighbouring rays share cells, so the lists and leaves are read
// coherently, and there is no stack.
// Order-preserving encodings of floats as unsigned (for atomic min / max).
__device__ __forceinline__ unsigned f2o(float x)
{
    unsigned const b = __float_as_uint(x);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
float o2f(unsigned o)
{
    unsigned const b = (o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o;
    float f;
    std::memcpy(&f, &b, sizeof(f));
    return f;
}

// (u, v) box of a leaf from its float corners; false for a box with a NaN (never listed, as the walk never
// reaches it)
__device__ __forceinline__ bool leaf_box_uv(const float4* __restrict__ leaf_uv, int64_t l, float margin, float& u0,
                                            float& v0, float& u1, float& v1)
{
    float4 const a = leaf_uv[kLeafF4 * l], b = leaf_uv[kLeafF4 * l + 1];
    u0 = fminf(fminf(a.x, a.z), b.x) - margin;
    u1 = fmaxf(fmaxf(a.x, a.z), b.x) + margin;
    v0 = fminf(fminf(a.y, a.w), b.y) - margin;
    v1 = fmaxf(fmaxf(a.y, a.w), b.y) + margin;
    bool const nan = isnan(a.x) || isnan(a.y) || isnan(a.z) || isnan(a.w) || isnan(b.x) || isnan(b.y);
    return !nan && u0 <= u1 && v0 <= v1;
}

// ext: min u, min v, max u, max v of the widened boxes, order-encoded
__global__ void k_cell_extent(const float4* __restrict__ leaf_uv, int64_t n, float margin, unsigned* ext)
{
    unsigned mn[2] = {0xFFFFFFFFu, 0xFFFFFFFFu}, mx[2] = {0u, 0u};
    for (int64_t l = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; l < n; l += int64_t(gridDim.x) * blockDim.x)
    {
        float u0, v0, u1, v1;
        if (!leaf_box_uv(leaf_uv, l, margin, u0, v0, u1, v1))
            continue;
        mn[0] = min(mn[0], f2o(u0));
        mn[1] = min(mn[1], f2o(v0));
        mx[0] = max(mx[0], f2o(u1));
        mx[1] = max(mx[1], f2o(v1));
    }
    for (int k = 0; k < 2; ++k)
        for (int o = 16; o > 0; o >>= 1)
        {
            mn[k] = min(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
            mx[k] = max(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
        }
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 2; ++k)
        {
            atomicMin(ext + k, mn[k]);
            atomicMax(ext + 2 + k, mx[k]);
        }
}

// counts[c] += 1 for every cell c of every leaf (cursor == nullptr), or the leaf written at its slot of each of
// its cells (cursor: a copy of the offsets)
__global__ void k_cell_bin(const float4* __restrict__ leaf_uv, int64_t n, float margin, CellView g,
                           unsigned* __restrict__ counts, unsigned long long* __restrict__ total,
                           unsigned* __restrict__ cursor, int* __restrict__ list)
{
    for (int64_t l = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; l < n; l += int64_t(gridDim.x) * blockDim.x)
    {
        float u0, v0, u1, v1;
        if (!leaf_box_uv(leaf_uv, l, margin, u0, v0, u1, v1))
            continue;
        int const iu0 = cell_of(u0, g.umin, g.inv_u, g.gu), iu1 = cell_of(u1, g.umin, g.inv_u, g.gu);
        int const iv0 = cell_of(v0, g.vmin, g.inv_v, g.gv), iv1 = cell_of(v1, g.vmin, g.inv_v, g.gv);
        if (total)
            atomicAdd(total, (unsigned long long)(iu1 - iu0 + 1) * (unsigned long long)(iv1 - iv0 + 1));
        for (int iv = iv0; iv <= iv1; ++iv)
            for (int iu = iu0; iu <= iu1; ++iu)
            {
                int64_t const c = int64_t(iv) * g.gu + iu;
                if (cursor)
                    list[atomicAdd(cursor + c, 1u)] = int(l);
                else
                    atomicAdd(counts + c, 1u);
            }
    }
}

// Double input: most candidates are decided in float by certain_leaf; the undecided ones take NaiveIntersector's
// exact test a warp's worth at a time (leafq_push).  Float input takes the exact test on every candidate, in place
// (its own test is float arithmetic, and its rounding is not small against the margin for very thin triangles).
// The loop over queries is warp-uniform: a lane past the end has no candidates.  stats: counters, or null.
template <class T>
__global__ void __launch_bounds__(kTravBlock, 8) k_cells(const BvhNode* __restrict__ nodes, const T* __restrict__ tri,
                                                      const float4* __restrict__ leaf_uv, float scene_scale,
                                                      Frame32 f, CellView g, const T* __restrict__ pos, int64_t n,
                                                      int32_t* __restrict__ counts, T dx, T dy, T dz, int* flags,
                                                      long long* stats)
{
    using S = typename exact_of<T>::type;
    constexpr bool kQueue = std::is_same_v<T, double>;
    __shared__ int s_leaf[kTravBlock / 32][kLeafQCap];
    __shared__ long long s_query[kTravBlock / 32][kLeafQCap];
    ev3<S> const dir{S(dx), S(dy), S(dz)};
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    LeafQueue lq;
    lq.leaf = s_leaf[warp];
    lq.query = s_query[warp];
    auto const exact = [&](long long qi, int leaf) -> int
    {
        ev3<S> const p{S(pos[3 * qi]), S(pos[3 * qi + 1]), S(pos[3 * qi + 2])};
        return leaf_test<T>(tri, leaf, p, dir);
    };
    long long n_q = 0, n_entries = 0, n_leaves = 0, n_exact = 0;
    int64_t const stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t base = blockIdx.x * int64_t(blockDim.x) + (threadIdx.x & ~31); base < n; base += stride)
    {
        int64_t const i = base + lane;
        int und[kUndecided];
        int nu = 0;
        if (i < n)
        {
            T const px = pos[3 * i], py = pos[3 * i + 1], pz = pos[3 * i + 2];
            float const ox = float(px), oy = float(py), oz = float(pz);
            float const u = f.r[0] * ox + f.r[1] * oy + f.r[2] * oz;
            float const v = f.r[3] * ox + f.r[4] * oy + f.r[5] * oz;
            float const w = f.r[6] * ox + f.r[7] * oy + f.r[8] * oz;
            float const qmax = fmaxf(fmaxf(fabsf(ox), fabsf(oy)), fabsf(oz));
            float const tol = (qmax + scene_scale) * 3.8146973e-6f + 1e-30f; // as in k_traverse
            float const m8 = margin_rotated(qmax, scene_scale);
            int sum = 0;
            auto const consider = [&](int leaf)
            {
                ++n_leaves;
                if constexpr (kQueue)
                {
                    int const c = certain_leaf(leaf_uv, leaf, u, v, w, m8);
                    if (c != 2)
                    {
                        sum += c;
                        return;
                    }
                    ++n_exact;
                    if (nu < kUndecided)
                    {
                        und[nu++] = leaf;
                        return;
                    }
                }
                else
                    ++n_exact;
                sum += leaf_test<T>(tri, leaf, ev3<S>{S(px), S(py), S(pz)}, dir);
            };
            if (tol <= g.tol_max)
                n_entries += cell_candidates(g, leaf_uv, u, v, w, tol, m8, consider);
            else if (!hier_walk(nodes, leaf_uv, u, v, w, tol, m8, consider))
                atomicOr(flags + FLAG_STACK, 1);
            counts[i] = sum;
            ++n_q;
        }
        if constexpr (kQueue)
            leafq_push(lq, und, nu, i, lane, counts, exact);
    }
    if constexpr (kQueue)
        leafq_drain(lq, lane, counts, exact);
    if (stats)
        integer_stats(stats, n_q, n_entries, n_leaves, n_exact);
}

// ---- every triangle against every query (NaiveIntersector's loop), with a bounding-box cull ------------------
// The scan tests each (query, triangle) pair with NaiveIntersector's own Moller-Trumbore arithmetic, skipping
// only pairs that test cannot count: in a frame whose third axis is the ray direction, the ray of a query is the
// point (u, v) of the query, and a counted hit lies within the triangle's (u, v) box up to the test's FP64
// rounding (~1e-15 of the coordinates).  Boxes are rounded outward to float and the query's point is widened by
// 2^-20 of (query + scene) coordinate scale, far above both roundings.  A triangle or query with a NaN or an
// infinity is never skipped.  So the counts, and the ties, are the full scan's; no hierarchy is involved.
constexpr int kScanBlock = 128;
constexpr int kScanK = 4;        // queries per thread
constexpr int kScanTile = 2048;  // boxes per shared-memory tile (32 KB)

// Box (umin, vmin, umax, vmax) of every triangle in the frame f, and the largest |vertex coordinate| as float bits
// (scale_bits, atomicMax; the coordinates' absolute values order like their bits).
__global__ void k_scan_boxes(const double* __restrict__ verts, const int32_t* __restrict__ idx, int64_t n_tri, Frame64 f,
                             float4* __restrict__ boxes, unsigned* __restrict__ scale_bits)
{
    float amax = 0.f;
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < n_tri; t += int64_t(gridDim.x) * blockDim.x)
    {
        double lo[2] = {INFINITY, INFINITY}, hi[2] = {-INFINITY, -INFINITY};
        bool finite = true;
        for (int c = 0; c < 3; ++c)
        {
            const double* x = verts + 3 * int64_t(idx[3 * t + c]);
            finite &= isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]);
            amax = fmaxf(amax, float(fmax(fmax(fabs(x[0]), fabs(x[1])), fabs(x[2]))));
            for (int r = 0; r < 2; ++r)
            {
                double const u = f.r[3 * r] * x[0] + f.r[3 * r + 1] * x[1] + f.r[3 * r + 2] * x[2];
                lo[r] = fmin(lo[r], u);
                hi[r] = fmax(hi[r], u);
            }
        }
        boxes[t] = finite ? make_float4(__double2float_rd(lo[0]), __double2float_rd(lo[1]), __double2float_ru(hi[0]),
                                        __double2float_ru(hi[1]))
                          : make_float4(-INFINITY, -INFINITY, INFINITY, INFINITY);
    }
    amax = isfinite(amax) ? amax : 0.f;
    for (int o = 16; o > 0; o >>= 1)
        amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    if ((threadIdx.x & 31) == 0)
        atomicMax(scale_bits, __float_as_uint(amax));
}

__global__ void __launch_bounds__(kScanBlock) k_scan(const double* __restrict__ verts, const int32_t* __restrict__ idx,
                                                     const float4* __restrict__ boxes, int64_t n_tri,
                                                     const unsigned* __restrict__ scale_bits, Frame64 f,
                                                     const double* __restrict__ pos, int64_t n,
                                                     int32_t* __restrict__ counts, int32_t* __restrict__ ties,
                                                     double dx, double dy, double dz)
{
    __shared__ float4 sbox[kScanTile];
    ev3<rd> const dir{rd(dx), rd(dy), rd(dz)};
    float const scene = __uint_as_float(*scale_bits);
    int64_t const per_block = int64_t(kScanBlock) * kScanK;
    for (int64_t base = blockIdx.x * per_block; base < n; base += int64_t(gridDim.x) * per_block)
    {
        float ulo[kScanK], uhi[kScanK], vlo[kScanK], vhi[kScanK];
        int sum[kScanK], tie[kScanK];
#pragma unroll
        for (int k = 0; k < kScanK; ++k)
        {
            int64_t const i = base + threadIdx.x + int64_t(k) * kScanBlock;
            sum[k] = 0;
            tie[k] = 0;
            if (i >= n)
            {
                ulo[k] = uhi[k] = vlo[k] = vhi[k] = __int_as_float(0x7fffffff); // NaN: every comparison fails
                continue;
            }
            double const x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
            double const u = f.r[0] * x + f.r[1] * y + f.r[2] * z, v = f.r[3] * x + f.r[4] * y + f.r[5] * z;
            float const m = 9.5367432e-7f * (float(fmax(fmax(fabs(x), fabs(y)), fabs(z))) + scene); // 2^-20
            bool const ok = fabs(u) < 1e30 && fabs(v) < 1e30 && isfinite(m); // else (NaN, huge) test everything
            ulo[k] = ok ? float(u) - m : -INFINITY;
            uhi[k] = ok ? float(u) + m : INFINITY;
            vlo[k] = ok ? float(v) - m : -INFINITY;
            vhi[k] = ok ? float(v) + m : INFINITY;
        }
        for (int64_t t0 = 0; t0 < n_tri; t0 += kScanTile)
        {
            int const cnt = int(n_tri - t0 < kScanTile ? n_tri - t0 : int64_t(kScanTile));
            __syncthreads();
            for (int j = threadIdx.x; j < cnt; j += kScanBlock)
                sbox[j] = boxes[t0 + j];
            __syncthreads();
            for (int j = 0; j < cnt; ++j)
            {
                float4 const b = sbox[j];
#pragma unroll
                for (int k = 0; k < kScanK; ++k)
                {
                    if (b.x <= uhi[k] && b.z >= ulo[k] && b.y <= vhi[k] && b.w >= vlo[k])
                    {
                        int64_t const i = base + threadIdx.x + int64_t(k) * kScanBlock;
                        int64_t const t = t0 + j;
                        const double* a = verts + 3 * int64_t(idx[3 * t]);
                        const double* bb = verts + 3 * int64_t(idx[3 * t + 1]);
                        const double* c = verts + 3 * int64_t(idx[3 * t + 2]);
                        bool tt = false;
                        int const h = mt_sign(ev3<rd>{rd(pos[3 * i]), rd(pos[3 * i + 1]), rd(pos[3 * i + 2])}, dir,
                                              ev3<rd>{rd(a[0]), rd(a[1]), rd(a[2])},
                                              ev3<rd>{rd(bb[0]), rd(bb[1]), rd(bb[2])},
                                              ev3<rd>{rd(c[0]), rd(c[1]), rd(c[2])}, &tt);
                        sum[k] += h;
                        tie[k] += (h != 0 && tt) ? 1 : 0;
                    }
                }
            }
        }
#pragma unroll
        for (int k = 0; k < kScanK; ++k)
        {
            int64_t const i = base + threadIdx.x + int64_t(k) * kScanBlock;
            if (i < n)
            {
                counts[i] = sum[k];
                if (ties)
                    ties[i] = tie[k];
            }
        }
    }
}

// RAII device buffer for build temporaries.
struct Tmp
{
    void* p = nullptr;
    ~Tmp()
    {
        if (p)
            cudaFree(p);
    }
    int alloc(size_t bytes)
    {
        cudaError_t const e = cudaMalloc(&p, bytes ? bytes : 1);
        if (e != cudaSuccess)
        {
            cudaGetLastError();
            p = nullptr;
            return fail(e == cudaErrorMemoryAllocation ? AGWN_ERR_NOMEM : AGWN_ERR_CUDA, "cudaMalloc(%zu): %s", bytes,
                        cudaGetErrorString(e));
        }
        return AGWN_OK;
    }
    template <class U>
    U* as() const
    {
        return static_cast<U*>(p);
    }
};

void bvh_free(Bvh* b)
{
    if (b && b->tri)
        cudaFree(b->tri);
    if (b)
        b->tri = nullptr;
}

// Copies the indexed triangles to the device.
template <class T>
int bvh_make(Context& ctx, const T* vertices, int64_t nv, const int32_t* indices, int64_t n_idx, Bvh* out)
{
    AGWN_CHECK_ARG(nv >= 0 && n_idx >= 0 && n_idx % 3 == 0, "index count must be a non-negative multiple of 3");
    AGWN_CHECK_ARG(n_idx / 3 < (int64_t(1) << 31) - 1, "too many triangles");
    AGWN_CHECK_ARG(n_idx == 0 || (vertices && indices && nv > 0), "null vertices/indices");
    int64_t const n_tri = n_idx / 3;
    out->scalar_bytes = int(sizeof(T));
    out->n_tri = n_tri;
    out->device = ctx.device;
    out->generation = g_generation.fetch_add(1);
    if (n_tri == 0)
        return AGWN_OK;
    cudaStream_t const st = ctx.stream;
    const void* dv = nullptr;
    const void* di = nullptr;
    AGWN_TRY(stage_in(ctx, vertices, sizeof(T) * 3 * nv, S_MISC0, &dv));
    AGWN_TRY(stage_in(ctx, indices, sizeof(int32_t) * n_idx, S_MISC1, &di));
    AGWN_TRY_CUDA(cudaMalloc(&out->tri, sizeof(T) * 9 * n_tri));
    Tmp misc;
    AGWN_TRY(misc.alloc(sizeof(unsigned)));
    AGWN_TRY_CUDA(cudaMemsetAsync(misc.p, 0, sizeof(unsigned), st));
    AGWN_TRY_CUDA(cudaMemsetAsync(ctx.d_flags + FLAG_COUNT - 1, 0, sizeof(int), st));
    int const g = std::min(div_up(n_tri, 256), 8 * ctx.sm_count);
    AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
    k_gather<T><<<g, 256, 0, st>>>(static_cast<const T*>(dv), nv, static_cast<const int32_t*>(di), n_tri,
                                   static_cast<T*>(out->tri), misc.as<unsigned>(), ctx.d_flags);
    AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
    unsigned scale_bits = 0;
    int bad = 0;
    AGWN_TRY_CUDA(cudaMemcpyAsync(&scale_bits, misc.p, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    AGWN_TRY_CUDA(cudaMemcpyAsync(&bad, ctx.d_flags + FLAG_COUNT - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    AGWN_TRY_CUDA(cudaStreamSynchronize(st));
    if (bad)
    {
        AGWN_TRY_CUDA(cudaMemsetAsync(ctx.d_flags + FLAG_COUNT - 1, 0, sizeof(int), st));
        return fail(AGWN_ERR_INVALID, "triangle index out of range [0, %lld)", (long long)nv);
    }
    float scale;
    std::memcpy(&scale, &scale_bits, sizeof(float));
    out->scene_scale = scale;
    return AGWN_OK;
}

} // namespace

Frame64 ray_frame(const double* dir)
{
    double const nn = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    double z[3] = {dir[0] / nn, dir[1] / nn, dir[2] / nn};
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
    double y[3] = {z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2], z[0] * x[1] - z[1] * x[0]};
    Frame64 f;
    for (int k = 0; k < 3; ++k)
    {
        f.r[k] = x[k];
        f.r[3 + k] = y[k];
        f.r[6 + k] = z[k];
    }
    return f;
}

template <class T>
int build_hier(Context& ctx, const T* tri_in, int64_t n_tri, const double* dir, Hier& out, unsigned* order_out)
{
    double const nn = dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2];
    AGWN_CHECK_ARG(nn > 0 && std::isfinite(nn), "ray direction must be finite and nonzero");
    cudaStream_t const st = ctx.stream;
    Frame64 const f = ray_frame(dir);
    AGWN_TRY_CUDA(cudaStreamSynchronize(st)); // the buffers may still be read by queued traversals
    AGWN_TRY(out.tri.reserve(sizeof(T) * 9 * std::max<int64_t>(1, n_tri)));
    AGWN_TRY(out.nodes.reserve(sizeof(BvhNode) * std::max<int64_t>(1, n_tri - 1)));
    AGWN_TRY(out.leaf_uv.reserve(sizeof(float4) * kLeafF4 * std::max<int64_t>(1, n_tri)));
    T* tri = static_cast<T*>(out.tri.ptr);
    int32_t depth = n_tri > 0 ? 1 : 0;
    unsigned scale_bits = 0;
    if (n_tri == 1)
    {
        AGWN_TRY_CUDA(cudaMemcpyAsync(tri, tri_in, sizeof(T) * 9, cudaMemcpyDeviceToDevice, st));
        if (order_out)
            AGWN_TRY_CUDA(cudaMemsetAsync(order_out, 0, sizeof(unsigned), st));
    }
    if (n_tri > 1)
    {
        Tmp box, cen, misc, keys0, vals0, keys1, vals1, hist, left, right, pnode, pleaf, nbox, visit, leafbox;
        AGWN_TRY(box.alloc(sizeof(float) * 6 * n_tri));
        AGWN_TRY(cen.alloc(sizeof(float) * 2 * n_tri));
        AGWN_TRY(misc.alloc(sizeof(unsigned) * 8));
        AGWN_TRY(keys0.alloc(sizeof(unsigned) * n_tri));
        AGWN_TRY(vals0.alloc(sizeof(unsigned) * n_tri));
        AGWN_TRY(keys1.alloc(sizeof(unsigned) * n_tri));
        AGWN_TRY(vals1.alloc(sizeof(unsigned) * n_tri));
        int const n_rs_blocks = div_up(n_tri, kRsTile);
        AGWN_TRY(hist.alloc(sizeof(unsigned) * 256 * n_rs_blocks));
        Tmp hsum;
        AGWN_TRY(hsum.alloc(sizeof(unsigned) * scan_sums_count(int64_t(256) * n_rs_blocks)));
        AGWN_TRY(left.alloc(sizeof(int) * n_tri));
        AGWN_TRY(right.alloc(sizeof(int) * n_tri));
        AGWN_TRY(pnode.alloc(sizeof(int) * n_tri));
        AGWN_TRY(pleaf.alloc(sizeof(int) * n_tri));
        AGWN_TRY(nbox.alloc(sizeof(float) * 6 * n_tri));
        AGWN_TRY(visit.alloc(sizeof(int) * n_tri));
        AGWN_TRY(leafbox.alloc(sizeof(float) * 6 * n_tri));
        // (u, v) min, (u, v) max, largest |coordinate| bits, -, -, depth
        unsigned init[8] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u, 0u, 0u, 0u};
        AGWN_TRY_CUDA(cudaMemcpyAsync(misc.p, init, sizeof(init), cudaMemcpyHostToDevice, st));
        AGWN_TRY_CUDA(cudaMemsetAsync(visit.p, 0, sizeof(int) * n_tri, st));
        int const g = std::min(div_up(n_tri, 256), 8 * ctx.sm_count);
        int const gb = div_up(n_tri, 256);
        AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
        k_ray_boxes<T><<<g, 256, 0, st>>>(tri_in, n_tri, f, box.as<float>(), cen.as<float>(), misc.as<unsigned>(),
                                          misc.as<unsigned>() + 4);
        k_morton2<<<g, 256, 0, st>>>(cen.as<float>(), n_tri, misc.as<unsigned>(), keys0.as<unsigned>(),
                                     vals0.as<unsigned>());
        unsigned *ka = keys0.as<unsigned>(), *va = vals0.as<unsigned>(), *kb = keys1.as<unsigned>(),
                 *vb = vals1.as<unsigned>();
        for (int pass = 0; pass < 4; ++pass)
        {
            int const shift = 8 * pass;
            k_rs_hist<<<n_rs_blocks, kRsBlock, 0, st>>>(ka, n_tri, shift, hist.as<unsigned>(), n_rs_blocks);
            scan_counters(st, hist.as<unsigned>(), int64_t(256) * n_rs_blocks, hsum.as<unsigned>());
            k_rs_scatter<<<n_rs_blocks, kRsBlock, 0, st>>>(ka, va, n_tri, shift, hist.as<unsigned>(), n_rs_blocks, kb,
                                                           vb);
            std::swap(ka, kb);
            std::swap(va, vb);
        }
        k_leaves<T><<<g, 256, 0, st>>>(tri_in, va, box.as<float>(), n_tri, f, tri, leafbox.as<float>(),
                                       static_cast<float*>(out.leaf_uv.ptr));
        k_karras<<<gb, 256, 0, st>>>(ka, int(n_tri), left.as<int>(), right.as<int>(), pnode.as<int>(),
                                     pleaf.as<int>());
        k_refit<<<gb, 256, 0, st>>>(int(n_tri), left.as<int>(), right.as<int>(), pnode.as<int>(), pleaf.as<int>(),
                                    leafbox.as<float>(), nbox.as<float>(), visit.as<int>(),
                                    static_cast<BvhNode*>(out.nodes.ptr));
        k_depth<<<gb, 256, 0, st>>>(int(n_tri), pnode.as<int>(), pleaf.as<int>(),
                                    reinterpret_cast<int*>(misc.as<unsigned>() + 7));
        AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
        if (order_out)
            AGWN_TRY_CUDA(cudaMemcpyAsync(order_out, va, sizeof(unsigned) * n_tri, cudaMemcpyDeviceToDevice, st));
        unsigned back[8];
        AGWN_TRY_CUDA(cudaMemcpyAsync(back, misc.p, sizeof(back), cudaMemcpyDeviceToHost, st));
        AGWN_TRY_CUDA(cudaStreamSynchronize(st));
        depth = int32_t(back[7]);
        scale_bits = back[4];
        if (depth > n_tri)
            return fail(AGWN_ERR_CUDA, "hierarchy build produced a broken parent chain (depth %d for %lld triangles)",
                        depth, (long long)n_tri);
    }
    float scale = 0.f;
    std::memcpy(&scale, &scale_bits, sizeof(float));
    for (int k = 0; k < 9; ++k)
        out.frame[k] = float(f.r[k]);
    out.depth = depth;
    out.n_tri = n_tri;
    out.scale = scale;
    return AGWN_OK;
}

template int build_hier<double>(Context&, const double*, int64_t, const double*, Hier&, unsigned*);
template int build_hier<float>(Context&, const float*, int64_t, const double*, Hier&, unsigned*);

namespace
{
// The hierarchy of `bvh` in the frame of `dir`, built into ctx.ray_cache unless it is already there.
template <class T>
int ray_hierarchy(Context& ctx, const Bvh& bvh, const T* dir_host)
{
    RayCache& rc = ctx.ray_cache;
    double const dir[3] = {double(dir_host[0]), double(dir_host[1]), double(dir_host[2])};
    if (rc.generation == bvh.generation && rc.scalar_bytes == bvh.scalar_bytes &&
        std::memcmp(rc.dir, dir, sizeof(dir)) == 0)
        return AGWN_OK;
    rc.generation = 0; // invalid until the build completes
    rc.cells.valid = false;
    AGWN_TRY(build_hier<T>(ctx, static_cast<const T*>(bvh.tri), bvh.n_tri, dir, rc.h, nullptr));
    std::memcpy(rc.dir, dir, sizeof(dir));
    rc.scalar_bytes = bvh.scalar_bytes;
    rc.generation = bvh.generation;
    bvh.depth = rc.h.depth;
    return AGWN_OK;
}
} // namespace

// The cell grid of the cached hierarchy (its leaves' float (u, v) corners), about 16 cells per leaf over the
// widened boxes' extent (at most 2^22 cells).  Finer cells hold fewer leaves, so a query reads fewer list entries:
// on a 76,496-triangle icosphere with 256^3 grid queries 2 cells per leaf read 5.06 entries per query (1.09 ms),
// 16 read 3.49 (0.83 ms); 32 and 64 gained no more.  Leaf boxes are widened by 4 * 2^-18 of the scene scale; a
// query takes the grid while its own tolerance (qmax + scene) * 2^-18 stays below 3.5 * 2^-18 of the scene scale
// (qmax <= 2.5 * scene), which leaves room for the one-ulp difference between the corners and the walk's
// outward-rounded boxes.
int build_cells(Context& ctx, const Hier& h, float scene_scale, CellGrid& g)
{
    g.valid = false;
    int64_t const n = h.n_tri;
    if (n < 2 || !(scene_scale > 0.f) || !std::isfinite(scene_scale))
        return AGWN_OK;
    cudaStream_t const st = ctx.stream;
    float const margin = 4.f * scene_scale * 3.8146973e-6f;
    const float4* leaf_uv = static_cast<const float4*>(h.leaf_uv.ptr);
    Tmp ext; // 4 order-encoded extents, then the 64-bit entry count
    AGWN_TRY(ext.alloc(sizeof(unsigned) * 6));
    unsigned const init[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u, 0u};
    AGWN_TRY_CUDA(cudaMemcpyAsync(ext.p, init, sizeof(init), cudaMemcpyHostToDevice, st));
    auto* const total64 = reinterpret_cast<unsigned long long*>(ext.as<unsigned>() + 4);
    int const gl = std::min(div_up(n, 256), 8 * ctx.sm_count);
    AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
    k_cell_extent<<<gl, 256, 0, st>>>(leaf_uv, n, margin, ext.as<unsigned>());
    AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
    unsigned back[4];
    AGWN_TRY_CUDA(cudaMemcpyAsync(back, ext.p, sizeof(back), cudaMemcpyDeviceToHost, st));
    AGWN_TRY_CUDA(cudaStreamSynchronize(st));
    if (back[0] == 0xFFFFFFFFu)
        return AGWN_OK; // no leaf with a finite box: keep the walk
    CellView v{};
    v.umin = o2f(back[0]);
    v.vmin = o2f(back[1]);
    v.umax = o2f(back[2]);
    v.vmax = o2f(back[3]);
    double const W = double(v.umax) - double(v.umin), H = double(v.vmax) - double(v.vmin);
    if (!(W > 0) || !(H > 0) || !std::isfinite(W) || !std::isfinite(H))
        return AGWN_OK;
    double const target = double(std::min<int64_t>(std::max<int64_t>(16 * n, 1024), int64_t(1) << 22));
    double const side = std::sqrt(W * H / target);
    v.gu = int(std::min(4096.0, std::max(1.0, std::ceil(W / side))));
    v.gv = int(std::min(4096.0, std::max(1.0, std::ceil(H / side))));
    v.inv_u = float(double(v.gu) / W);
    v.inv_v = float(double(v.gv) / H);
    int64_t const n_cells = int64_t(v.gu) * v.gv;
    AGWN_TRY(g.offsets.reserve(sizeof(unsigned) * (n_cells + 1)));
    unsigned* const off = static_cast<unsigned*>(g.offsets.ptr);
    AGWN_TRY_CUDA(cudaMemsetAsync(off, 0, sizeof(unsigned) * (n_cells + 1), st));
    Tmp osum;
    AGWN_TRY(osum.alloc(sizeof(unsigned) * scan_sums_count(n_cells + 1)));
    AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
    k_cell_bin<<<gl, 256, 0, st>>>(leaf_uv, n, margin, v, off, total64, nullptr, nullptr);
    scan_counters(st, off, n_cells + 1, osum.as<unsigned>());
    AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
    unsigned long long total = 0;
    AGWN_TRY_CUDA(cudaMemcpyAsync(&total, total64, sizeof(total), cudaMemcpyDeviceToHost, st));
    AGWN_TRY_CUDA(cudaStreamSynchronize(st));
    if (total >= (1ull << 31))
        return AGWN_OK; // the lists would not fit 32-bit offsets: keep the walk
    AGWN_TRY(g.list.reserve(sizeof(int) * std::max<unsigned long long>(1, total)));
    Tmp cursor;
    AGWN_TRY(cursor.alloc(sizeof(unsigned) * n_cells));
    AGWN_TRY_CUDA(cudaMemcpyAsync(cursor.p, off, sizeof(unsigned) * n_cells, cudaMemcpyDeviceToDevice, st));
    AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
    k_cell_bin<<<gl, 256, 0, st>>>(leaf_uv, n, margin, v, nullptr, nullptr, cursor.as<unsigned>(),
                                   static_cast<int*>(g.list.ptr));
    AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
    AGWN_TRY_CUDA(cudaStreamSynchronize(st)); // the cursor is freed on return
    g.gu = v.gu;
    g.gv = v.gv;
    g.umin = v.umin;
    g.vmin = v.vmin;
    g.umax = v.umax;
    g.vmax = v.vmax;
    g.inv_u = v.inv_u;
    g.inv_v = v.inv_v;
    g.margin = margin;
    g.tol_max = 3.5f * scene_scale * 3.8146973e-6f;
    g.entries = int64_t(total);
    g.valid = true;
    return AGWN_OK;
}

template <class T>
int integer_prepare(Context& ctx, const Bvh& bvh, const T* dir_host)
{
    if (bvh.n_tri == 0)
        return AGWN_OK;
    AGWN_TRY(ray_hierarchy<T>(ctx, bvh, dir_host));
    CellGrid& cg = ctx.ray_cache.cells;
    if (ctx.integer_cells && bvh.n_tri > 1 && !cg.valid)
        AGWN_TRY(build_cells(ctx, ctx.ray_cache.h, float(bvh.scene_scale), cg));
    return AGWN_OK;
}

template int integer_prepare<double>(Context&, const Bvh&, const double*);
template int integer_prepare<float>(Context&, const Bvh&, const float*);

template <class T>
int integer_run(Context& ctx, const Bvh& bvh, const T* d_pos, int64_t n, int32_t* d_counts, const T* dir_host)
{
    if (n == 0)
        return AGWN_OK;
    if (bvh.n_tri == 0)
    {
        AGWN_TRY_CUDA(cudaMemsetAsync(d_counts, 0, sizeof(int32_t) * n, ctx.stream));
        return AGWN_OK;
    }
    AGWN_TRY(integer_prepare<T>(ctx, bvh, dir_host));
    Frame32 f;
    for (int k = 0; k < 9; ++k)
        f.r[k] = ctx.ray_cache.h.frame[k];
    int const block = kTravBlock;
    int const grid = int(std::min<int64_t>(div_up(n, block), int64_t(ctx.sm_count) * 16));
    CellGrid& cg = ctx.ray_cache.cells;
    if (ctx.integer_cells && bvh.n_tri > 1 && cg.valid)
    {
        CellView const v = cell_view(cg);
        AGWN_TRY(ctx.launch_begin(AGWN_K_INTEGER));
        k_cells<T><<<grid, block, 0, ctx.stream>>>(static_cast<const BvhNode*>(ctx.ray_cache.h.nodes.ptr),
                                                  static_cast<const T*>(ctx.ray_cache.h.tri.ptr),
                                                  static_cast<const float4*>(ctx.ray_cache.h.leaf_uv.ptr),
                                                  float(bvh.scene_scale), f, v, d_pos, n, d_counts, dir_host[0],
                                                  dir_host[1], dir_host[2], ctx.d_flags,
                                                  ctx.timing ? ctx.d_counters : nullptr);
        return ctx.launch_end(AGWN_K_INTEGER);
    }
    AGWN_TRY(ctx.launch_begin(AGWN_K_INTEGER));
    k_traverse<T><<<grid, block, 0, ctx.stream>>>(static_cast<const BvhNode*>(ctx.ray_cache.h.nodes.ptr),
                                                  static_cast<const T*>(ctx.ray_cache.h.tri.ptr),
                                                  static_cast<const float4*>(ctx.ray_cache.h.leaf_uv.ptr), bvh.n_tri,
                                                  float(bvh.scene_scale), f, d_pos, n, d_counts, dir_host[0],
                                                  dir_host[1], dir_host[2], ctx.d_flags);
    return ctx.launch_end(AGWN_K_INTEGER);
}

template int integer_run<double>(Context&, const Bvh&, const double*, int64_t, int32_t*, const double*);
template int integer_run<float>(Context&, const Bvh&, const float*, int64_t, int32_t*, const float*);

namespace
{
template <class T>
int bvh_create(agwn_context* ctx, const T* vertices, int64_t nv, const int32_t* indices, int64_t n_idx, agwn_bvh** out)
{
    AGWN_CHECK_ARG(ctx && out, "null context/out");
    *out = nullptr;
    clear_message();
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    auto* b = new agwn_bvh{};
    int const s = bvh_make<T>(*ctx, vertices, nv, indices, n_idx, b);
    if (s != AGWN_OK)
    {
        bvh_free(b);
        delete b;
        return s;
    }
    *out = b;
    return AGWN_OK;
}

template <class T>
int batch_integer(agwn_context* ctx, const agwn_bvh* bvh, const T* positions, int64_t n, int32_t* out, const T* dir)
{
    AGWN_CHECK_ARG(ctx && bvh && dir, "null context/intersector/dir");
    AGWN_CHECK_ARG(n >= 0, "negative size");
    AGWN_CHECK_ARG(n == 0 || (positions && out), "null positions/out");
    AGWN_CHECK_ARG(bvh->scalar_bytes == int(sizeof(T)), "intersector precision does not match the queries");
    clear_message();
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    if (n == 0)
        return AGWN_OK;
    const void* dpos = nullptr;
    void* dout = nullptr;
    bool host_out = false;
    AGWN_TRY(stage_in(*ctx, positions, sizeof(T) * 3 * n, S_QUERIES, &dpos));
    AGWN_TRY(stage_out(*ctx, out, sizeof(int32_t) * n, S_COUNTS, &dout, &host_out));
    if (bvh->n_tri == 0)
        AGWN_TRY_CUDA(cudaMemsetAsync(dout, 0, sizeof(int32_t) * n, ctx->stream));
    else
        AGWN_TRY(integer_run<T>(*ctx, *bvh, static_cast<const T*>(dpos), n, static_cast<int32_t*>(dout), dir));
    if (host_out)
    {
        AGWN_TRY_CUDA(cudaMemcpyAsync(out, dout, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
        return ctx->check_flags();
    }
    if (dpos != positions)
        return ctx->check_flags();
    return AGWN_OK;
}
} // namespace
} // namespace agwn

using namespace agwn;

extern "C"
{
int agwn_bvh_create_f64(agwn_context* ctx, const double* vertices, int64_t n_vertices, const int32_t* indices,
                        int64_t n_indices, agwn_bvh** out)
{
    return bvh_create<double>(ctx, vertices, n_vertices, indices, n_indices, out);
}
int agwn_bvh_create_f32(agwn_context* ctx, const float* vertices, int64_t n_vertices, const int32_t* indices,
                        int64_t n_indices, agwn_bvh** out)
{
    return bvh_create<float>(ctx, vertices, n_vertices, indices, n_indices, out);
}
int agwn_bvh_destroy(agwn_bvh* bvh)
{
    if (!bvh)
        return AGWN_OK;
    cudaSetDevice(bvh->device);
    cudaDeviceSynchronize();
    bvh_free(bvh);
    delete bvh;
    return AGWN_OK;
}
int agwn_bvh_info(const agwn_bvh* bvh, int64_t* n_triangles, int32_t* depth)
{
    AGWN_CHECK_ARG(bvh, "null intersector");
    if (n_triangles)
        *n_triangles = bvh->n_tri;
    if (depth)
        *depth = bvh->depth;
    return AGWN_OK;
}
int agwn_mesh_batch_integer_f64(agwn_context* ctx, const agwn_bvh* bvh, const double* positions, int64_t n,
                                int32_t* out_counts, const double* dir)
{
    return batch_integer<double>(ctx, bvh, positions, n, out_counts, dir);
}
int agwn_mesh_batch_integer_f32(agwn_context* ctx, const agwn_bvh* bvh, const float* positions, int64_t n,
                                int32_t* out_counts, const float* dir)
{
    return batch_integer<float>(ctx, bvh, positions, n, out_counts, dir);
}
static int bruteforce_f64(agwn_context* ctx, const double* vertices, int64_t n_vertices, const int32_t* indices,
                          int64_t n_indices, const double* positions, int64_t n, int32_t* out_counts, const double* dir,
                          int32_t* out_ties)
{
    AGWN_CHECK_ARG(ctx && dir, "null context/dir");
    AGWN_CHECK_ARG(n >= 0 && n_vertices >= 0 && n_indices >= 0 && n_indices % 3 == 0, "bad sizes");
    AGWN_CHECK_ARG(n == 0 || (positions && out_counts), "null positions/out");
    clear_message();
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    if (n == 0)
        return AGWN_OK;
    const void *dv = nullptr, *di = nullptr, *dpos = nullptr;
    void *dout = nullptr, *dties = nullptr;
    bool host_out = false, host_ties = false;
    AGWN_TRY(stage_in(*ctx, vertices, sizeof(double) * 3 * n_vertices, S_MISC0, &dv));
    AGWN_TRY(stage_in(*ctx, indices, sizeof(int32_t) * n_indices, S_MISC1, &di));
    AGWN_TRY(stage_in(*ctx, positions, sizeof(double) * 3 * n, S_QUERIES, &dpos));
    AGWN_TRY(stage_out(*ctx, out_counts, sizeof(int32_t) * n, S_COUNTS, &dout, &host_out));
    if (out_ties)
        AGWN_TRY(stage_out(*ctx, out_ties, sizeof(int32_t) * n, S_OUT, &dties, &host_ties));
    // indices are trusted here as in NaiveIntersector; validate them on the host when they live there
    if (!is_device_pointer(indices))
        for (int64_t i = 0; i < n_indices; ++i)
            AGWN_CHECK_ARG(indices[i] >= 0 && indices[i] < n_vertices, "triangle index out of range");
    int64_t const n_tri = n_indices / 3;
    if (n_tri == 0)
    {
        AGWN_TRY_CUDA(cudaMemsetAsync(dout, 0, sizeof(int32_t) * n, ctx->stream));
        if (dties)
            AGWN_TRY_CUDA(cudaMemsetAsync(dties, 0, sizeof(int32_t) * n, ctx->stream));
    }
    else
    {
        double const dn = dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2];
        AGWN_CHECK_ARG(dn > 0 && std::isfinite(dn), "ray direction must be finite and nonzero");
        void* boxes = nullptr;
        AGWN_TRY(ctx->scratch_reserve(S_MISC2, sizeof(float4) * n_tri + 256, &boxes));
        unsigned* const scale_bits = reinterpret_cast<unsigned*>(static_cast<char*>(boxes) + sizeof(float4) * n_tri);
        AGWN_TRY_CUDA(cudaMemsetAsync(scale_bits, 0, sizeof(unsigned), ctx->stream));
        Frame64 const f = ray_frame(dir);
        AGWN_TRY(ctx->launch_begin(AGWN_K_OTHER));
        k_scan_boxes<<<int(std::min<int64_t>(div_up(n_tri, 256), 4 * int64_t(ctx->sm_count))), 256, 0, ctx->stream>>>(
            static_cast<const double*>(dv), static_cast<const int32_t*>(di), n_tri, f, static_cast<float4*>(boxes),
            scale_bits);
        AGWN_TRY(ctx->launch_end(AGWN_K_OTHER));
        int const grid = int(std::min<int64_t>(div_up(n, int64_t(kScanBlock) * kScanK), int64_t(ctx->sm_count) * 8));
        AGWN_TRY(ctx->launch_begin(AGWN_K_INTEGER));
        k_scan<<<grid, kScanBlock, 0, ctx->stream>>>(static_cast<const double*>(dv), static_cast<const int32_t*>(di),
                                                     static_cast<const float4*>(boxes), n_tri, scale_bits, f,
                                                     static_cast<const double*>(dpos), n, static_cast<int32_t*>(dout),
                                                     static_cast<int32_t*>(dties), dir[0], dir[1], dir[2]);
        AGWN_TRY(ctx->launch_end(AGWN_K_INTEGER));
    }
    if (host_out)
        AGWN_TRY_CUDA(cudaMemcpyAsync(out_counts, dout, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (host_ties)
        AGWN_TRY_CUDA(cudaMemcpyAsync(out_ties, dties, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    return ctx->check_flags();
}

int agwn_mesh_batch_integer_bruteforce_f64(agwn_context* ctx, const double* vertices, int64_t n_vertices,
                                           const int32_t* indices, int64_t n_indices, const double* positions,
                                           int64_t n, int32_t* out_counts, const double* dir)
{
    return bruteforce_f64(ctx, vertices, n_vertices, indices, n_indices, positions, n, out_counts, dir, nullptr);
}

int agwn_mesh_batch_integer_ties_f64(agwn_context* ctx, const double* vertices, int64_t n_vertices,
                                     const int32_t* indices, int64_t n_indices, const double* positions, int64_t n,
                                     int32_t* out_counts, int32_t* out_ties, const double* dir)
{
    AGWN_CHECK_ARG(n == 0 || out_ties, "null out_ties");
    return bruteforce_f64(ctx, vertices, n_vertices, indices, n_indices, positions, n, out_counts, dir, out_ties);
}
} // extern "C"
