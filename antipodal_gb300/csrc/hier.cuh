// The ray-frame hierarchy shared by the integer term (lbvh.cu) and the robust evaluator (robust.cu): node layout,
// the conservative float pre-test of a leaf, a walk that reports candidate leaves, and the builder's interface.
#pragma once

#include "agwn_internal.cuh"

namespace agwn
{
// Internal node: boxes of both children in the ray frame, so one 64-byte fetch decides both.  lo_l.w / lo_r.w
// hold the child codes as int bits: >= 0 an internal node, < 0 the leaf ~code.  Only the upper w bound is used.
struct alignas(16) BvhNode
{
    float4 lo_l, hi_l, lo_r, hi_r;
};

constexpr int kStackDepth = 64;

struct Frame64
{
    double r[9]; // rows e1, e2, e3 (e3 = dir / |dir|)
};

struct Frame32
{
    float r[9];
};

// Conservative float pre-test of a leaf: false only if the query's (u, v) point lies outside the projected
// triangle by more than the rounding of every coordinate involved can explain, i.e. on the positive side of one
// edge and the negative side of another, each by more than its margin.  `delta` bounds the absolute error of any
// float (u, v) coordinate (the query's, rotated in float, and the vertices', rounded from FP64).  An edge function
// e = du*rv - dv*ru then errs by at most 3*delta*(|du| + |dv| + |ru| + |rv|); the margin takes 8*delta.  The exact
// Moller-Trumbore test decides every leaf that passes.
// Leaf data: 3 float4 per leaf, (u_a, v_a, u_b, v_b), (u_c, v_c, w_a, w_b), (w_c, 0, 0, 0): the triangle's corners
// in the ray frame, rounded to float.
constexpr int kLeafF4 = 3;

// m8 = 8 delta for may_hit and certain_leaf, from the query's largest |coordinate| qmax and the mesh's
// scene_scale (eps = 2^-24).  delta must bound (1) the error of every float (u, v, w) coordinate and (2) a quarter
// of the rounding of the float edge functions, 4 eps R with R the largest |query - corner| coordinate difference:
// then certain_leaf's error model (3 delta (|du| + |dv| + |ru| + |rv|) per edge function, 2 delta per depth, both
// doubled in the depth test) holds, and may_hit's threshold 8 delta leaves a factor above it.
// Rotated frame (the mesh intersector's hierarchy for any direction): a query coordinate is rounded to float and
// rotated by the float frame (rows within eps of the FP64 frame) in at most five rounded operations, so it errs by at
// most 7 eps sum_i |r_i| |p_i| <= 7 sqrt(3) eps qmax = 7.3e-7 qmax; a leaf corner is projected in FP64 and rounded
// once, within sqrt(3) eps scene_scale = 1.04e-7 scene_scale; R <= sqrt(3) (qmax + scene_scale), so 4 eps R <=
// 4.13e-7 (qmax + scene_scale).  delta = 8e-7 qmax + 4.2e-7 scene_scale covers both.
__device__ __forceinline__ float margin_rotated(float qmax, float scene_scale)
{
    return 8.0f * fmaf(8e-7f, qmax, 4.2e-7f * scene_scale);
}
// Permutation frame (the robust evaluator's (z, y, -x) for the -x ray): products by 0 and 1 and sums with zeros are
// exact, so a query coordinate only carries its rounding to float (eps qmax) and a corner its own (eps
// scene_scale); R <= qmax + scene_scale, so 4 eps R <= 2.4e-7 (qmax + scene_scale).  delta = 3e-7 (qmax +
// scene_scale) covers both.
__device__ __forceinline__ float margin_permuted(float qmax, float scene_scale)
{
    return 8.0f * 3e-7f * (qmax + scene_scale);
}

__device__ __forceinline__ bool may_hit(const float4* __restrict__ leaf_uv, int leaf, float u, float v, float m8)
{
    float4 const a = leaf_uv[kLeafF4 * leaf], b = leaf_uv[kLeafF4 * leaf + 1];
    float const pu[3] = {a.x, a.z, b.x}, pv[3] = {a.y, a.w, b.y};
    bool pos = false, neg = false;
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        int const k1 = (k + 1) % 3;
        float const du = pu[k1] - pu[k], dv = pv[k1] - pv[k], ru = u - pu[k], rv = v - pv[k];
        float const e = du * rv - dv * ru;
        float const m = m8 * (fabsf(du) + fabsf(dv) + fabsf(ru) + fabsf(rv));
        pos |= e > m;
        neg |= e < -m;
    }
    return !(pos && neg);
}

// The companion of may_hit that decides a leaf in float when it can: 1 or -1 (the ray certainly crosses the
// triangle, with that orientation), 0 (it certainly does not), 2 (undecided: run the exact test).  Inside: every
// edge function beyond its may_hit margin, all with one sign (that sign is the projected orientation, and the frame
// is right-handed, so it is the sign of the triangle normal along the ray).  In front or behind: the plane's depth
// at (u, v) minus the query's, (e1 dw_a + e2 dw_b + e0 dw_c) / E with E = e0 + e1 + e2, against the bound that the
// edge functions' errors (3 delta (|du| + |dv| + |ru| + |rv|) each, delta = m8 / 8) and the depths' (2 delta each)
// carry through that quotient, doubled.  delta bounds the error of the float coordinates and a quarter of the
// edge functions' rounding (margin_rotated, margin_permuted), and the exact test's own rounding is ~1e-16 of the
// coordinates, so a decided leaf gets the exact test's answer; only points within that margin of an edge, a vertex
// or the plane go to the exact test.
__device__ __forceinline__ int certain_leaf(const float4* __restrict__ leaf_uv, int leaf, float u, float v, float w,
                                            float m8)
{
    float4 const a = leaf_uv[kLeafF4 * leaf], b = leaf_uv[kLeafF4 * leaf + 1], c = leaf_uv[kLeafF4 * leaf + 2];
    float const pu[3] = {a.x, a.z, b.x}, pv[3] = {a.y, a.w, b.y};
    float const dw[3] = {b.z - w, b.w - w, c.x - w}; // depths of a, b, c relative to the query
    float e[3], err[3];
    bool pos = true, neg = true;
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        int const k1 = (k + 1) % 3;
        float const du = pu[k1] - pu[k], dv = pv[k1] - pv[k], ru = u - pu[k], rv = v - pv[k];
        float const sabs = fabsf(du) + fabsf(dv) + fabsf(ru) + fabsf(rv);
        e[k] = du * rv - dv * ru;
        err[k] = 0.375f * m8 * sabs;
        pos &= e[k] > m8 * sabs;
        neg &= e[k] < -m8 * sabs;
    }
    if (!(pos || neg))
        return 2;
    // e[k] is the weight of the vertex opposite edge k: e0 -> c, e1 -> a, e2 -> b
    float const E = e[0] + e[1] + e[2];
    float const errE = err[0] + err[1] + err[2];
    float const N = e[1] * dw[0] + e[2] * dw[1] + e[0] * dw[2];
    float const two_delta = 0.25f * m8;
    float const errN = err[1] * fabsf(dw[0]) + err[2] * fabsf(dw[1]) + err[0] * fabsf(dw[2]) +
                       two_delta * (fabsf(e[0]) + fabsf(e[1]) + fabsf(e[2]));
    float const aE = fabsf(E);
    if (!(aE > 2.f * errE))
        return 2;
    float const depth = N / E;
    float const bound = 2.f * (errN + fabsf(depth) * errE) / (aE - errE);
    if (depth > bound)
        return pos ? 1 : -1;
    if (depth < -bound)
        return 0;
    return 2;
}

// Walks the hierarchy for the query point (u, v) and depth w, calling emit(leaf) for every leaf whose box the ray
// {(u, v, w') : w' >= w} meets (widened by tol) and that passes may_hit.  Returns false if the stack of kStack
// pending subtrees overflowed (a hierarchy of depth d needs at most d - 1).
template <int kStack = kStackDepth, class Emit>
__device__ __forceinline__ bool hier_walk(const BvhNode* __restrict__ nodes, const float4* __restrict__ leaf_uv,
                                          float u, float v, float w, float tol, float m8, Emit&& emit)
{
    float const ulo = u + tol, uhi = u - tol, vlo = v + tol, vhi = v - tol, wq = w - tol;
    int stack[kStack];
    int sp = 0;
    int node = 0;
    while (true)
    {
        BvhNode const nd = nodes[node];
        int const lc = __float_as_int(nd.lo_l.w), rc = __float_as_int(nd.lo_r.w);
        bool const hl =
            nd.lo_l.x <= ulo && nd.hi_l.x >= uhi && nd.lo_l.y <= vlo && nd.hi_l.y >= vhi && nd.hi_l.z >= wq;
        bool const hr =
            nd.lo_r.x <= ulo && nd.hi_r.x >= uhi && nd.lo_r.y <= vlo && nd.hi_r.y >= vhi && nd.hi_r.z >= wq;
        int next = -1;
        if (hl)
        {
            if (lc >= 0)
                next = lc;
            else if (may_hit(leaf_uv, ~lc, u, v, m8))
                emit(~lc);
        }
        if (hr)
        {
            if (rc < 0)
            {
                if (may_hit(leaf_uv, ~rc, u, v, m8))
                    emit(~rc);
            }
            else if (next < 0)
                next = rc;
            else
            {
                if (sp == kStack)
                    return false;
                stack[sp++] = rc;
            }
        }
        if (next >= 0)
            node = next;
        else if (sp > 0)
            node = stack[--sp];
        else
            return true;
    }
}

// A cell grid (CellGrid, agwn_internal.cuh) as the kernels read it.
struct CellView
{
    const unsigned* offsets;
    const int* list;
    int gu, gv;
    float umin, vmin, umax, vmax, inv_u, inv_v;
    float tol_max;
};
inline CellView cell_view(const CellGrid& g)
{
    return CellView{static_cast<const unsigned*>(g.offsets.ptr), static_cast<const int*>(g.list.ptr), g.gu, g.gv,
                    g.umin, g.vmin, g.umax, g.vmax, g.inv_u, g.inv_v, g.tol_max};
}

// Cell column / row of a coordinate: monotone in x, so a point inside a widened box maps into the box's cells.
__device__ __forceinline__ int cell_of(float x, float lo, float inv, int g)
{
    int const i = int(floorf((x - lo) * inv));
    return i < 0 ? 0 : (i >= g ? g - 1 : i);
}

// The leaves listed in the cell of a query's (u, v) point that the walk's leaf conditions admit (the top of the
// leaf above the query's depth, may_hit), passed to emit; a query outside the grid's extent has none.  The caller
// takes the hierarchy walk instead when the query's tolerance exceeds g.tol_max.  Returns the list entries read.
template <class Emit>
__device__ __forceinline__ unsigned cell_candidates(CellView const& g, const float4* __restrict__ leaf_uv, float u,
                                                    float v, float w, float tol, float m8, Emit&& emit)
{
    if (!(u >= g.umin && u <= g.umax && v >= g.vmin && v <= g.vmax))
        return 0;
    int64_t const c = int64_t(cell_of(v, g.vmin, g.inv_v, g.gv)) * g.gu + cell_of(u, g.umin, g.inv_u, g.gu);
    unsigned const b = g.offsets[c], e = g.offsets[c + 1];
    float const wq = w - tol;
    for (unsigned j = b; j < e; ++j)
    {
        int const leaf = g.list[j];
        float4 const lb = leaf_uv[kLeafF4 * leaf + 1];
        float const wc = leaf_uv[kLeafF4 * leaf + 2].x;
        if (fmaxf(fmaxf(lb.z, lb.w), wc) >= wq && may_hit(leaf_uv, leaf, u, v, m8))
            emit(leaf);
    }
    return e - b;
}

// ---- exact tests of undecided leaves, a warp's worth at a time -----------------------------------------------
// The float decision (certain_leaf) leaves a few candidates per warp undecided, at different points of each lane's
// candidate loop, so testing them in place runs each exact test with one or two lanes active.  Instead a query
// keeps up to kUndecided of them; after its candidates, the warp appends every lane's to a queue in shared memory,
// and whenever 32 are queued each lane takes one and runs the exact test (for its owner's query, reloaded by
// index), adding the result to the owner's count.  The query's own float-decided sum is stored first, so the
// additions are atomic adds to it.
constexpr int kUndecided = 4;  // undecided leaves a query holds; any beyond are tested in place (rare)
constexpr unsigned kLeafQCap = 64; // > 31 left over + 32 appended per round

struct LeafQueue
{
    int* leaf;         // kLeafQCap entries of this warp
    long long* query;  // their queries' indices
    unsigned head = 0, tail = 0; // warp-uniform
};

// Runs the exact test exact(query, leaf) -> -1, 0 or 1 on the c (<= 32) oldest entries, one per lane.
template <class Exact>
__device__ __forceinline__ void leafq_flush(LeafQueue& lq, unsigned c, int lane, int32_t* __restrict__ counts,
                                            Exact&& exact)
{
    __syncwarp(); // the entries, and the owners' counts, are visible to the warp
    if (unsigned(lane) < c)
    {
        unsigned const s = (lq.head + unsigned(lane)) & (kLeafQCap - 1);
        long long const qi = lq.query[s];
        int const r = exact(qi, lq.leaf[s]);
        if (r)
            atomicAdd(counts + qi, r);
    }
    lq.head += c;
    __syncwarp(); // the slots are free again
}

// Appends each lane's nu undecided leaves und[0..nu) of query qi (every lane of the warp calls it, after storing
// its query's count) and tests full batches of 32.
template <class Exact>
__device__ __forceinline__ void leafq_push(LeafQueue& lq, int const (&und)[kUndecided], int nu, long long qi, int lane,
                                           int32_t* __restrict__ counts, Exact&& exact)
{
    unsigned const lt = (1u << lane) - 1u;
    int const most = __reduce_max_sync(0xffffffffu, nu);
#pragma unroll
    for (int j = 0; j < kUndecided; ++j)
    {
        if (j >= most)
            break;
        bool const has = j < nu;
        unsigned const m = __ballot_sync(0xffffffffu, has);
        if (has)
        {
            unsigned const s = (lq.tail + unsigned(__popc(m & lt))) & (kLeafQCap - 1);
            lq.leaf[s] = und[j];
            lq.query[s] = qi;
        }
        lq.tail += unsigned(__popc(m));
        if (lq.tail - lq.head >= 32)
            leafq_flush(lq, 32, lane, counts, exact);
    }
}

// Tests what is left in the queue (at the end of the kernel).
template <class Exact>
__device__ __forceinline__ void leafq_drain(LeafQueue& lq, int lane, int32_t* __restrict__ counts, Exact&& exact)
{
    while (lq.tail != lq.head)
        leafq_flush(lq, min(32u, lq.tail - lq.head), lane, counts, exact);
}

// Integer-term statistics (AGWN_OPT_TIMING): one warp's sums added to counters[4..7] = queries, cell-list entries
// read, candidate leaves decided, exact tests.
__device__ __forceinline__ void integer_stats(long long* counters, long long queries, long long entries,
                                              long long leaves, long long exact_tests)
{
    long long v[4] = {queries, entries, leaves, exact_tests};
#pragma unroll
    for (int k = 0; k < 4; ++k)
    {
        for (int o = 16; o > 0; o >>= 1)
            v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    }
    if ((threadIdx.x & 31) == 0)
    {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (v[k])
                atomicAdd(reinterpret_cast<unsigned long long*>(counters + 4 + k), static_cast<unsigned long long>(v[k]));
    }
}

// Builds the cell grid of hierarchy h (lbvh.cu); leaves g invalid when a grid does not apply.
int build_cells(Context& ctx, const Hier& h, float scene_scale, CellGrid& g);

// Orthonormal frame whose third row is dir / |dir|.
Frame64 ray_frame(const double* dir);

// Builds the hierarchy of n triangles (device array of 9 scalars each) in the frame of dir into `out` (its buffers
// are reused when large enough; the stream is synchronised first).  If `order_out` is not null it receives, for
// every leaf, the index of its triangle in the input.
template <class T>
int build_hier(Context& ctx, const T* tri_in, int64_t n_tri, const double* dir, Hier& out, unsigned* order_out);
} // namespace agwn
