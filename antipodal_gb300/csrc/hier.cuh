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
__device__ __forceinline__ bool may_hit(const float4* __restrict__ leaf_uv, int leaf, float u, float v, float m8)
{
    float4 const a = leaf_uv[2 * leaf], b = leaf_uv[2 * leaf + 1];
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

// Orthonormal frame whose third row is dir / |dir|.
Frame64 ray_frame(const double* dir);

// Builds the hierarchy of n triangles (device array of 9 scalars each) in the frame of dir into `out` (its buffers
// are reused when large enough; the stream is synchronised first).  If `order_out` is not null it receives, for
// every leaf, the index of its triangle in the input.
template <class T>
int build_hier(Context& ctx, const T* tri_in, int64_t n_tri, const double* dir, Hier& out, unsigned* order_out);
} // namespace agwn
