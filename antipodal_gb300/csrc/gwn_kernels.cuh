// Declarations shared by the translation units of libantipodal_gb300.
#pragma once

#include "agwn_internal.cuh"

namespace agwn
{
// Device state of a CudaIntersector: its triangles, copied.  The hierarchy that accelerates the integer term is
// built per ray direction and cached in the context that queries it (see lbvh.cu).
struct Bvh
{
    int device = 0;
    int scalar_bytes = 8;                // 8: double geometry, 4: float geometry
    int64_t n_tri = 0;
    void* tri = nullptr;                 // n_tri x 9 scalars (a, b, c) in input order
    double scene_scale = 1.0;            // max |coordinate| of the geometry, for the traversal tolerance
    unsigned long long generation = 0;   // unique per intersector, keys the contexts' hierarchy caches
    mutable int32_t depth = 0;           // depth of the most recently built hierarchy (0 before any query)
};

// Fractional term of the mesh GWN for `n` device-resident queries; adds `counts[i]` (if non-null).
template <class T>
int fractional_run(Context& ctx, const T* d_pos, int64_t n, T* d_out, const int32_t* d_counts, const T* x0_host,
                   const T* d_seg_raw, int64_t n_seg);

// The robust evaluator's fractional term under the exact_float policy in mixed precision (frac.cu): the mesh
// functions' mixed kernel along the -x ray over the raw segments d_raw (7 doubles each, the evaluator's input
// orientation), with the robust FP64 rule for the pairs it turns down (rseg: the evaluator's RSeg<double> array,
// same order).  out = fractional term + counts (counts may be null).
int frac_mixed_robust_pf(Context& ctx, const double* d_pos, int64_t n, double* d_out, const int32_t* d_counts,
                         const double* d_raw, int64_t n_seg, const void* rseg);
// The same with the counts made chunk by chunk: the queries run in 8 chunks whose kernels alternate between the
// context's stream and a second compute stream (count(user, ctx, chunk queries, m, chunk counts) launches a chunk's
// counts on ctx.stream, then the chunk's fractional kernel adds them), so that one chunk's counts overlap another's
// fractional term.  d_counts: n ints of scratch.
using ChunkCounts = int (*)(void* user, Context& ctx, const double* d_pos, int64_t m, int32_t* d_counts);
int frac_mixed_robust_pf_chunked(Context& ctx, const double* d_pos, int64_t n, double* d_out, int32_t* d_counts,
                                 const double* d_raw, int64_t n_seg, const void* rseg, ChunkCounts count,
                                 void* user);

// Integer term over a BVH for `n` device-resident queries.
template <class T>
int integer_run(Context& ctx, const Bvh& bvh, const T* d_pos, int64_t n, int32_t* d_counts, const T* dir_host);
// The hierarchy along dir_host and its cell grid (when enabled), built on ctx.stream unless cached.
template <class T>
int integer_prepare(Context& ctx, const Bvh& bvh, const T* dir_host);

// Spatial order of the queries for the mixed kernels (order.cu).  For n >= kOrderMinQueries device-resident
// queries whose order is incoherent across the direction dir (3 doubles, host), *perm receives a permutation (device
// scratch S_ORDER0, valid until the next call) that sorts them along a 2D Morton curve across dir; otherwise (a
// coherent order, fewer queries, or certification off) null.  With cacheable (the caller's own device array) the
// decision is cached per (d_pos, n, dir); staged copies of host arrays are sampled on every call.
constexpr int64_t kOrderMinQueries = int64_t(1) << 20;
int query_order(Context& ctx, const double* d_pos, int64_t n, const double* dir, bool cacheable,
                const int32_t** perm);
// d_sorted[i] = d_pos[perm[i]] (three doubles each)
int gather_queries(Context& ctx, const double* d_pos, const int32_t* perm, int64_t n, double* d_sorted);
// d_out[perm[i]] = d_sorted[i] (double and int32_t)
template <class T>
int scatter_back(Context& ctx, const T* d_sorted, const int32_t* perm, int64_t n, T* d_out);
} // namespace agwn

struct agwn_bvh : agwn::Bvh
{
};
