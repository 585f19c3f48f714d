/*
 * antipodal_gb300.h -- C ABI of the GB300 batch generalized-winding-number (GWN) library.
 *
 * One shared library, libantipodal_gb300.so, built for sm_103a.  Every entry point takes plain pointers and
 * sizes and returns an int status (AGWN_OK == 0).  A failing call leaves a human-readable reason in
 * agwn_last_error_message() (per host thread).  The header-only C++20 front end
 * (include/antipodal/cuda/gwn_cuda.hh) turns a non-zero status into std::runtime_error.
 *
 * Memory.  Every array argument may be host memory (pageable or pinned) or device memory; the library asks the
 * CUDA runtime which one it is.  A call whose inputs and outputs are all device memory is asynchronous on the
 * context's stream; a call that reads or writes any host array returns only after the host outputs are written.
 * Device-side error flags (exhausted traversal stack, a bounded wait that ran out) are reported by the call
 * that synchronises: the synchronous call itself, or agwn_context_synchronize().
 *
 * Layouts are the antipodal library's own value types, so spans of them can be passed straight through:
 *   vec3<T>              3 x T                      (src/antipodal/math/common.hh:32-45)
 *   weighted_segment3<T> pos0, pos1, weight = 7 x T (src/antipodal/math/common.hh:50-65)
 *   triangle indices     3 x int32 per triangle     (NaiveIntersector::indices, intersector/intersector.hh:59)
 * Paths cited in this header are relative to the antipodal project root.
 *
 * Threading: a context is used by one host thread at a time (the reference's PoolDispatcher likewise runs one
 * job at a time, dispatcher/dispatcher_threadpool.hh:22-23).  Geometry handles (agwn_bvh, agwn_robust) are
 * read-only after creation and may be shared by contexts on the same device.
 */
#ifndef ANTIPODAL_GB300_H
#define ANTIPODAL_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AGWN_ABI_VERSION 2

/* ---- status ---------------------------------------------------------------------------------------------- */
enum agwn_status
{
    AGWN_OK = 0,
    AGWN_ERR_INVALID = 1,     /* bad argument: null pointer, negative size, unknown enum value            */
    AGWN_ERR_CUDA = 2,        /* a CUDA runtime call failed                                               */
    AGWN_ERR_NOMEM = 3,       /* a device allocation failed                                               */
    AGWN_ERR_STACK = 4,       /* a BVH traversal stack was exhausted (degenerate hierarchy)               */
    AGWN_ERR_TIMEOUT = 5,     /* a bounded device-side wait ran out; the result is not valid              */
    AGWN_ERR_UNSUPPORTED = 6, /* combination not provided (e.g. the mixed fractional mode for float input) */
    AGWN_ERR_NO_DEVICE = 7    /* no CUDA device, or the device ordinal does not exist                      */
};

const char* agwn_status_string(int status);
/* Detail of the last failing call on this host thread ("" if none). */
const char* agwn_last_error_message(void);
int agwn_abi_version(void);

/* ---- context: device, stream, scratch arena, options ----------------------------------------------------- */
typedef struct agwn_context agwn_context;

/* stream: a cudaStream_t to run on (cudaStreamLegacy, i.e. (void*)1, for the legacy default stream), or NULL to
   let the context create its own non-blocking stream. */
int agwn_context_create(int device, void* stream, agwn_context** out);
int agwn_context_destroy(agwn_context* ctx);
/* Waits for all work of the context and reports device-side error flags raised since the last check. */
int agwn_context_synchronize(agwn_context* ctx);

enum agwn_option
{
    /* Fractional-term precision for double inputs: AGWN_FRAC_EXACT (default) or AGWN_FRAC_MIXED.  The mixed mode
       runs the exact kernels for calls below AGWN_OPT_MIXED_MIN_PAIRS and for boundaries of 2^24 segments or
       more. */
    AGWN_OPT_FRAC_MODE = 0,
    /* Mixed mode: a (query, segment) pair whose nearer endpoint is closer than tau * segment length is
       evaluated in FP64 with the reference arithmetic.  Default 4. */
    AGWN_OPT_MIXED_TAU = 1,
    /* Queries owned by each thread in the fractional kernels (1, 2, 4 or 8; the mixed kernel packs them in pairs
       and runs 1 as 2).  Default 2. */
    AGWN_OPT_QUERIES_PER_THREAD = 2,
    /* Threads per block of the fractional kernels (64..256, a multiple of 32), or 0 (default): 128, and 256 for the
       mixed kernel when the boundary spans more than one segment tile (more queries share each staged tile). */
    AGWN_OPT_FRAC_BLOCK = 3,
    /* Record CUDA events around the library's kernels and accumulate their device time (0/1).  Default 0. */
    AGWN_OPT_TIMING = 4,
    /* Segments per shared-memory tile of the fractional kernels (32..2048).  Default 512. */
    AGWN_OPT_SEG_TILE = 5,
    /* Mixed mode: a pair whose first-order FP32 error bound exceeds this many radians is evaluated in FP64.
       Default 6e-8. */
    AGWN_OPT_MIXED_TERM_ERR = 6,
    /* Robust evaluator's fractional term: AGWN_ROBUST_EXACT (default, the reference's FP64 arithmetic) or
       AGWN_ROBUST_MIXED.  int64_grid: FP32 pairs on the exact integer differences under a first-order error
       estimate (AGWN_OPT_ROBUST_TERM_ERR), the others -- num == 0 branches, ill-conditioned or large differences --
       in FP64.  exact_float with double queries: the mesh functions' mixed kernel along -x (AGWN_OPT_MIXED_TERM_ERR)
       with the evaluator's FP64 rule, exact branches included, for the pairs it turns down.  Counts unchanged;
       int128_grid and the multi-mesh batch's exact_float meshes stay exact. */
    AGWN_OPT_ROBUST_MODE = 7,
    /* Robust mixed mode: the per-pair estimate above which a pair is evaluated in FP64, radians.  Default 1e-7. */
    AGWN_OPT_ROBUST_TERM_ERR = 8,
    /* Parametric integrator arithmetic: AGWN_PARAM_EXACT (default, FP64 with the reference's operation order, bit
       for bit) or AGWN_PARAM_MIXED (double-float on the FP32 pipe, ~44 significant bits; the same tree rule,
       tolerances and summation order, with the integrand and the curve in algebraically equal forms of fewer
       operations).  Mixed values agree with FP64 to ~1e-13 on typical pairs and to a few 1e-8 absolute where
       leaves are forced at max_depth near a curve, where FP64 is itself only that accurate. */
    AGWN_OPT_PARAM_MODE = 9,
    /* Integer term of the mesh functions (intersector of more than one triangle): 1 (default) looks up each ray's
       candidate triangles in a uniform grid over the plane across the ray direction, built once per (intersector,
       direction) and cached with the hierarchy; 0 walks the hierarchy for every ray.  Counts are the same. */
    AGWN_OPT_INTEGER_CELLS = 10,
    /* Mixed modes (mesh, and the robust evaluator's exact_float): below this many (query, segment) pairs in one
       call, or on a boundary of fewer than 32 segments, the exact FP64 kernels run instead, which are the faster
       ones there (the mixed form's boundary preparation costs more than the FP64 pairs it saves, and over long
       segments most pairs fall within the near distance that sends them to FP64).  Default 2^14; 0 always runs
       the mixed form. */
    AGWN_OPT_MIXED_MIN_PAIRS = 11,
    /* Mixed kernel: 1 (default) evaluates the boundary groups that a warp's queries certify (every pair far enough
       across the ray for its error bound to pass and its angle to lie in the first octant) without the per-pair
       bound and octant unfolding; 0 takes the per-pair path everywhere.  The results are the same bit for bit. */
    AGWN_OPT_MIXED_CERTIFY = 12
};
enum agwn_param_mode
{
    AGWN_PARAM_EXACT = 0,
    AGWN_PARAM_MIXED = 1
};
enum agwn_robust_mode
{
    AGWN_ROBUST_EXACT = 0,
    AGWN_ROBUST_MIXED = 1
};
enum agwn_frac_mode
{
    AGWN_FRAC_EXACT = 0, /* the reference's arithmetic in the input precision, unfused (plain)             */
    AGWN_FRAC_MIXED = 1  /* FP32 pairs with TwoSum accumulation; FP64 for near / branch-cut pairs          */
};
int agwn_context_set_option(agwn_context* ctx, int option, double value);
int agwn_context_get_option(agwn_context* ctx, int option, double* value);

enum agwn_kernel_class
{
    AGWN_K_FRACTIONAL = 0, /* fractional (boundary) kernels                        */
    AGWN_K_INTEGER = 1,    /* integer-term traversal kernels                       */
    AGWN_K_ROBUST = 2,     /* robust evaluator kernels                             */
    AGWN_K_PARAMETRIC = 3, /* parametric GK15 kernels                              */
    AGWN_K_OTHER = 4,      /* preparation, build and copy kernels                  */
    AGWN_K_COUNT = 5
};
typedef struct agwn_stats
{
    double kernel_ms[AGWN_K_COUNT];   /* device time between the events around each launch (AGWN_OPT_TIMING) */
    int64_t launches[AGWN_K_COUNT];   /* launches of the library's kernels, by class (always counted)        */
    int64_t fp64_pairs;               /* mixed mode: (query, segment) pairs evaluated in FP64 (when timing)  */
    int64_t pairs;                    /* mixed mode: all (query, segment) pairs evaluated (when timing)      */
    /* integer term through the cell grid (mesh counts and robust counts), when timing: */
    int64_t int_queries;              /* queries                                                              */
    int64_t int_cell_entries;         /* cell-list entries read (each a leaf index and the leaf's corners)     */
    int64_t int_leaves;               /* candidate leaves decided (in float, or by the exact test)             */
    int64_t int_exact_tests;          /* leaves the float decision left to the exact test                      */
    /* the Bezier-patch intersector, when timing: */
    int64_t patch_pairs;              /* (query, patch) pairs past the box test                                */
    int64_t patch_cells;              /* parameter cells whose control net was blossomed and tested            */
    int64_t patch_pieces;             /* boundary-cubic pieces blossomed and tested for the winding numbers    */
    int64_t patch_fp64_pairs;         /* decisions float could not make, taken in FP64 (a cell's winding or   
                                         a cell's subtree)                                                     */
    int64_t certified_pairs;          /* mixed mode: pairs in boundary groups the warp certified (when timing;
                                         counted over whole warps, padding lanes of the last query tile too)    */
} agwn_stats;
/* Reads (synchronising the stream first) and optionally resets the accumulated statistics. */
int agwn_context_get_stats(agwn_context* ctx, agwn_stats* out, int reset);

/* ---- mesh GWN: fractional term ----------------------------------------------------------------------------
 * Replaces eval_gwnr_mesh_batch_fractional (src/antipodal/gwn_mesh.hh:67-83): for each query p,
 * sum over boundary segments of weight * signed_spherical_tri_area_half_unorm(-x0, pos0 - p, pos1 - p),
 * divided by 2 pi.  x0 is 3 values in host memory; it is not validated (the reference does not either). */
int agwn_mesh_batch_fractional_f64(agwn_context* ctx, const double* positions, int64_t n, double* out,
                                   const double* x0, const double* boundary, int64_t n_segments);
int agwn_mesh_batch_fractional_f32(agwn_context* ctx, const float* positions, int64_t n, float* out,
                                   const float* x0, const float* boundary, int64_t n_segments);

/* ---- mesh GWN: integer term over a device LBVH -------------------------------------------------------------
 * A CudaIntersector's device state: the triangles, copied, and a linear BVH built on the device (Morton codes,
 * radix sort, Karras hierarchy, bottom-up boxes).  The counting rule is NaiveIntersector's Moller-Trumbore
 * (src/antipodal/intersector/intersector.hh:61-100) in the input precision with unfused arithmetic, so counts
 * match it bit for bit, including its double count of a ray through a shared edge. */
typedef struct agwn_bvh agwn_bvh;
int agwn_bvh_create_f64(agwn_context* ctx, const double* vertices, int64_t n_vertices, const int32_t* indices,
                        int64_t n_indices, agwn_bvh** out);
int agwn_bvh_create_f32(agwn_context* ctx, const float* vertices, int64_t n_vertices, const int32_t* indices,
                        int64_t n_indices, agwn_bvh** out);
int agwn_bvh_destroy(agwn_bvh* bvh);
/* Hierarchy depth, nodes, triangles (for tests and roofline accounting). */
int agwn_bvh_info(const agwn_bvh* bvh, int64_t* n_triangles, int32_t* depth);

/* Replaces eval_gwnr_mesh_batch_integer (src/antipodal/gwn_mesh.hh:127-143) and
 * NaiveIntersector::signed_intersection_count: out_counts[i] = signed crossings of the ray (p_i, dir). */
int agwn_mesh_batch_integer_f64(agwn_context* ctx, const agwn_bvh* bvh, const double* positions, int64_t n,
                                int32_t* out_counts, const double* dir);
int agwn_mesh_batch_integer_f32(agwn_context* ctx, const agwn_bvh* bvh, const float* positions, int64_t n,
                                int32_t* out_counts, const float* dir);

/* Replaces eval_gwnr_mesh_batch (src/antipodal/gwn_mesh.hh:201-219): fractional + integer, fused per query.
 * bvh may be NULL for a closed-free evaluation (integer term 0); boundary may be empty (n_segments 0). */
int agwn_mesh_batch_f64(agwn_context* ctx, const agwn_bvh* bvh, const double* positions, int64_t n, double* out,
                        const double* x0, const double* boundary, int64_t n_segments);
int agwn_mesh_batch_f32(agwn_context* ctx, const agwn_bvh* bvh, const float* positions, int64_t n, float* out,
                        const float* x0, const float* boundary, int64_t n_segments);

/* Brute-force integer term (every query against every triangle; no hierarchy).  Same counting rule as above.
 * For small meshes and as a cross-check of the traversal. */
int agwn_mesh_batch_integer_bruteforce_f64(agwn_context* ctx, const double* vertices, int64_t n_vertices,
                                           const int32_t* indices, int64_t n_indices, const double* positions,
                                           int64_t n, int32_t* out_counts, const double* dir);
/* The same scan, also reporting ties: out_ties[i] = how many of the hits counted for query i lie exactly on a
 * triangle's edge or vertex (u = 0, v = 0 or u + v = 1 in Moller-Trumbore's arithmetic) or at the query itself
 * (t = 0).  NaiveIntersector (intersector.hh:55-100) counts a crossing through a shared edge once per triangle, so
 * these are the queries whose counts carry its double count (test/test_intersector.cc:85-89). */
int agwn_mesh_batch_integer_ties_f64(agwn_context* ctx, const double* vertices, int64_t n_vertices,
                                     const int32_t* indices, int64_t n_indices, const double* positions, int64_t n,
                                     int32_t* out_counts, int32_t* out_ties, const double* dir);

/* ---- robust mesh GWN ---------------------------------------------------------------------------------------
 * Replaces RobustMeshGwn<T, Precision> (src/antipodal/gwn_mesh_robust.hh:170-424) and eval_gwnr_mesh_batch_robust
 * (:441-456): fractional and integer terms along the fixed -x ray, both decided by one exact predicate
 * (src/antipodal/math/robust_predicates.hh).  The evaluator owns device copies of the quantised (or, for
 * exact_float, double) triangles and swapped boundary, and a hierarchy that replaces Embree's traversal; the
 * caller's arrays need not outlive it.  Counts equal the reference's bit for bit; the fractional term matches it
 * up to the last bits of atan2.  Precision policy: */
enum agwn_robust_policy
{
    AGWN_ROBUST_INT64_GRID = 0,  /* 20-bit grid, 64-bit determinants (the reference's default for float)     */
    AGWN_ROBUST_INT128_GRID = 1, /* 50-bit grid, 128-bit determinants                                        */
    AGWN_ROBUST_EXACT_FLOAT = 2  /* double coordinates, exact determinant signs (the default for double)     */
};
typedef struct agwn_robust agwn_robust;
int agwn_robust_create_f64(agwn_context* ctx, int policy, const double* vertices, int64_t n_vertices,
                           const int32_t* indices, int64_t n_indices, const double* boundary, int64_t n_segments,
                           agwn_robust** out);
int agwn_robust_create_f32(agwn_context* ctx, int policy, const float* vertices, int64_t n_vertices,
                           const int32_t* indices, int64_t n_indices, const float* boundary, int64_t n_segments,
                           agwn_robust** out);
int agwn_robust_destroy(agwn_robust* robust);
/* Quantisation centre (3 doubles) and scale, and the hierarchy depth. */
int agwn_robust_info(const agwn_robust* robust, double* center, double* scale, int32_t* depth);
/* out_gwn[i] = RobustMeshGwn::eval(p_i); optional out_counts[i] = signed_intersection_count(p_i) and
 * out_frac[i] = fractional(p_i) (either may be NULL). */
int agwn_robust_eval_f64(agwn_context* ctx, const agwn_robust* robust, const double* positions, int64_t n,
                         double* out_gwn, int32_t* out_counts, double* out_frac);
int agwn_robust_eval_f32(agwn_context* ctx, const agwn_robust* robust, const float* positions, int64_t n,
                         float* out_gwn, int32_t* out_counts, float* out_frac);

/* RobustMeshGwn::eval over an axis-aligned grid, without query arrays or a hierarchy walk.  Cell (ix, iy, iz),
 * stored at ((iz * ny) + iy) * nx + ix, is the point (T(start[0] + ix * spacing[0]), T(start[1] + iy * spacing[1]),
 * T(start[2] + iz * spacing[2])), each coordinate computed in double without fused multiply-add and rounded to the
 * evaluator's scalar type; spacing > 0.  The integer term is rasterized per (y, z) column with the evaluator's exact
 * -x crossing rule and prefix-summed along x, so every output equals agwn_robust_eval_* at that point (counts bit
 * for bit).  The reference's OpenGL grid evaluator (gwn_mesh_opengl.hh:519) does the same in float; this one is
 * exact.  out_counts / out_frac may be NULL. */
int agwn_robust_eval_grid_f64(agwn_context* ctx, const agwn_robust* robust, const double* start, const double* spacing,
                              int64_t nx, int64_t ny, int64_t nz, double* out_gwn, int32_t* out_counts,
                              double* out_frac);
int agwn_robust_eval_grid_f32(agwn_context* ctx, const agwn_robust* robust, const double* start, const double* spacing,
                              int64_t nx, int64_t ny, int64_t nz, float* out_gwn, int32_t* out_counts, float* out_frac);

/* ---- open boundary of a mesh ------------------------------------------------------------------------------
 * Replaces build_boundary_segments (src/antipodal/math/common.hh:123-174) on the device: every triangle edge
 * u -> v adds +1 (u < v) or -1 to its undirected edge {min, max}; edges with a non-zero net count become
 * weighted_segment3 rows (7 scalars) directed lo -> hi for a positive count and hi -> lo otherwise, weight |count|.
 * The reference emits in hash-map order; these rows come in ascending (lo, hi) order.  *n_segments receives the
 * number of rows; min(*n_segments, capacity) of them are written to out (host or device, may be NULL to query
 * the count).  An index outside [0, n_vertices) is rejected with AGWN_ERR_INVALID. */
int agwn_build_boundary_segments_f64(agwn_context* ctx, const double* vertices, int64_t n_vertices,
                                     const int32_t* indices, int64_t n_indices, double* out, int64_t capacity,
                                     int64_t* n_segments);
int agwn_build_boundary_segments_f32(agwn_context* ctx, const float* vertices, int64_t n_vertices,
                                     const int32_t* indices, int64_t n_indices, float* out, int64_t capacity,
                                     int64_t* n_segments);

/* ---- many robust meshes in one persistent launch ----------------------------------------------------------
 * No single reference counterpart: the result equals calling eval_gwnr_mesh_batch_robust
 * (src/antipodal/gwn_mesh_robust.hh:441-456) once per mesh -- out_i[j] = meshes[i].eval(positions_i[j]) --
 * bit for bit, for meshes and query arrays of any (uneven) sizes.  All meshes share the scalar type and the
 * precision policy; positions[i] (n_queries[i] * 3 scalars), out[i] and the optional counts[i] (integer term)
 * are device memory and, like the meshes, must outlive the plan.  The plan holds the device work list (ranges of
 * one mesh's queries, longest first) and the launch configuration.
 *   agwn_batch_tune: times every configuration {block 128/256, queries per thread 1/2, segment tile 256/512/1024,
 *     traversal stack 32/64 (32 only where every hierarchy is shallower)} on a sample of every mesh's queries,
 *     `repeats` times each, and keeps the fastest.
 *   agwn_batch_run: one persistent launch over the whole work list on the context's stream; with use_graph the
 *     queue reset and the launch are captured into a CUDA graph on the first run (and again after the
 *     configuration changes) and replayed afterwards.
 *   agwn_batch_info: config = {block, queries per thread, segment tile, stack}; *n_candidates in: capacity of
 *     tune_ms, out: number of candidates; tune_ms: each candidate's sample time (-1 = did not fit / not run). */
typedef struct agwn_batch agwn_batch;
int agwn_batch_create(agwn_context* ctx, const agwn_robust* const* meshes, int32_t n_meshes,
                      const void* const* positions, const int64_t* n_queries, void* const* out,
                      int32_t* const* counts, agwn_batch** plan);
int agwn_batch_destroy(agwn_batch* plan);
int agwn_batch_tune(agwn_context* ctx, agwn_batch* plan, int32_t repeats);
int agwn_batch_set_config(agwn_batch* plan, const int32_t* config);
int agwn_batch_info(const agwn_batch* plan, int32_t* config, int32_t* n_candidates, double* tune_ms,
                    int64_t* n_items, int64_t* total_queries, double* total_pairs);
int agwn_batch_run(agwn_context* ctx, agwn_batch* plan, int32_t use_graph);

/* ---- parametric surfaces ----------------------------------------------------------------------------------
 * Replaces eval_gwnr_parametric_batch_fractional (src/antipodal/gwn_parametric.hh:168-186) with the default
 * IntegratorGK15 (src/antipodal/math/integrate_gk15.hh:63-290) and integrate_config {min_depth, max_depth, tol}
 * (src/antipodal/math/integrate.hh:11-22), for boundaries made of cubic Bezier curves: `curves` holds 12 doubles
 * per curve (control points c0..c3, xyz each), in the order for_each_boundary would visit them.  The reference
 * takes the curve as a functor; the C ABI fixes it to this one curve type (the only one the reference's tests
 * integrate besides straight lines, which are cubics with collinear control points).
 * out[i] = (sum over curves of the adaptive GK15 integral of w - d_eta on [0, 1]) / (4 pi), bit-identical to the
 * reference's double evaluation.  max_depth <= 24.
 * start_depth (nullable, n * n_curves bytes, row-major [query][curve]): panels shallower than start_depth are split
 * without being evaluated -- the hook for a proposed refinement depth (agwn_param_propose_depth); NULL = the plain
 * integrator.  pair_stats (nullable, n * n_curves uint32): accepted leaves | shallowest leaf depth << 16 | deepest
 * leaf depth << 24.  nodes_per_query (nullable, n int32): panels evaluated for each query. */
int agwn_param_batch_fractional_bezier3_f64(agwn_context* ctx, const double* positions, int64_t n, double* out,
                                            const double* x0, const double* curves, int64_t n_curves, int min_depth,
                                            int max_depth, double tol, const uint8_t* start_depth,
                                            uint32_t* pair_stats, int32_t* nodes_per_query);

/* ---- learned GK15 depth proposal ----------------------------------------------------------------------------
 * No counterpart in the reference.  A 12 -> 64 -> 64 -> 16 MLP (ReLU; BF16 weights and activations on the
 * tensor cores, FP32 accumulation, FP32 master weights) predicts, for each (query, curve) pair, the shallowest
 * depth at which the plain integrator accepts a panel (the "label": bits 16..23 of pair_stats).  Its proposal is
 * passed to agwn_param_batch_fractional_bezier3_f64 as start_depth; every evaluated panel is still accepted or
 * split by the plain error test, and wherever the proposal does not exceed the label the result is bit-identical
 * to the plain integrator's.
 * Parameter blob (agwn_mlp_param_count() floats): W1[64][16] (input columns 12..15 unused, kept 0), b1[64],
 * W2[64][64], b2[64], W3[16][64], b3[16]; each W is [out][in]. */
typedef struct agwn_mlp agwn_mlp;
int agwn_mlp_param_count(void);
int agwn_mlp_create(agwn_context* ctx, uint64_t seed, agwn_mlp** out); /* He-uniform weights, zero biases */
int agwn_mlp_destroy(agwn_mlp* mlp);
int agwn_mlp_set_params(agwn_context* ctx, agwn_mlp* mlp, const float* params); /* host blob; resets Adam */
int agwn_mlp_get_params(agwn_context* ctx, const agwn_mlp* mlp, float* params);  /* host blob */
/* The 12 features of every (query, curve) pair, row-major [n * n_curves][12] floats (host or device). */
int agwn_param_features_bezier3_f64(agwn_context* ctx, const double* positions, int64_t n, const double* x0,
                                    const double* curves, int64_t n_curves, double tol, float* features);
/* Mean softmax cross-entropy over the first n_classes logits and its gradient (agwn_mlp_param_count() floats,
 * host) on n labelled feature rows, computed by the training kernels. */
int agwn_mlp_loss_grad(agwn_context* ctx, const agwn_mlp* mlp, const float* features, const uint8_t* labels,
                       int64_t n, int n_classes, float* grads, double* loss);
/* `steps` Adam steps (lr, beta1 0.9, beta2 0.999) on mini-batches of `batch` rows (a multiple of 128) drawn from
 * the n rows by a hash of (seed, step, row).  loss_per_step (nullable, host): each step's mean loss. */
int agwn_mlp_train(agwn_context* ctx, agwn_mlp* mlp, const float* features, const uint8_t* labels, int64_t n,
                   int n_classes, int steps, int batch, float lr, uint64_t seed, float* loss_per_step);
/* Proposed start depth of every (query, curve) pair ([n][n_curves] bytes): the largest s whose predicted
 * probability of a shallower label, P(label < s), is at most alpha, raised to min_depth and capped at max_depth.
 * logits (nullable): [n * n_curves][16] floats. */
int agwn_param_propose_depth_bezier3_f64(agwn_context* ctx, const agwn_mlp* mlp, const double* positions, int64_t n,
                                         const double* x0, const double* curves, int64_t n_curves, int n_classes,
                                         int min_depth, int max_depth, double tol, float alpha,
                                         uint8_t* start_depth, float* logits);

/* The per-panel network of the double-float integrator (AGWN_PARAM_MIXED): before a panel below max_depth is
 * evaluated, the warp runs `mlp` (2 classes: split, accept) on its lanes' panels -- features of the panel's piece
 * of the curve -- and splits without evaluating those whose predicted chance of acceptance is below beta.  Every
 * evaluated panel is still accepted or split by the plain error test.  NULL turns it off.  The context keeps the
 * pointer: the network must outlive its use. */
int agwn_param_set_panel_network(agwn_context* ctx, const agwn_mlp* mlp, float beta);
/* Training data for it: runs the integrator (in the context's arithmetic) and logs every evaluated panel below
 * max_depth as 2 words, the pair's index (query * n_curves + curve, below 2^32) and
 * (depth << 25) | (j << 1) | accepted.  *n_entries = panels logged; min(*n_entries, capacity) are written. */
int agwn_param_panel_log_bezier3_f64(agwn_context* ctx, const double* positions, int64_t n, const double* x0,
                                     const double* curves, int64_t n_curves, int min_depth, int max_depth, double tol,
                                     uint32_t* log, int64_t capacity, int64_t* n_entries);
/* The 12 features of logged panels ([n_entries][12] floats) and their labels (accepted, nullable). */
int agwn_param_panel_features_bezier3_f64(agwn_context* ctx, const double* positions, int64_t n, const double* x0,
                                          const double* curves, int64_t n_curves, double tol, const uint32_t* log,
                                          int64_t n_entries, float* features, uint8_t* labels);
/* ---- parametric integer term: an Intersector over bicubic Bezier patches ---------------------------------------
 * eval_gwnr_parametric_batch_integer and eval_gwnr_parametric_batch (src/antipodal/gwn_parametric.hh:204-284)
 * forward the integer term to an Intersector; the reference ships none for parametric surfaces.  This one counts,
 * for the ray p + lambda x0 (lambda >= 0), every crossing with a patch S(u, v) = sum B_i(v) B_j(u) P[i][j] by
 * sign(N . x0), N = S_u x S_v: the mesh intersector's rule, and the orientation under which boundary curves that
 * run counter-clockwise in (u, v) make fractional + integer the winding number.  The count over a parameter cell
 * that lies in front of the query is the topological degree of the patch's projection at the ray: the winding
 * number of the cell boundary's image (4 cubics) about it.  Cells are split while their depth range holds 0 and
 * their control box holds the ray; every box test keeps a margin above its rounding (float first, FP64 for the
 * cells whose decision float cannot make), so the count is exact for the exact patch except in the degenerate
 * cases: the ray within 2^-42 of the coordinates' scale of a cell boundary's image, or the query that close to the
 * surface.
 * control_points: n_patches x 4 x 4 x 3 doubles, P[patch][i = v index][j = u index][xyz] (host or device); the
 * patches are copied to the device. */
typedef struct agwn_patches agwn_patches;
int agwn_patches_create_f64(agwn_context* ctx, const double* control_points, int64_t n_patches, agwn_patches** out);
int agwn_patches_destroy(agwn_patches* patches);
/* out_counts[i] = the signed crossing count of query i along x0 (eval_gwnr_parametric_batch_integer). */
int agwn_param_batch_integer_bezier3x3_f64(agwn_context* ctx, agwn_patches* patches, const double* positions,
                                           int64_t n, int32_t* out_counts, const double* x0);
/* The same counts, and out_degenerate[i] = how many of query i's decisions were degenerate (decided by a fixed
 * rule: a cell's winding taken as the chords give it, a cell on the surface counted when its mean depth is >= 0). */
int agwn_param_batch_integer_degenerate_bezier3x3_f64(agwn_context* ctx, agwn_patches* patches,
                                                      const double* positions, int64_t n, int32_t* out_counts,
                                                      int32_t* out_degenerate, const double* x0);
/* out_wnrs[i] += the same count: after agwn_param_batch_fractional_bezier3_f64 into out_wnrs, the full parametric
 * GWN of eval_gwnr_parametric_batch. */
int agwn_param_add_integer_bezier3x3_f64(agwn_context* ctx, agwn_patches* patches, const double* positions,
                                         int64_t n, double* out_wnrs, const double* x0);

/* agwn_param_batch_fractional_bezier3_f64 with start depths proposed by `mlp` in the same call (kept in device
 * scratch): the learned form of eval_gwnr_parametric_batch_fractional. */
int agwn_param_batch_fractional_learned_bezier3_f64(agwn_context* ctx, const agwn_mlp* mlp, const double* positions,
                                                    int64_t n, double* out, const double* x0, const double* curves,
                                                    int64_t n_curves, int n_classes, int min_depth, int max_depth,
                                                    double tol, float alpha, uint32_t* pair_stats,
                                                    int32_t* nodes_per_query);

/* The robust evaluator's exact predicates (robust_predicates.hh:273-402: edge_sign :315-331, atan2_num :340-356,
 * project_into_tri :391-402), evaluated on the device for caller-given coordinates so that they can be checked
 * against the reference's own predicate vectors.  Row i takes the triples q[i], q0[i], q1[i], q2[i] (int32 under
 * AGWN_ROBUST_INT64_GRID, int64 under AGWN_ROBUST_INT128_GRID, double under AGWN_ROBUST_EXACT_FLOAT) and writes
 * edge_sign(q, q0, q1), atan2_num(q, q0, q1) rounded to double, project_into_tri(q, q0, q1, q2).sign and, when
 * weights is not NULL, its weights w0, w1, w2 (3 doubles per row).  These are the functions the robust kernels
 * call.  Arrays may be host or device memory. */
int agwn_robust_predicates(agwn_context* ctx, int policy, const void* q, const void* q0, const void* q1,
                           const void* q2, int64_t n, int32_t* edge_sign, double* num, int32_t* inside,
                           double* weights);
/* a[i]*b[i] - c[i]*d[i] in the predicates' 128-bit integer arithmetic (robust_predicates.hh:60-143, int128::mul
 * and its subtraction and double conversion): the low and high words and the double.  No other use. */
int agwn_probe_i128_mul_sub(agwn_context* ctx, const int64_t* a, const int64_t* b, const int64_t* c,
                            const int64_t* d, int64_t n, uint64_t* lo, int64_t* hi, double* dbl);

/* ---- mixed-precision fractional term without allocation --------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device memory -- a program whose own pool
 * allocator owns the GPU's memory budget, or a plugin inside a framework whose allocator must not be bypassed --
 * this runs the mixed form of agwn_mesh_batch_fractional_f64 (default tau and term-error bound, no integer term)
 * with no context and no allocation.  Its scratch is one static device array of 1,409,120 bytes, sized for at most
 * 8192 boundary segments and held on every GPU that loads the library until the process exits; more segments are
 * rejected with AGWN_ERR_INVALID.  positions, out and boundary must be device memory of the current device;
 * x0 is 3 host doubles.  stream may be NULL (the default stream).  The first call on a device looks up the
 * scratch array's device address, so make that first call before any stream capture.  Every call is synchronous:
 * it waits for its kernels on `stream` and reads the device's error flags back before it returns.  All calls
 * share the one scratch array, which keeps the last call's contents: calls that overlap on the GPU (from several
 * host threads or streams) race and must be serialised by the caller. */
int agwn_mesh_batch_fractional_mixed_noalloc_f64(void* stream, const double* positions, int64_t n, double* out,
                                                 const double* x0, const double* boundary, int64_t n_segments);

/* ---- measurement ------------------------------------------------------------------------------------------
 * FP32 fused-multiply-add throughput of the context's GPU at its current clocks, in TFLOP/s (best of three timed
 * launches of independent FMA chains).  No reference counterpart: it is the denominator of the fractional
 * kernel's compute roofline. */
int agwn_probe_fp32_peak(agwn_context* ctx, double* tflops);
/* The same for FP64 fused multiply-add: the denominator of the parametric integrator's roofline. */
int agwn_probe_fp64_peak(agwn_context* ctx, double* tflops);
/* The mixed kernel's own float atan2 and CUDA's atan2f on the same n inputs (host or device arrays), for testing
 * the former's error.  No reference counterpart. */
int agwn_probe_atan2(agwn_context* ctx, const float* y, const float* x, int64_t n, float* ours, float* cuda_ref);

#ifdef __cplusplus
}
#endif
#endif /* ANTIPODAL_GB300_H */
