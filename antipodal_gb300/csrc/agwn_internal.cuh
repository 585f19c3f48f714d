// Shared internals of libantipodal_gb300: error reporting, the context (stream, scratch arena, options,
// timing), host/device pointer handling and small device helpers.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "../../include/antipodal_gb300.h"

namespace agwn
{
// ---- errors --------------------------------------------------------------------------------------------------
void set_message(const char* fmt, ...);
int fail(int status, const char* fmt, ...);
void clear_message();

#define AGWN_TRY_CUDA(expr)                                                                                        \
    do                                                                                                             \
    {                                                                                                              \
        cudaError_t agwn_e_ = (expr);                                                                              \
        if (agwn_e_ != cudaSuccess)                                                                                \
            return ::agwn::fail(agwn_e_ == cudaErrorMemoryAllocation ? AGWN_ERR_NOMEM : AGWN_ERR_CUDA,             \
                                "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(agwn_e_), __FILE__, __LINE__); \
    } while (0)

#define AGWN_TRY(expr)                                                                                             \
    do                                                                                                             \
    {                                                                                                              \
        int agwn_s_ = (expr);                                                                                      \
        if (agwn_s_ != AGWN_OK)                                                                                    \
            return agwn_s_;                                                                                        \
    } while (0)

#define AGWN_CHECK_ARG(cond, ...)                                                                                  \
    do                                                                                                             \
    {                                                                                                              \
        if (!(cond))                                                                                               \
            return ::agwn::fail(AGWN_ERR_INVALID, __VA_ARGS__);                                                    \
    } while (0)

// Device-side error flags, one word each, set with atomicOr by kernels and read by the host at synchronisation.
constexpr int kCounters = 12; // device statistics counters of a context

enum flag_slot
{
    FLAG_STACK = 0,   // traversal stack exhausted
    FLAG_TIMEOUT = 1, // bounded wait ran out
    FLAG_COUNT = 8
};

// ---- device scratch ----------------------------------------------------------------------------------------
// A grow-only device buffer.  Slots are reused across calls of one context.
struct DevBuf
{
    void* ptr = nullptr;
    size_t cap = 0;
    int reserve(size_t bytes);
    void release();
};

enum scratch_slot
{
    S_QUERIES = 0,
    S_OUT = 1,
    S_COUNTS = 2,
    S_SEGS = 3,
    S_SEGS_RAW = 4,
    S_FRAME = 5,
    S_MISC0 = 6,
    S_MISC1 = 7,
    S_MISC2 = 8,
    S_MISC3 = 9,
    S_PARTIAL = 10, // the parametric integrator's per-group partial sums
    S_ORDER0 = 11,  // the spatial order of the queries: sort keys, indices, digit counters (order.cu)
    S_ORDER1 = 12,  // the queries in that order and their outputs
    S_COUNT = 13
};

// A hierarchy over triangles in the frame of one ray direction (built by build_hier, lbvh.cu): internal nodes,
// the triangles in leaf order, their projected (u, v) corners, the frame and the depth.
struct Hier
{
    DevBuf nodes;
    DevBuf tri;
    DevBuf leaf_uv;
    int32_t depth = 0;
    int64_t n_tri = 0;
    float frame[9] = {};
    double scale = 1.0; // largest |coordinate| of the triangles
    void release()
    {
        nodes.release();
        tri.release();
        leaf_uv.release();
    }
};

// A uniform grid over the (u, v) plane of a ray-frame hierarchy: per cell (CSR), the leaves whose (u, v) box,
// widened by `margin`, overlaps the cell (lbvh.cu).
struct CellGrid
{
    DevBuf offsets; // n_cells + 1 unsigned
    DevBuf list;    // leaf indices
    int gu = 0, gv = 0;
    float umin = 0, vmin = 0, umax = 0, vmax = 0, inv_u = 0, inv_v = 0;
    float margin = 0;  // the widening of every leaf's box
    float tol_max = 0; // queries whose own tolerance exceeds this take the hierarchy walk
    int64_t entries = 0;
    bool valid = false;
    void release()
    {
        offsets.release();
        list.release();
        valid = false;
    }
};

// The hierarchy of one intersector along one direction, cached per context.  Keyed by the intersector's
// generation number and the direction's bits.
struct RayCache
{
    unsigned long long generation = 0;
    double dir[3] = {0, 0, 0};
    int scalar_bytes = 0;
    Hier h;
    CellGrid cells; // built on first use, invalid whenever h is rebuilt
};

struct Context
{
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int* d_flags = nullptr;        // FLAG_COUNT ints
    int* h_flags = nullptr;        // pinned mirror
    long long* d_counters = nullptr; // kCounters: [0] fp64 pairs, [1] pairs, [2] parametric skips, [3] certified pairs, [4..7] integer, [8..11] patches
                                     // term: queries, cell-list entries, candidate leaves, exact tests
    DevBuf scratch[S_COUNT];
    int sm_count = 0;
    RayCache ray_cache;
    // host-array pipeline (mesh batch): upload and download streams and their events, created on first use
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    cudaStream_t compute2 = nullptr; // the host-array pipeline runs alternate chunks' kernels here
    cudaEvent_t pipe_ev[8] = {};
    int ensure_pipeline();

    // options
    int frac_mode = AGWN_FRAC_EXACT;
    double mixed_tau = 4.0;
    double mixed_term_err = 6e-8;
    int robust_mode = AGWN_ROBUST_EXACT;
    double robust_term_err = 1e-7;
    int param_mode = AGWN_PARAM_EXACT;
    const agwn_mlp* panel_mlp = nullptr; // the per-panel network of the double-float integrator (or none)
    float panel_beta = 0.02f;
    int integer_cells = 1;
    double mixed_min_pairs = double(1 << 14);
    bool mixed_certify = true;
    // the spatial order of the queries (order.cu): the last decision and its key, and whether an evaluation on an
    // ordered copy is running (no second ordering inside it)
    const void* order_ptr = nullptr;
    int64_t order_n = 0;
    double order_dir[3] = {0, 0, 0};
    bool order_incoherent = false;
    float order_lo[2] = {0.f, 0.f};
    float order_scale = 1.f;
    bool ordering = false;
    int queries_per_thread = 2;
    int frac_block = 0; // 0: chosen per launch (frac.cu)
    int seg_tile = 512;
    int timing = 0;

    // statistics
    double kernel_ms[AGWN_K_COUNT] = {};
    long long launches[AGWN_K_COUNT] = {};
    static constexpr int kMaxPending = 64;
    cudaEvent_t ev_begin[kMaxPending] = {};
    cudaEvent_t ev_end[kMaxPending] = {};
    int pending_class[kMaxPending] = {};
    int n_pending = 0;

    // Whether a mixed-mode call of `pairs` (query, segment) pairs over a boundary of n_seg segments runs the mixed
    // kernels: at least mixed_min_pairs pairs over at least kMixedMinSegments segments, or always with the minimum 0.
    // The exact kernel's time follows the boundary's length (each thread's chain of FP64 terms), the mixed kernel's
    // has a fixed part (the boundary's preparation) and, over long segments, many pairs within the near distance
    // that go to FP64 anyway: on a GB300 the exact kernels were faster below 32 segments at every query count tried
    // (2,000 to 200,000 random queries; 4 segments and 2e5 queries: 202 against 297 us), the mixed ones from 64
    // segments at every count (64 segments and 2,000 queries: 293 against 537 us; 128: 198 against 1,065 us).
    static constexpr int64_t kMixedMinSegments = 32;
    bool use_mixed(double pairs, int64_t n_seg) const
    {
        return mixed_min_pairs == 0.0 || (pairs >= mixed_min_pairs && n_seg >= kMixedMinSegments);
    }

    int scratch_reserve(int slot, size_t bytes, void** out);
    // Brackets a launch with timing events when AGWN_OPT_TIMING is on; always counts the launch.
    int launch_begin(int kclass);
    int launch_end(int kclass);
    int drain_timing(); // folds finished events into kernel_ms (synchronises the stream)
    int check_flags();  // synchronises and reports device flags
};

// ---- host/device pointers ----------------------------------------------------------------------------------
bool is_device_pointer(const void* p);

// Makes `count` elements of `src` readable by the device: returns src itself for device memory, else copies
// it into scratch `slot` on the context's stream.
int stage_in(Context& ctx, const void* src, size_t bytes, int slot, const void** dev);
// Output staging: returns `dst` for device memory, else scratch `slot`; `*host` tells whether a copy back is due.
int stage_out(Context& ctx, void* dst, size_t bytes, int slot, void** dev, bool* host);

// ---- parametric path (param.cu, mlp.cu) ----------------------------------------------------------------------
// Device-side runners behind the parametric entry points; all pointers are device memory of the context's GPU.
int param_run(Context& ctx, const double* d_pos, int64_t n, double* d_out, const double* x0, const double* d_curves,
              int64_t n_curves, int min_depth, int max_depth, double tol, const uint8_t* d_start, uint32_t* d_stats,
              int32_t* d_nodes, uint32_t* d_panel_log = nullptr, unsigned long long* d_log_count = nullptr,
              long long log_cap = 0);
// The device copies of a network's weights (BF16 layouts) and FP32 parameters.
void mlp_device_weights(const agwn_mlp* mlp, const void** bf16_weights, const float** params);
int mlp_propose_run(Context& ctx, const agwn_mlp* mlp, const double* d_pos, int64_t n, const double* x0,
                    const double* d_curves, int64_t n_curves, int n_classes, int min_depth, int max_depth, double tol,
                    float alpha, uint8_t* d_start, float* d_logits);

// ---- launch geometry ---------------------------------------------------------------------------------------
inline int div_up(int64_t a, int64_t b)
{
    return int((a + b - 1) / b);
}
} // namespace agwn

struct agwn_context : agwn::Context
{
};

// ---- device helpers ----------------------------------------------------------------------------------------
namespace agwn
{
// Unfused IEEE arithmetic.  Each operation rounds once, like the reference's default (FMA-free) CPU build, so a
// formula written with these reproduces the CPU's values exactly.  The intrinsics are never contracted.
struct rd
{
    double v;
    rd() = default;
    __host__ __device__ __forceinline__ constexpr rd(double x) : v(x) {}
    __device__ __forceinline__ friend rd operator+(rd a, rd b) { return rd(__dadd_rn(a.v, b.v)); }
    __device__ __forceinline__ friend rd operator-(rd a, rd b) { return rd(__dsub_rn(a.v, b.v)); }
    __device__ __forceinline__ friend rd operator*(rd a, rd b) { return rd(__dmul_rn(a.v, b.v)); }
    __device__ __forceinline__ friend rd operator/(rd a, rd b) { return rd(__ddiv_rn(a.v, b.v)); }
    __device__ __forceinline__ friend rd operator-(rd a) { return rd(-a.v); }
};
struct rf
{
    float v;
    rf() = default;
    __device__ __forceinline__ constexpr rf(float x) : v(x) {}
    __device__ __forceinline__ friend rf operator+(rf a, rf b) { return rf(__fadd_rn(a.v, b.v)); }
    __device__ __forceinline__ friend rf operator-(rf a, rf b) { return rf(__fsub_rn(a.v, b.v)); }
    __device__ __forceinline__ friend rf operator*(rf a, rf b) { return rf(__fmul_rn(a.v, b.v)); }
    __device__ __forceinline__ friend rf operator/(rf a, rf b) { return rf(__fdiv_rn(a.v, b.v)); }
    __device__ __forceinline__ friend rf operator-(rf a) { return rf(-a.v); }
};
template <class T>
struct exact_of;
template <>
struct exact_of<double>
{
    using type = rd;
};
template <>
struct exact_of<float>
{
    using type = rf;
};

__device__ __forceinline__ rd ex_sqrt(rd a)
{
    return rd(__dsqrt_rn(a.v));
}
__device__ __forceinline__ rf ex_sqrt(rf a)
{
    return rf(__fsqrt_rn(a.v));
}
__device__ __forceinline__ double ex_atan2(rd y, rd x)
{
    return atan2(y.v, x.v);
}
__device__ __forceinline__ float ex_atan2(rf y, rf x)
{
    return atan2f(y.v, x.v);
}

template <class S>
struct ev3
{
    S x, y, z;
};
template <class S>
__device__ __forceinline__ ev3<S> operator-(ev3<S> a, ev3<S> b)
{
    return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <class S>
__device__ __forceinline__ S edot(ev3<S> a, ev3<S> b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <class S>
__device__ __forceinline__ ev3<S> ecross(ev3<S> a, ev3<S> b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Bounded spin limits: every device-side wait gives up after this many polls and raises FLAG_TIMEOUT.
constexpr long long kSpinLimit = 1ll << 22;
} // namespace agwn
