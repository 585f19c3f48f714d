// Fractional (boundary) term of the mesh GWN, and the C ABI of the mesh batch functions.
//
// The reference evaluates, per query p, sum_s w_s * atan2(num, den) / (2 pi) with the unnormalised
// Van Oosterom-Strackee half area of (x1 = -x0, pos0 - p, pos1 - p)
// (src/antipodal/math/common.hh:181-189, src/antipodal/gwn_mesh.hh:34-46).
//
// Work decomposition.  Each CTA walks the boundary in tiles of segments staged into shared memory by
// cp.async.bulk (mbarrier-completed, bounded waits), double-buffered when the boundary spans more than one
// tile.  All lanes of a warp read the same segment (a shared-memory broadcast) and every thread owns K
// queries, so one segment read feeds 32*K (query, segment) pairs.  CTAs are persistent over query tiles.
//
// Two arithmetic forms:
//  * exact  -- the reference formula in the input precision with unfused, correctly rounded operations
//              (rd/rf), summed in segment order: the same values as the CPU reference up to atan2's last bit.
//  * mixed  -- double input only.  Queries and segments are moved to a frame where x1 is +z and centred on the
//              boundary; queries and boundary vertices are held as float pairs hi + lo and the segment vector
//              d = P1 - P0 is rounded from FP64.  The boundary is walked as chains of segments that share
//              vertices (k_prep_mixed), so v = (P_hi - Q_hi) + (P_lo - Q_lo), |v| and the half-angle form of each
//              vertex are computed once for the two segments that meet there.  A pair (query, segment) is
//              evaluated in FP32 from v0, v1 and d:
//                num = v0.x*d.y - v0.y*d.x  (no cancellation for a far segment: d is accurate on its own),
//                den = (l0 + z0)(l1 + z1) + v0.x*v1.x + v0.y*v1.y  with l + z = (x^2 + y^2)/(l - z) for z < 0
//              and atan2f, summed with TwoSum compensation.  Each term is then accurate to about eps32 times its
//              angular size, whether or not the segments close into loops.  Pairs where that is not safe go to
//              FP64:
//                near:   the nearer endpoint is closer than tau * |segment|, evaluated with the exact form;
//                ill-conditioned: the first-order error bound of atan2(num, den) from the FP32 rounding of num and
//                        den exceeds term_err radians (the antipodal axis passes close to an endpoint);
//                branch: den < 0 and |num| within the FP32 error bound, i.e. the antipodal ray passes so close to
//                        the segment that the atan2 branch (+-pi) is decided by rounding.  The sign of num is
//                        then recomputed with the reference's FP64 formula, so the branch taken is the CPU's.
//              The FP64 terms and the compensated FP32 sum are combined in FP64.

#include "agwn_internal.cuh"

#include <algorithm>
#include "frac_kernels.cuh"
#include "gwn_kernels.cuh"
#include "robust.cuh"
#include "tma.cuh"

#include <cmath>

namespace agwn
{
namespace
{
template <class Kern>
int launch_persistent(Context& ctx, Kern kernel, int block, size_t smem, int64_t n_qtiles, int* grid)
{
    // opt in for the dynamic size on every launch: static shared memory counts against the 48 KB default too
    AGWN_TRY_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int per_sm = 0;
    AGWN_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem));
    if (per_sm < 1)
        return fail(AGWN_ERR_UNSUPPORTED, "fractional kernel does not fit on an SM (block %d, smem %zu)", block, smem);
    int64_t const g = std::min<int64_t>(n_qtiles, int64_t(per_sm) * ctx.sm_count);
    *grid = int(std::max<int64_t>(g, 1));
    return AGWN_OK;
}
} // namespace

namespace
{
// A boundary prepared for the fractional kernels (device scratch of the context), reusable by any number of
// launches on the same context stream until the next preparation.
// The largest entry stream the mixed kernel stages as one shared-memory tile (57.6 KB: three 256-thread blocks per
// SM).
constexpr int64_t kSingleTileEntries = 1200;

template <class T>
struct FracPlan
{
    int64_t n_seg = 0;
    bool mixed = false;
    int tile = 0;     // segments (exact) or entries (mixed) per shared-memory tile
    int nbuf = 1;     // shared-memory buffers
    T x0[3] = {};
    double x0d[3] = {};
    Rot rot{};
    SegX<T>* seg = nullptr;     // exact form
    SegM* segm = nullptr;       // mixed form: the entry stream
    SegX<double>* seg64 = nullptr;
    Frame* frame = nullptr;
};

// n_queries: the queries the plan will serve.  On a boundary shorter than 32 segments, or below ctx.mixed_min_pairs
// (query, segment) pairs, the mixed mode runs the exact kernels (Context::use_mixed: there they are the faster ones,
// and the exact form is the more accurate one).  So does a boundary of 2^24 segments or more, beyond the mixed
// kernel's FP64 queue entries (24-bit segment indices).
// force_mixed: the mixed form whatever the context's fractional mode and the size (double only).
template <class T>
int fractional_prepare(Context& ctx, const T* x0_host, const T* d_seg_raw, int64_t n_seg, int64_t n_queries,
                       FracPlan<T>* plan, bool force_mixed = false)
{
    FracPlan<T>& p = *plan;
    p = FracPlan<T>{};
    p.n_seg = n_seg;
    for (int k = 0; k < 3; ++k)
    {
        p.x0[k] = x0_host[k];
        p.x0d[k] = double(x0_host[k]);
    }
    if (n_seg == 0)
        return AGWN_OK;
    AGWN_CHECK_ARG(n_seg < (int64_t(1) << 31), "at most 2^31 - 1 boundary segments");
    p.mixed = (force_mixed || (ctx.frac_mode == AGWN_FRAC_MIXED && n_seg < (int64_t(1) << 24) &&
                               ctx.use_mixed(double(n_queries) * double(n_seg), n_seg))) &&
              sizeof(T) == 8;
    if (!p.mixed)
    {
        p.tile = int(std::min<int64_t>(ctx.seg_tile, n_seg));
        p.nbuf = n_seg > p.tile ? 2 : 1;
        AGWN_TRY(ctx.scratch_reserve(S_SEGS, sizeof(SegX<T>) * n_seg, reinterpret_cast<void**>(&p.seg)));
        AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
        k_prep_exact<T><<<std::min<int64_t>(div_up(n_seg, 256), 4 * ctx.sm_count), 256, 0, ctx.stream>>>(
            d_seg_raw, n_seg, p.seg);
        return ctx.launch_end(AGWN_K_OTHER);
    }
    AGWN_CHECK_ARG(n_seg < (int64_t(1) << 24), "the mixed form takes at most 2^24 - 1 boundary segments");
    double const x0n = p.x0d[0] * p.x0d[0] + p.x0d[1] * p.x0d[1] + p.x0d[2] * p.x0d[2];
    AGWN_CHECK_ARG(x0n > 0 && std::isfinite(x0n), "mixed mode needs a finite nonzero x0");
    p.rot = make_rotation(p.x0d);
    // the entry stream holds between n_seg + 1 and 2 n_seg entries; the tile (even) and the buffers are sized for
    // the most, the kernel reads the count k_prep_mixed wrote
    int64_t const max_entries = 2 * n_seg;
    p.tile = int(std::min<int64_t>(ctx.seg_tile, max_entries));
    p.nbuf = max_entries > p.tile ? 2 : 1;
    int64_t const n_order = chain_scratch_ints(n_seg);
    AGWN_TRY(ctx.scratch_reserve(S_SEGS, sizeof(SegM) * max_entries + sizeof(int) * n_order,
                                 reinterpret_cast<void**>(&p.segm)));
    int* const order = reinterpret_cast<int*>(p.segm + max_entries);
    AGWN_TRY(ctx.scratch_reserve(S_SEGS_RAW, sizeof(SegX<double>) * n_seg, reinterpret_cast<void**>(&p.seg64)));
    AGWN_TRY(ctx.scratch_reserve(S_FRAME, sizeof(Frame), reinterpret_cast<void**>(&p.frame)));
    AGWN_TRY(ctx.launch_begin(AGWN_K_OTHER));
    k_prep_mixed<<<1, 1024, 0, ctx.stream>>>(reinterpret_cast<const double*>(d_seg_raw), n_seg, p.rot,
                                             float(ctx.mixed_tau), p.frame, p.segm, p.seg64, order);
    AGWN_TRY(ctx.launch_end(AGWN_K_OTHER));
    // The stream holds n_seg + (number of chains) entries, at most 2 n_seg.  When that bound would take several
    // tiles but the boundary could fit one, the actual count is read back (a wait on the stream): one tile runs
    // without block barriers (a 1,066-segment boundary in 20 loops, 1e7 queries: 34.9 ms in three tiles, 33.6 ms
    // in one).
    if (p.nbuf > 1 && n_seg <= kSingleTileEntries)
    {
        long long m = 0;
        AGWN_TRY_CUDA(cudaMemcpyAsync(&m, &p.frame->n_entries, sizeof(m), cudaMemcpyDeviceToHost, ctx.stream));
        AGWN_TRY_CUDA(cudaStreamSynchronize(ctx.stream));
        if (m <= kSingleTileEntries)
        {
            p.tile = int(m);
            p.nbuf = 1;
        }
    }
    return AGWN_OK;
}

template <class T, class FB>
int fractional_launch_mixed(Context& ctx, const FracPlan<T>& p, const double* d_pos, int64_t n, double* d_out,
                            const int32_t* d_counts, FB fb);

template <class T>
int fractional_launch(Context& ctx, const FracPlan<T>& p, const T* d_pos, int64_t n, T* d_out,
                      const int32_t* d_counts)
{
    if (n == 0)
        return AGWN_OK;
    if (p.n_seg == 0)
    {
        AGWN_TRY(ctx.launch_begin(AGWN_K_FRACTIONAL));
        k_fill_counts<T><<<std::min<int64_t>(div_up(n, 256), 4 * ctx.sm_count), 256, 0, ctx.stream>>>(d_out, d_counts,
                                                                                                      n);
        return ctx.launch_end(AGWN_K_FRACTIONAL);
    }
    int const K = ctx.queries_per_thread;
    int const block = ctx.frac_block ? ctx.frac_block : 128;
    int64_t const per_tile = int64_t(block) * K;
    int64_t const n_qtiles = (n + per_tile - 1) / per_tile;
    if (!p.mixed)
    {
        size_t const smem = size_t(p.nbuf) * p.tile * sizeof(SegX<T>);
        auto launch = [&](auto kern) -> int
        {
            int grid = 0;
            AGWN_TRY(launch_persistent(ctx, kern, block, smem, n_qtiles, &grid));
            AGWN_TRY(ctx.launch_begin(AGWN_K_FRACTIONAL));
            kern<<<grid, block, smem, ctx.stream>>>(d_pos, n, d_out, d_counts, p.x0[0], p.x0[1], p.x0[2], p.seg,
                                                    p.n_seg, p.tile, ctx.d_flags);
            return ctx.launch_end(AGWN_K_FRACTIONAL);
        };
        switch (K)
        {
        case 1:
            return launch(k_frac_exact<T, 1>);
        case 2:
            return launch(k_frac_exact<T, 2>);
        case 4:
            return launch(k_frac_exact<T, 4>);
        default:
            return launch(k_frac_exact<T, 8>);
        }
    }
    return fractional_launch_mixed(ctx, p, reinterpret_cast<const double*>(d_pos), n, reinterpret_cast<double*>(d_out),
                                   d_counts, MeshFallback{p.seg64});
}

// The mixed kernel over a prepared plan, with the FP64 rule fb for the pairs it turns down.
template <class T, class FB>
int fractional_launch_mixed(Context& ctx, const FracPlan<T>& p, const double* d_pos, int64_t n, double* d_out,
                            const int32_t* d_counts, FB fb)
{
    int const K = std::max(2, ctx.queries_per_thread); // the kernel packs its queries in pairs
    // measured: one tile, 128 threads (10.2 ms against 10.6 on a 212-segment boundary); several tiles, 256 threads
    // (34.9 ms against 40.5 on 1,066 segments), since more queries share each staged tile and its barriers
    int const block = ctx.frac_block ? ctx.frac_block : (p.nbuf > 1 || p.tile > 512 ? 256 : 128);
    int64_t const n_qtiles = (n + int64_t(block) * K - 1) / (int64_t(block) * K);
    size_t const smem = size_t(p.nbuf) * p.tile * sizeof(SegM);
    auto launch = [&](auto kern) -> int
    {
        int grid = 0;
        AGWN_TRY(launch_persistent(ctx, kern, block, smem, n_qtiles, &grid));
        AGWN_TRY(ctx.launch_begin(AGWN_K_FRACTIONAL));
        kern<<<grid, block, smem, ctx.stream>>>(d_pos, n, d_out, d_counts, p.x0d[0], p.x0d[1], p.x0d[2], p.rot,
                                                p.frame, int(ctx.mixed_certify), float(ctx.mixed_term_err), p.segm, fb,
                                                p.n_seg, p.tile,
                                                ctx.d_flags, ctx.d_counters, ctx.timing);
        return ctx.launch_end(AGWN_K_FRACTIONAL);
    };
    switch (K)
    {
    case 2:
        return launch(k_frac_mixed<2, FB>);
    case 4:
        return launch(k_frac_mixed<4, FB>);
    default:
        return launch(k_frac_mixed<8, FB>);
    }
}

// The robust evaluator's FP64 rule (exact_float policy) for a pair the mixed kernel turns down: the reference's
// per-segment branches (gwn_mesh_robust.hh:272-321) on the query's own doubles and the evaluator's swapped segment,
// so the branch of every pair near the ray is the reference's exact decision.
struct RobustFallbackPF
{
    const RSeg<double>* seg;
    // not inlined: the rule's registers stay out of the kernel's FP32 loop (it runs once per 32 routed pairs)
    __device__ __noinline__ double operator()(const double* __restrict__ pos, int64_t i, uint32_t s, ev3<rd>) const
    {
        RSeg<double> const g = seg[s];
        qv3<double> const q{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        return __dmul_rn(g.w, robust_contrib<PF>(q, g));
    }
};
} // namespace

template <class T>
int fractional_run(Context& ctx, const T* d_pos, int64_t n, T* d_out, const int32_t* d_counts, const T* x0_host,
                   const T* d_seg_raw, int64_t n_seg)
{
    if (n == 0)
        return AGWN_OK;
    FracPlan<T> plan;
    AGWN_TRY(fractional_prepare<T>(ctx, x0_host, d_seg_raw, n_seg, n, &plan));
    return fractional_launch<T>(ctx, plan, d_pos, n, d_out, d_counts);
}

template int fractional_run<double>(Context&, const double*, int64_t, double*, const int32_t*, const double*,
                                    const double*, int64_t);
template int fractional_run<float>(Context&, const float*, int64_t, float*, const int32_t*, const float*, const float*,
                                   int64_t);

int frac_mixed_robust_pf(Context& ctx, const double* d_pos, int64_t n, double* d_out, const int32_t* d_counts,
                         const double* d_raw, int64_t n_seg, const void* rseg)
{
    if (n == 0)
        return AGWN_OK;
    // the robust term along the -x ray is the mesh term with x0 = -x on the unswapped segments (x1 = +x: the same
    // numerator and l + x denominator)
    double const x0[3] = {-1.0, 0.0, 0.0};
    FracPlan<double> plan;
    AGWN_TRY(fractional_prepare<double>(ctx, x0, d_raw, n_seg, n, &plan, true));
    if (n_seg == 0)
        return fractional_launch<double>(ctx, plan, d_pos, n, d_out, d_counts);
    return fractional_launch_mixed(ctx, plan, d_pos, n, d_out, d_counts,
                                   RobustFallbackPF{static_cast<const RSeg<double>*>(rseg)});
}

int frac_mixed_robust_pf_chunked(Context& ctx, const double* d_pos, int64_t n, double* d_out, int32_t* d_counts,
                                 const double* d_raw, int64_t n_seg, const void* rseg, ChunkCounts count, void* user)
{
    if (n == 0)
        return AGWN_OK;
    AGWN_TRY(ctx.ensure_pipeline());
    int64_t chunk = std::max<int64_t>(int64_t(1) << 20, (n + 7) / 8);
    chunk = (chunk + 1023) / 1024 * 1024;
    double const x0[3] = {-1.0, 0.0, 0.0};
    FracPlan<double> plan;
    AGWN_TRY(fractional_prepare<double>(ctx, x0, d_raw, n_seg, n, &plan, true));
    cudaEvent_t const ready = ctx.pipe_ev[6];
    cudaEvent_t const joined = ctx.pipe_ev[7];
    cudaStream_t const main = ctx.stream;
    cudaStream_t const cs[2] = {main, ctx.compute2};
    AGWN_TRY_CUDA(cudaEventRecord(ready, main));
    AGWN_TRY_CUDA(cudaStreamWaitEvent(cs[1], ready, 0));
    int rc = AGWN_OK;
    for (int64_t i = 0; i * chunk < n && rc == AGWN_OK; ++i)
    {
        int64_t const q0 = i * chunk, m = std::min(chunk, n - q0);
        ctx.stream = cs[i & 1];
        rc = count(user, ctx, d_pos + 3 * q0, m, d_counts + q0);
        if (rc == AGWN_OK)
            rc = n_seg == 0 ? fractional_launch<double>(ctx, plan, d_pos + 3 * q0, m, d_out + q0, d_counts + q0)
                            : fractional_launch_mixed(ctx, plan, d_pos + 3 * q0, m, d_out + q0, d_counts + q0,
                                                      RobustFallbackPF{static_cast<const RSeg<double>*>(rseg)});
        ctx.stream = main;
    }
    AGWN_TRY_CUDA(cudaEventRecord(joined, cs[1]));
    AGWN_TRY_CUDA(cudaStreamWaitEvent(main, joined, 0));
    return rc;
}

// --------------------------------------------------------------------------------------------------------------
// C ABI: mesh batch functions
// --------------------------------------------------------------------------------------------------------------
namespace
{
// Host queries and host results: the batch runs in chunks through two device buffers, so that uploading chunk
// i + 1 and downloading chunk i - 1 (each on its own copy stream) overlap the kernels of chunk i on the context's
// stream.  Events order every reuse of a buffer: an upload waits until the kernels of the chunk two back have read
// its buffer, and the kernels wait until that chunk's results have left theirs.
template <class T>
int mesh_batch_pipelined(Context& ctx, const agwn_bvh* bvh, const T* positions, int64_t n, T* out, const T* x0,
                         const T* dseg, int64_t n_seg, bool want_frac)
{
    AGWN_TRY(ctx.ensure_pipeline());
    int64_t chunk = std::max<int64_t>(int64_t(1) << 20, (n + 7) / 8);
    chunk = (chunk + 1023) / 1024 * 1024;
    void *qbuf = nullptr, *obuf = nullptr;
    int32_t* dcounts = nullptr;
    AGWN_TRY(ctx.scratch_reserve(S_QUERIES, 2 * sizeof(T) * 3 * size_t(chunk), &qbuf));
    AGWN_TRY(ctx.scratch_reserve(S_OUT, 2 * sizeof(T) * size_t(chunk), &obuf));
    bool const with_int = bvh && bvh->n_tri > 0;
    if (with_int)
        AGWN_TRY(ctx.scratch_reserve(S_COUNTS, 2 * sizeof(int32_t) * size_t(chunk),
                                     reinterpret_cast<void**>(&dcounts)));
    cudaEvent_t* const up = ctx.pipe_ev;       // [b]: chunk uploaded into buffer b
    cudaEvent_t* const done = ctx.pipe_ev + 2; // [b]: kernels on buffer b finished
    cudaEvent_t* const down = ctx.pipe_ev + 4; // [b]: results of buffer b downloaded
    cudaEvent_t const ready = ctx.pipe_ev[6];  // the staged boundary and its preparation
    cudaEvent_t const joined = ctx.pipe_ev[7]; // the second compute stream's last kernels
    // The kernels of chunk i run on compute stream i & 1 (the context's stream and a second one), so the next
    // chunk's kernels fill the SMs that the end of the current chunk's fractional kernel leaves idle.
    cudaStream_t const main = ctx.stream;
    cudaStream_t const cs[2] = {main, ctx.compute2};
    // the boundary is prepared once, while the first chunk uploads, and serves every chunk
    AGWN_TRY_CUDA(cudaEventRecord(done[0], main));
    AGWN_TRY_CUDA(cudaStreamWaitEvent(ctx.copy_in, done[0], 0));
    FracPlan<T> plan;
    AGWN_TRY(fractional_prepare<T>(ctx, x0, dseg, want_frac ? n_seg : 0, n, &plan));
    if (with_int && n >= 1)
        AGWN_TRY(integer_prepare<T>(ctx, *bvh, x0)); // the hierarchy and its cell grid, built on the main stream
    AGWN_TRY_CUDA(cudaEventRecord(ready, main));
    AGWN_TRY_CUDA(cudaStreamWaitEvent(cs[1], ready, 0));
    int64_t const n_chunks = (n + chunk - 1) / chunk;
    int rc = AGWN_OK;
    for (int64_t i = 0; i < n_chunks && rc == AGWN_OK; ++i)
    {
        int const b = int(i & 1);
        int64_t const q0 = i * chunk, m = std::min(chunk, n - q0);
        T* const qb = static_cast<T*>(qbuf) + size_t(b) * 3 * chunk;
        T* const ob = static_cast<T*>(obuf) + size_t(b) * chunk;
        int32_t* const cb = with_int ? dcounts + size_t(b) * chunk : nullptr;
        if (i >= 2)
            AGWN_TRY_CUDA(cudaStreamWaitEvent(ctx.copy_in, done[b], 0));
        AGWN_TRY_CUDA(cudaMemcpyAsync(qb, positions + 3 * q0, sizeof(T) * 3 * m, cudaMemcpyHostToDevice, ctx.copy_in));
        AGWN_TRY_CUDA(cudaEventRecord(up[b], ctx.copy_in));
        AGWN_TRY_CUDA(cudaStreamWaitEvent(cs[b], up[b], 0));
        if (i >= 2)
            AGWN_TRY_CUDA(cudaStreamWaitEvent(cs[b], down[b], 0));
        ctx.stream = cs[b]; // the launches below go to this chunk's compute stream
        if (with_int)
            rc = integer_run<T>(ctx, *bvh, qb, m, cb, x0);
        if (rc == AGWN_OK)
            rc = fractional_launch<T>(ctx, plan, qb, m, ob, cb);
        ctx.stream = main;
        if (rc != AGWN_OK)
            break;
        AGWN_TRY_CUDA(cudaEventRecord(done[b], cs[b]));
        AGWN_TRY_CUDA(cudaStreamWaitEvent(ctx.copy_out, done[b], 0));
        AGWN_TRY_CUDA(cudaMemcpyAsync(out + q0, ob, sizeof(T) * m, cudaMemcpyDeviceToHost, ctx.copy_out));
        AGWN_TRY_CUDA(cudaEventRecord(down[b], ctx.copy_out));
    }
    // the main stream continues after everything of the second one
    AGWN_TRY_CUDA(cudaEventRecord(joined, cs[1]));
    AGWN_TRY_CUDA(cudaStreamWaitEvent(main, joined, 0));
    if (rc != AGWN_OK)
    {
        cudaStreamSynchronize(ctx.copy_out);
        cudaStreamSynchronize(main);
        return rc;
    }
    AGWN_TRY_CUDA(cudaStreamSynchronize(ctx.copy_out));
    return ctx.check_flags();
}

// Device queries and device results of the full GWN: the batch runs in 4 chunks (of 2^20 queries at least) whose
// kernels alternate between the context's stream and a second compute stream, as the host-array pipeline's do, so
// that the next chunk's integer and fractional kernels fill the SMs that the end of the current chunk's fractional
// kernel leaves idle.  Each chunk reads and writes its own slices (queries, counts, results), so no chunk waits for
// another; the boundary, the hierarchy and its cell grid are prepared once on the context's stream before either
// stream starts.  (On 256^3 queries of a 212-segment boundary: 4 chunks 7.18 ms, 8 chunks 7.25, 16 chunks 7.57.)
template <class T>
int mesh_batch_chunked(Context& ctx, const agwn_bvh* bvh, const T* dpos, int64_t n, T* dout, const T* x0,
                       const T* dseg, int64_t n_seg)
{
    AGWN_TRY(ctx.ensure_pipeline());
    int64_t chunk = std::max<int64_t>(int64_t(1) << 20, (n + 3) / 4);
    chunk = (chunk + 1023) / 1024 * 1024;
    bool const with_int = bvh && bvh->n_tri > 0;
    int32_t* dcounts = nullptr;
    if (with_int)
        AGWN_TRY(ctx.scratch_reserve(S_COUNTS, sizeof(int32_t) * size_t(n), reinterpret_cast<void**>(&dcounts)));
    cudaEvent_t const ready = ctx.pipe_ev[6];  // the prepared boundary, hierarchy and cell grid
    cudaEvent_t const joined = ctx.pipe_ev[7]; // the second compute stream's last kernels
    cudaStream_t const main = ctx.stream;
    cudaStream_t const cs[2] = {main, ctx.compute2};
    FracPlan<T> plan;
    AGWN_TRY(fractional_prepare<T>(ctx, x0, dseg, n_seg, n, &plan));
    if (with_int)
        AGWN_TRY(integer_prepare<T>(ctx, *bvh, x0));
    AGWN_TRY_CUDA(cudaEventRecord(ready, main));
    AGWN_TRY_CUDA(cudaStreamWaitEvent(cs[1], ready, 0));
    int64_t const n_chunks = (n + chunk - 1) / chunk;
    int rc = AGWN_OK;
    for (int64_t i = 0; i < n_chunks && rc == AGWN_OK; ++i)
    {
        int64_t const q0 = i * chunk, m = std::min(chunk, n - q0);
        int32_t* const cb = with_int ? dcounts + q0 : nullptr;
        ctx.stream = cs[i & 1]; // the launches below go to this chunk's compute stream
        if (with_int)
            rc = integer_run<T>(ctx, *bvh, dpos + 3 * q0, m, cb, x0);
        if (rc == AGWN_OK)
            rc = fractional_launch<T>(ctx, plan, dpos + 3 * q0, m, dout + q0, cb);
        ctx.stream = main;
    }
    // the context's stream continues after everything of the second one
    AGWN_TRY_CUDA(cudaEventRecord(joined, cs[1]));
    AGWN_TRY_CUDA(cudaStreamWaitEvent(main, joined, 0));
    return rc;
}

template <class T>
int mesh_batch(agwn_context* ctx, const agwn_bvh* bvh, const T* positions, int64_t n, T* out, const T* x0,
               const T* boundary, int64_t n_seg, bool want_frac)
{
    AGWN_CHECK_ARG(ctx, "null context");
    AGWN_CHECK_ARG(n >= 0 && n_seg >= 0, "negative size");
    AGWN_CHECK_ARG(n == 0 || (positions && out), "null positions/out");
    AGWN_CHECK_ARG(x0, "null x0");
    AGWN_CHECK_ARG(n_seg == 0 || boundary, "null boundary");
    if (bvh)
        AGWN_CHECK_ARG(bvh->scalar_bytes == int(sizeof(T)), "intersector precision does not match the queries");
    if (!want_frac && ctx->frac_mode == AGWN_FRAC_MIXED && sizeof(T) == 4)
        (void)0;
    clear_message();
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    if (n == 0)
        return AGWN_OK;
    const void* dpos = nullptr;
    const void* dseg = nullptr;
    void* dout = nullptr;
    bool host_out = false;
    if (n >= (int64_t(1) << 21) && !is_device_pointer(positions) && !is_device_pointer(out))
    {
        AGWN_TRY(stage_in(*ctx, boundary, sizeof(T) * 7 * n_seg, S_MISC0, &dseg));
        return mesh_batch_pipelined<T>(*ctx, bvh, positions, n, out, x0, static_cast<const T*>(dseg), n_seg,
                                       want_frac);
    }
    if constexpr (sizeof(T) == 8)
    {
        // mixed mode on device arrays: an incoherent query order runs on a spatially sorted copy (order.cu), where
        // the mixed kernel certifies far more boundary groups; the values are the same bit for bit
        if (want_frac && n_seg > 0 && ctx->frac_mode == AGWN_FRAC_MIXED && !ctx->ordering &&
            n_seg < (int64_t(1) << 24) && ctx->use_mixed(double(n) * double(n_seg), n_seg) &&
            is_device_pointer(positions) && is_device_pointer(out))
        {
            double const dir[3] = {x0[0], x0[1], x0[2]};
            const int32_t* perm = nullptr;
            AGWN_TRY(query_order(*ctx, positions, n, dir, true, &perm));
            if (perm)
            {
                double* ps = nullptr;
                AGWN_TRY(ctx->scratch_reserve(S_ORDER1, sizeof(double) * 4 * size_t(n), reinterpret_cast<void**>(&ps)));
                double* const os = ps + 3 * size_t(n);
                AGWN_TRY(gather_queries(*ctx, positions, perm, n, ps));
                ctx->ordering = true;
                int const rc = mesh_batch<T>(ctx, bvh, ps, n, os, x0, boundary, n_seg, want_frac);
                ctx->ordering = false;
                AGWN_TRY(rc);
                return scatter_back<double>(*ctx, os, perm, n, out);
            }
        }
    }
    if (n >= (int64_t(1) << 21) && want_frac && bvh && bvh->n_tri > 0 && is_device_pointer(positions) &&
        is_device_pointer(out))
    {
        AGWN_TRY(stage_in(*ctx, boundary, sizeof(T) * 7 * n_seg, S_MISC0, &dseg));
        AGWN_TRY(mesh_batch_chunked<T>(*ctx, bvh, positions, n, out, x0, static_cast<const T*>(dseg), n_seg));
        if (dseg != boundary)
            return ctx->check_flags(); // a staged host boundary must outlive its copy: finish before returning
        return AGWN_OK;
    }
    AGWN_TRY(stage_in(*ctx, positions, sizeof(T) * 3 * n, S_QUERIES, &dpos));
    AGWN_TRY(stage_in(*ctx, boundary, sizeof(T) * 7 * n_seg, S_MISC0, &dseg));
    AGWN_TRY(stage_out(*ctx, out, sizeof(T) * n, S_OUT, &dout, &host_out));
    int32_t* dcounts = nullptr;
    if (bvh && bvh->n_tri > 0)
    {
        AGWN_TRY(ctx->scratch_reserve(S_COUNTS, sizeof(int32_t) * n, reinterpret_cast<void**>(&dcounts)));
        AGWN_TRY(integer_run<T>(*ctx, *bvh, static_cast<const T*>(dpos), n, dcounts, x0));
    }
    if (want_frac)
        AGWN_TRY(fractional_run<T>(*ctx, static_cast<const T*>(dpos), n, static_cast<T*>(dout), dcounts, x0,
                                   static_cast<const T*>(dseg), n_seg));
    else
        AGWN_TRY(fractional_run<T>(*ctx, static_cast<const T*>(dpos), n, static_cast<T*>(dout), dcounts, x0,
                                   static_cast<const T*>(dseg), 0));
    if (host_out)
    {
        AGWN_TRY_CUDA(cudaMemcpyAsync(out, dout, sizeof(T) * n, cudaMemcpyDeviceToHost, ctx->stream));
        return ctx->check_flags();
    }
    if (dpos != positions || dseg != boundary)
        return ctx->check_flags(); // staged host inputs must outlive the copies: finish before returning
    return AGWN_OK;
}
} // namespace
} // namespace agwn

using namespace agwn;

extern "C"
{
int agwn_mesh_batch_fractional_f64(agwn_context* ctx, const double* positions, int64_t n, double* out,
                                   const double* x0, const double* boundary, int64_t n_segments)
{
    return mesh_batch<double>(ctx, nullptr, positions, n, out, x0, boundary, n_segments, true);
}
int agwn_mesh_batch_fractional_f32(agwn_context* ctx, const float* positions, int64_t n, float* out, const float* x0,
                                   const float* boundary, int64_t n_segments)
{
    return mesh_batch<float>(ctx, nullptr, positions, n, out, x0, boundary, n_segments, true);
}
int agwn_mesh_batch_f64(agwn_context* ctx, const agwn_bvh* bvh, const double* positions, int64_t n, double* out,
                        const double* x0, const double* boundary, int64_t n_segments)
{
    return mesh_batch<double>(ctx, bvh, positions, n, out, x0, boundary, n_segments, true);
}
int agwn_mesh_batch_f32(agwn_context* ctx, const agwn_bvh* bvh, const float* positions, int64_t n, float* out,
                        const float* x0, const float* boundary, int64_t n_segments)
{
    return mesh_batch<float>(ctx, bvh, positions, n, out, x0, boundary, n_segments, true);
}
} // extern "C"
