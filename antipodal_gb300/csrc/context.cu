// Context, errors, scratch memory and option handling of libantipodal_gb300.

#include "agwn_internal.cuh"

#include <cmath>

namespace agwn
{
namespace
{
thread_local char g_message[1024] = "";
}

void set_message(const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_message, sizeof(g_message), fmt, ap);
    va_end(ap);
}

int fail(int status, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_message, sizeof(g_message), fmt, ap);
    va_end(ap);
    return status;
}

void clear_message()
{
    g_message[0] = 0;
}

int DevBuf::reserve(size_t bytes)
{
    if (bytes <= cap)
        return AGWN_OK;
    release();
    size_t const want = bytes + bytes / 4 + 256;
    cudaError_t const e = cudaMalloc(&ptr, want);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        ptr = nullptr;
        cap = 0;
        return fail(e == cudaErrorMemoryAllocation ? AGWN_ERR_NOMEM : AGWN_ERR_CUDA, "cudaMalloc(%zu) failed: %s",
                    want, cudaGetErrorString(e));
    }
    cap = want;
    return AGWN_OK;
}

void DevBuf::release()
{
    if (ptr)
        cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
}

int Context::scratch_reserve(int slot, size_t bytes, void** out)
{
    // Scratch is shared by calls on this context's stream; a growing reallocation must not free memory that
    // queued work may still read.
    if (bytes > scratch[slot].cap)
        AGWN_TRY_CUDA(cudaStreamSynchronize(stream));
    AGWN_TRY(scratch[slot].reserve(bytes == 0 ? 1 : bytes));
    *out = scratch[slot].ptr;
    return AGWN_OK;
}

int Context::launch_begin(int kclass)
{
    launches[kclass] += 1;
    if (!timing)
        return AGWN_OK;
    if (n_pending == kMaxPending)
        AGWN_TRY(drain_timing());
    int const i = n_pending;
    if (!ev_begin[i])
    {
        AGWN_TRY_CUDA(cudaEventCreate(&ev_begin[i]));
        AGWN_TRY_CUDA(cudaEventCreate(&ev_end[i]));
    }
    pending_class[i] = kclass;
    AGWN_TRY_CUDA(cudaEventRecord(ev_begin[i], stream));
    return AGWN_OK;
}

int Context::launch_end(int kclass)
{
    (void)kclass;
    AGWN_TRY_CUDA(cudaGetLastError());
    if (!timing)
        return AGWN_OK;
    AGWN_TRY_CUDA(cudaEventRecord(ev_end[n_pending], stream));
    n_pending += 1;
    return AGWN_OK;
}

int Context::drain_timing()
{
    if (n_pending == 0)
        return AGWN_OK;
    for (int i = 0; i < n_pending; ++i)
    {
        // each launch's own end event: chunked calls record them on more than one stream
        AGWN_TRY_CUDA(cudaEventSynchronize(ev_end[i]));
        float ms = 0.f;
        AGWN_TRY_CUDA(cudaEventElapsedTime(&ms, ev_begin[i], ev_end[i]));
        kernel_ms[pending_class[i]] += ms;
    }
    n_pending = 0;
    return AGWN_OK;
}

int Context::check_flags()
{
    AGWN_TRY_CUDA(cudaMemcpyAsync(h_flags, d_flags, sizeof(int) * FLAG_COUNT, cudaMemcpyDeviceToHost, stream));
    AGWN_TRY_CUDA(cudaStreamSynchronize(stream));
    int stack = h_flags[FLAG_STACK], timeout = h_flags[FLAG_TIMEOUT];
    if (stack || timeout)
    {
        AGWN_TRY_CUDA(cudaMemsetAsync(d_flags, 0, sizeof(int) * FLAG_COUNT, stream));
        AGWN_TRY_CUDA(cudaStreamSynchronize(stream));
        if (timeout)
            return fail(AGWN_ERR_TIMEOUT, "a bounded device wait ran out (code %d); results of the call are invalid",
                        timeout);
        return fail(AGWN_ERR_STACK, "BVH traversal stack exhausted; results of the call are invalid");
    }
    return AGWN_OK;
}

bool is_device_pointer(const void* p)
{
    if (!p)
        return false;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
    {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int Context::ensure_pipeline()
{
    if (!copy_in)
        AGWN_TRY_CUDA(cudaStreamCreateWithFlags(&copy_in, cudaStreamNonBlocking));
    if (!copy_out)
        AGWN_TRY_CUDA(cudaStreamCreateWithFlags(&copy_out, cudaStreamNonBlocking));
    if (!compute2)
        AGWN_TRY_CUDA(cudaStreamCreateWithFlags(&compute2, cudaStreamNonBlocking));
    for (cudaEvent_t& e : pipe_ev)
        if (!e)
            AGWN_TRY_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return AGWN_OK;
}

int stage_in(Context& ctx, const void* src, size_t bytes, int slot, const void** dev)
{
    if (bytes == 0 || is_device_pointer(src))
    {
        *dev = src;
        return AGWN_OK;
    }
    void* d = nullptr;
    AGWN_TRY(ctx.scratch_reserve(slot, bytes, &d));
    AGWN_TRY_CUDA(cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, ctx.stream));
    *dev = d;
    return AGWN_OK;
}

int stage_out(Context& ctx, void* dst, size_t bytes, int slot, void** dev, bool* host)
{
    if (bytes == 0 || is_device_pointer(dst))
    {
        *dev = dst;
        *host = false;
        return AGWN_OK;
    }
    AGWN_TRY(ctx.scratch_reserve(slot, bytes, dev));
    *host = true;
    return AGWN_OK;
}
} // namespace agwn

using namespace agwn;

extern "C"
{
const char* agwn_status_string(int status)
{
    switch (status)
    {
    case AGWN_OK:
        return "ok";
    case AGWN_ERR_INVALID:
        return "invalid argument";
    case AGWN_ERR_CUDA:
        return "CUDA runtime error";
    case AGWN_ERR_NOMEM:
        return "out of device memory";
    case AGWN_ERR_STACK:
        return "BVH traversal stack exhausted";
    case AGWN_ERR_TIMEOUT:
        return "device wait timed out";
    case AGWN_ERR_UNSUPPORTED:
        return "unsupported";
    case AGWN_ERR_NO_DEVICE:
        return "no CUDA device";
    default:
        return "unknown status";
    }
}

const char* agwn_last_error_message(void)
{
    return g_message;
}

int agwn_abi_version(void)
{
    return AGWN_ABI_VERSION;
}

int agwn_context_create(int device, void* stream, agwn_context** out)
{
    AGWN_CHECK_ARG(out != nullptr, "agwn_context_create: out is null");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
    {
        cudaGetLastError();
        return fail(AGWN_ERR_NO_DEVICE, "no CUDA device available (%s)", cudaGetErrorString(e));
    }
    AGWN_CHECK_ARG(device >= 0 && device < n, "agwn_context_create: device %d out of range [0, %d)", device, n);
    AGWN_TRY_CUDA(cudaSetDevice(device));
    auto* ctx = new agwn_context{};
    ctx->device = device;
    int status = AGWN_OK;
    do
    {
        if (stream)
            ctx->stream = static_cast<cudaStream_t>(stream);
        else
        {
            if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess)
                break;
            ctx->own_stream = true;
        }
        if ((e = cudaMalloc(&ctx->d_flags, sizeof(int) * FLAG_COUNT)) != cudaSuccess)
            break;
        if ((e = cudaMemset(ctx->d_flags, 0, sizeof(int) * FLAG_COUNT)) != cudaSuccess)
            break;
        if ((e = cudaMalloc(&ctx->d_counters, sizeof(long long) * kCounters)) != cudaSuccess)
            break;
        if ((e = cudaMemset(ctx->d_counters, 0, sizeof(long long) * kCounters)) != cudaSuccess)
            break;
        if ((e = cudaMallocHost(&ctx->h_flags, sizeof(int) * FLAG_COUNT)) != cudaSuccess)
            break;
        if ((e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess)
            break;
    } while (false);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        status = fail(AGWN_ERR_CUDA, "agwn_context_create: %s", cudaGetErrorString(e));
        agwn_context_destroy(ctx);
        return status;
    }
    *out = ctx;
    return AGWN_OK;
}

int agwn_context_destroy(agwn_context* ctx)
{
    if (!ctx)
        return AGWN_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream)
        cudaStreamSynchronize(ctx->stream);
    for (auto& b : ctx->scratch)
        b.release();
    ctx->ray_cache.h.release();
    ctx->ray_cache.cells.release();
    for (int i = 0; i < Context::kMaxPending; ++i)
    {
        if (ctx->ev_begin[i])
            cudaEventDestroy(ctx->ev_begin[i]);
        if (ctx->ev_end[i])
            cudaEventDestroy(ctx->ev_end[i]);
    }
    if (ctx->d_flags)
        cudaFree(ctx->d_flags);
    if (ctx->d_counters)
        cudaFree(ctx->d_counters);
    if (ctx->h_flags)
        cudaFreeHost(ctx->h_flags);
    for (cudaEvent_t e : ctx->pipe_ev)
        if (e)
            cudaEventDestroy(e);
    if (ctx->copy_in)
        cudaStreamDestroy(ctx->copy_in);
    if (ctx->copy_out)
        cudaStreamDestroy(ctx->copy_out);
    if (ctx->compute2)
        cudaStreamDestroy(ctx->compute2);
    if (ctx->own_stream && ctx->stream)
        cudaStreamDestroy(ctx->stream);
    delete ctx;
    return AGWN_OK;
}

int agwn_context_synchronize(agwn_context* ctx)
{
    AGWN_CHECK_ARG(ctx, "agwn_context_synchronize: null context");
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    return ctx->check_flags();
}

int agwn_context_set_option(agwn_context* ctx, int option, double value)
{
    AGWN_CHECK_ARG(ctx, "agwn_context_set_option: null context");
    switch (option)
    {
    case AGWN_OPT_FRAC_MODE:
        AGWN_CHECK_ARG(value == AGWN_FRAC_EXACT || value == AGWN_FRAC_MIXED, "frac mode must be 0 or 1");
        ctx->frac_mode = int(value);
        return AGWN_OK;
    case AGWN_OPT_MIXED_TAU:
        AGWN_CHECK_ARG(std::isfinite(value) && value >= 0.0 && value <= 1e6, "tau must be in [0, 1e6]");
        ctx->mixed_tau = value;
        return AGWN_OK;
    case AGWN_OPT_QUERIES_PER_THREAD:
        AGWN_CHECK_ARG(value == 1 || value == 2 || value == 4 || value == 8, "queries per thread must be 1, 2, 4 or 8");
        ctx->queries_per_thread = int(value);
        return AGWN_OK;
    case AGWN_OPT_FRAC_BLOCK:
        AGWN_CHECK_ARG(value == 0 || (value >= 64 && value <= 256 && std::fmod(value, 32.0) == 0.0),
                       "block must be 0 (automatic) or a multiple of 32 in [64, 256]");
        ctx->frac_block = int(value);
        return AGWN_OK;
    case AGWN_OPT_TIMING:
        ctx->timing = value != 0.0;
        return AGWN_OK;
    case AGWN_OPT_SEG_TILE:
        AGWN_CHECK_ARG(value >= 32 && value <= 2048 && std::fmod(value, 32.0) == 0.0,
                       "segment tile must be a multiple of 32 in [32, 2048]");
        ctx->seg_tile = int(value);
        return AGWN_OK;
    case AGWN_OPT_MIXED_TERM_ERR:
        AGWN_CHECK_ARG(std::isfinite(value) && value > 0.0 && value <= 1.0, "term error bound must be in (0, 1]");
        ctx->mixed_term_err = value;
        return AGWN_OK;
    case AGWN_OPT_ROBUST_MODE:
        AGWN_CHECK_ARG(value == AGWN_ROBUST_EXACT || value == AGWN_ROBUST_MIXED, "robust mode must be 0 or 1");
        ctx->robust_mode = int(value);
        return AGWN_OK;
    case AGWN_OPT_ROBUST_TERM_ERR:
        AGWN_CHECK_ARG(std::isfinite(value) && value > 0.0 && value <= 1.0, "term error bound must be in (0, 1]");
        ctx->robust_term_err = value;
        return AGWN_OK;
    case AGWN_OPT_PARAM_MODE:
        AGWN_CHECK_ARG(value == AGWN_PARAM_EXACT || value == AGWN_PARAM_MIXED, "parametric mode must be 0 or 1");
        ctx->param_mode = int(value);
        return AGWN_OK;
    case AGWN_OPT_INTEGER_CELLS:
        AGWN_CHECK_ARG(value == 0 || value == 1, "integer cells must be 0 or 1");
        ctx->integer_cells = int(value);
        return AGWN_OK;
    case AGWN_OPT_MIXED_MIN_PAIRS:
        AGWN_CHECK_ARG(std::isfinite(value) && value >= 0.0, "mixed minimum pairs must be finite and >= 0");
        ctx->mixed_min_pairs = value;
        return AGWN_OK;
    case AGWN_OPT_MIXED_CERTIFY:
        AGWN_CHECK_ARG(value == 0 || value == 1, "mixed certify must be 0 or 1");
        ctx->mixed_certify = value != 0.0;
        return AGWN_OK;
    default:
        return fail(AGWN_ERR_INVALID, "unknown option %d", option);
    }
}

int agwn_context_get_option(agwn_context* ctx, int option, double* value)
{
    AGWN_CHECK_ARG(ctx && value, "agwn_context_get_option: null argument");
    switch (option)
    {
    case AGWN_OPT_FRAC_MODE:
        *value = ctx->frac_mode;
        return AGWN_OK;
    case AGWN_OPT_MIXED_TAU:
        *value = ctx->mixed_tau;
        return AGWN_OK;
    case AGWN_OPT_QUERIES_PER_THREAD:
        *value = ctx->queries_per_thread;
        return AGWN_OK;
    case AGWN_OPT_FRAC_BLOCK:
        *value = ctx->frac_block;
        return AGWN_OK;
    case AGWN_OPT_TIMING:
        *value = ctx->timing;
        return AGWN_OK;
    case AGWN_OPT_SEG_TILE:
        *value = ctx->seg_tile;
        return AGWN_OK;
    case AGWN_OPT_ROBUST_MODE:
        *value = ctx->robust_mode;
        return AGWN_OK;
    case AGWN_OPT_ROBUST_TERM_ERR:
        *value = ctx->robust_term_err;
        return AGWN_OK;
    case AGWN_OPT_PARAM_MODE:
        *value = ctx->param_mode;
        return AGWN_OK;
    case AGWN_OPT_MIXED_TERM_ERR:
        *value = ctx->mixed_term_err;
        return AGWN_OK;
    case AGWN_OPT_INTEGER_CELLS:
        *value = ctx->integer_cells;
        return AGWN_OK;
    case AGWN_OPT_MIXED_MIN_PAIRS:
        *value = ctx->mixed_min_pairs;
        return AGWN_OK;
    case AGWN_OPT_MIXED_CERTIFY:
        *value = ctx->mixed_certify ? 1.0 : 0.0;
        return AGWN_OK;
    default:
        return fail(AGWN_ERR_INVALID, "unknown option %d", option);
    }
}

int agwn_context_get_stats(agwn_context* ctx, agwn_stats* out, int reset)
{
    AGWN_CHECK_ARG(ctx && out, "agwn_context_get_stats: null argument");
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    AGWN_TRY(ctx->drain_timing());
    long long counters[kCounters] = {};
    AGWN_TRY_CUDA(cudaMemcpyAsync(counters, ctx->d_counters, sizeof(counters), cudaMemcpyDeviceToHost, ctx->stream));
    AGWN_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int k = 0; k < AGWN_K_COUNT; ++k)
    {
        out->kernel_ms[k] = ctx->kernel_ms[k];
        out->launches[k] = ctx->launches[k];
    }
    out->fp64_pairs = counters[0];
    out->pairs = counters[1];
    out->int_queries = counters[4];
    out->int_cell_entries = counters[5];
    out->int_leaves = counters[6];
    out->int_exact_tests = counters[7];
    out->patch_pairs = counters[8];
    out->patch_cells = counters[9];
    out->patch_pieces = counters[10];
    out->patch_fp64_pairs = counters[11];
    out->certified_pairs = counters[3];
    if (reset)
    {
        for (int k = 0; k < AGWN_K_COUNT; ++k)
        {
            ctx->kernel_ms[k] = 0;
            ctx->launches[k] = 0;
        }
        AGWN_TRY_CUDA(cudaMemsetAsync(ctx->d_counters, 0, sizeof(counters), ctx->stream));
    }
    return AGWN_OK;
}
} // extern "C"
