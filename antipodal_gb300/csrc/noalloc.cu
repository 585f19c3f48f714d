// Mixed-precision fractional GWN for callers that cannot allocate device memory.
//
// Some programs that would call this library own every byte of device memory themselves: an application or
// engine that hands all of the GPU to its own pool allocator and fixes its memory budget up front, or a plugin
// running inside a framework whose caching allocator must not be bypassed.  For them a cudaMalloc inside a
// library call is not allowed -- it can fail against the budget, fragment the owner's pool, or stall the device
// at a moment the caller does not control.  The regular entry points keep their scratch buffers in a context
// (agwn_context_create allocates), so they cannot be used there.
//
// agwn_mesh_batch_fractional_mixed_noalloc_f64 runs the same two kernels as agwn_mesh_batch_fractional_f64 in
// the mixed mode, but its scratch -- the prepared boundary, the frame and the error flags -- lives in one
// file-scope static __device__ array of fixed size (kNoAllocMaxSegments segments, 1,409,120 bytes), created when
// the library is loaded and held by every GPU that loads it until the process exits.  The caller passes the
// inputs and the output in memory it already owns.  Nothing here calls cudaMalloc, cudaFree or any other
// allocating routine.

#include "agwn_internal.cuh"
#include "frac_kernels.cuh"

#include <mutex>

namespace agwn
{
namespace
{
constexpr int64_t kNoAllocMaxSegments = 8192;
constexpr int kNoAllocK = 4;
constexpr int kNoAllocBlock = 256;
constexpr int kNoAllocTile = 512;
constexpr int kMaxDevices = 64;

struct NoAllocScratch
{
    SegM seg[2 * kNoAllocMaxSegments]; // the boundary entry stream: at most two entries per segment
    int order[chain_scratch_ints(kChainMax)];
    SegX<double> seg64[kNoAllocMaxSegments];
    Frame frame;
    int flags[FLAG_COUNT];
    long long counters[4];
};
// The size the header states; a change of the layout must update it there as well.
constexpr size_t kNoAllocScratchBytes = 1409120;
static_assert(sizeof(NoAllocScratch) == kNoAllocScratchBytes, "update the scratch size stated in antipodal_gb300.h");

// The scratch array.  Host code must not pass this symbol to a kernel: on the host it names a stand-in object,
// not device memory.  Its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

bool on_device(const void* p, int device)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
    {
        cudaGetLastError();
        return false;
    }
    return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) && a.device == device;
}

std::mutex g_noalloc_mutex;
NoAllocScratch* g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up with that device current on the first call
// there.  A cached address that no longer lies in this device's memory (the library's module was loaded again,
// e.g. after cudaDeviceReset) is looked up again.
int noalloc_scratch(int device, NoAllocScratch** out)
{
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device] || !on_device(g_noalloc_ptr[device], device))
    {
        void* p = nullptr;
        cudaError_t const e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
        {
            cudaGetLastError();
            return fail(AGWN_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed on device %d: %s", device,
                        cudaGetErrorString(e));
        }
        g_noalloc_ptr[device] = static_cast<NoAllocScratch*>(p);
    }
    *out = g_noalloc_ptr[device];
    return AGWN_OK;
}
} // namespace
} // namespace agwn

using namespace agwn;

extern "C" int agwn_mesh_batch_fractional_mixed_noalloc_f64(void* stream, const double* positions, int64_t n,
                                                            double* out, const double* x0, const double* boundary,
                                                            int64_t n_segments)
{
    clear_message();
    AGWN_CHECK_ARG(n >= 0 && n_segments >= 0, "negative size");
    AGWN_CHECK_ARG(n_segments <= kNoAllocMaxSegments,
                   "%lld boundary segments exceed this entry point's fixed scratch of %lld segments; use "
                   "agwn_mesh_batch_fractional_f64 (which allocates) for larger boundaries",
                   (long long)n_segments, (long long)kNoAllocMaxSegments);
    AGWN_CHECK_ARG(x0 != nullptr, "null x0");
    if (n == 0)
        return AGWN_OK;
    int device = 0;
    AGWN_TRY_CUDA(cudaGetDevice(&device));
    AGWN_CHECK_ARG(device >= 0 && device < kMaxDevices, "device ordinal %d not supported", device);
    AGWN_CHECK_ARG(positions && out && on_device(positions, device) && on_device(out, device),
                   "positions and out must be device memory of the current device %d", device);
    AGWN_CHECK_ARG(n_segments == 0 || (boundary && on_device(boundary, device)),
                   "boundary must be device memory of the current device %d", device);
    double const x0n = x0[0] * x0[0] + x0[1] * x0[1] + x0[2] * x0[2];
    AGWN_CHECK_ARG(x0n > 0 && std::isfinite(x0n), "x0 must be finite and nonzero");

    NoAllocScratch* scr = nullptr;
    AGWN_TRY(noalloc_scratch(device, &scr));
    cudaStream_t const st = static_cast<cudaStream_t>(stream);
    // the array keeps the previous call's contents: the flags must start at zero, the rest is rewritten below
    AGWN_TRY_CUDA(cudaMemsetAsync(scr->flags, 0, sizeof(scr->flags), st));

    int sm_count = 0;
    AGWN_TRY_CUDA(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device));
    if (n_segments == 0)
    {
        k_fill_counts<double><<<std::min<int64_t>(div_up(n, 256), 4 * sm_count), 256, 0, st>>>(out, nullptr, n);
        AGWN_TRY_CUDA(cudaGetLastError());
        AGWN_TRY_CUDA(cudaStreamSynchronize(st));
        return AGWN_OK;
    }
    Context defaults; // option defaults only (no resources)
    Rot const rot = make_rotation(x0);
    k_prep_mixed<<<1, 1024, 0, st>>>(boundary, n_segments, rot, float(defaults.mixed_tau), &scr->frame, scr->seg,
                                     scr->seg64, scr->order);
    AGWN_TRY_CUDA(cudaGetLastError());

    int64_t const max_entries = 2 * n_segments;
    int const tile = int(std::min<int64_t>(kNoAllocTile, max_entries));
    int const n_tiles = int((max_entries + tile - 1) / tile);
    size_t const smem = size_t(n_tiles == 1 ? 1 : 2) * tile * sizeof(SegM);
    auto kern = k_frac_mixed<kNoAllocK, MeshFallback>;
    AGWN_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int per_sm = 0;
    AGWN_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kNoAllocBlock, smem));
    AGWN_CHECK_ARG(per_sm > 0, "fractional kernel does not fit on an SM");
    int64_t const per_tile = int64_t(kNoAllocBlock) * kNoAllocK;
    int64_t const n_qtiles = (n + per_tile - 1) / per_tile;
    int const grid = int(std::max<int64_t>(1, std::min<int64_t>(n_qtiles, int64_t(per_sm) * sm_count)));
    kern<<<grid, kNoAllocBlock, smem, st>>>(positions, n, out, nullptr, x0[0], x0[1], x0[2], rot, &scr->frame,
                                            int(defaults.mixed_certify), float(defaults.mixed_term_err), scr->seg,
                                            MeshFallback{scr->seg64}, n_segments, tile, scr->flags, scr->counters, 0);
    AGWN_TRY_CUDA(cudaGetLastError());
    AGWN_TRY_CUDA(cudaStreamSynchronize(st));
    int flags[FLAG_COUNT] = {};
    AGWN_TRY_CUDA(cudaMemcpy(flags, scr->flags, sizeof(flags), cudaMemcpyDeviceToHost));
    if (flags[FLAG_TIMEOUT])
        return fail(AGWN_ERR_TIMEOUT, "a bounded device wait ran out (code %d); the output is not valid",
                    flags[FLAG_TIMEOUT]);
    return AGWN_OK;
}
