// Open boundary of a triangle mesh on the device: build_boundary_segments (src/antipodal/math/common.hh:123-174).
// Every triangle edge u -> v adds +1 (u < v) or -1 (u >= v) to its undirected edge {min, max}; edges whose net count
// is not zero are emitted as weighted segments, directed lo -> hi when the count is positive and hi -> lo otherwise,
// with weight |count|.  The reference accumulates in a hash map and emits in the map's order; here the edges are
// sorted by (lo, hi) -- 64-bit keys, LSD radix sort over only the bits the vertex count needs -- reduced by key and
// compacted with a scan, so the output is in ascending (lo, hi) order, deterministically.

#include "agwn_internal.cuh"
#include "radix.cuh"

#include <algorithm>

namespace agwn
{
namespace
{
constexpr int kScanBlock = 1024;

__global__ void k_edge_keys(const int32_t* __restrict__ idx, int64_t n_tri, int64_t nv,
                            unsigned long long* __restrict__ keys, int* __restrict__ vals, int* flags)
{
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < 3 * n_tri;
         i += int64_t(gridDim.x) * blockDim.x)
    {
        int64_t const t = i / 3;
        int const e = int(i - 3 * t);
        int32_t const u = idx[3 * t + e], v = idx[3 * t + (e + 1) % 3];
        if (u < 0 || v < 0 || u >= nv || v >= nv)
        {
            atomicOr(flags + FLAG_COUNT - 1, 1); // the invalid-index slot, as in the hierarchy build
            keys[i] = 0ull;
            vals[i] = 0;
            continue;
        }
        unsigned long long const lo = unsigned(min(u, v)), hi = unsigned(max(u, v));
        keys[i] = (lo << 32) | hi;
        vals[i] = u < v ? 1 : -1;
    }
}

// Net count of each run of equal keys, at the run's first element (0 elsewhere), and whether it is emitted.
__global__ void k_edge_reduce(const unsigned long long* __restrict__ keys, const int* __restrict__ vals, int64_t m,
                              int* __restrict__ net, unsigned* __restrict__ emit)
{
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < m; i += int64_t(gridDim.x) * blockDim.x)
    {
        bool const head = i == 0 || keys[i] != keys[i - 1];
        int s = 0;
        if (head)
            for (int64_t j = i; j < m && keys[j] == keys[i]; ++j)
                s += vals[j];
        net[i] = s;
        emit[i] = head && s != 0 ? 1u : 0u;
    }
}

// Exclusive scan, phase 1: each block of kScanBlock flags -> its sum.
__global__ void __launch_bounds__(kScanBlock) k_scan_sums(const unsigned* __restrict__ f, int64_t m,
                                                          unsigned* __restrict__ sums)
{
    __shared__ unsigned part[kScanBlock / 32];
    int64_t const i = int64_t(blockIdx.x) * kScanBlock + threadIdx.x;
    unsigned v = i < m ? f[i] : 0u;
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0)
        part[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32)
    {
        unsigned w = part[threadIdx.x];
        for (int o = 16; o > 0; o >>= 1)
            w += __shfl_down_sync(0xffffffffu, w, o);
        if (threadIdx.x == 0)
            sums[blockIdx.x] = w;
    }
}

// Phase 3: positions = block offset (phase 2 scanned the sums) + exclusive scan within the block.
__global__ void __launch_bounds__(kScanBlock) k_scan_apply(const unsigned* __restrict__ f, int64_t m,
                                                           const unsigned* __restrict__ offs, unsigned* __restrict__ pos)
{
    __shared__ unsigned wsum[kScanBlock / 32];
    int64_t const i = int64_t(blockIdx.x) * kScanBlock + threadIdx.x;
    unsigned const v = i < m ? f[i] : 0u;
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned x = v; // inclusive within the warp
    for (int o = 1; o < 32; o <<= 1)
    {
        unsigned const y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o)
            x += y;
    }
    if (lane == 31)
        wsum[warp] = x;
    __syncthreads();
    if (warp == 0)
    {
        unsigned w = wsum[lane];
        for (int o = 1; o < 32; o <<= 1)
        {
            unsigned const y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o)
                w += y;
        }
        wsum[lane] = w; // inclusive over warps
    }
    __syncthreads();
    unsigned const before = warp ? wsum[warp - 1] : 0u;
    if (i < m)
        pos[i] = offs[blockIdx.x] + before + x - v;
}

template <class T>
__global__ void k_edge_emit(const unsigned long long* __restrict__ keys, const int* __restrict__ net,
                            const unsigned* __restrict__ emit, const unsigned* __restrict__ pos, int64_t m,
                            const T* __restrict__ verts, T* __restrict__ out)
{
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < m; i += int64_t(gridDim.x) * blockDim.x)
    {
        if (!emit[i])
            continue;
        int64_t const lo = int64_t(keys[i] >> 32), hi = int64_t(keys[i] & 0xffffffffull);
        int const s = net[i];
        int64_t const a = s > 0 ? lo : hi, b = s > 0 ? hi : lo;
        T* const o = out + 7 * int64_t(pos[i]);
        for (int k = 0; k < 3; ++k)
        {
            o[k] = verts[3 * a + k];
            o[3 + k] = verts[3 * b + k];
        }
        o[6] = T(s > 0 ? s : -s);
    }
}

struct Buf
{
    void* p = nullptr;
    ~Buf()
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
    template <class X>
    X* as() const
    {
        return static_cast<X*>(p);
    }
};

template <class T>
int boundary_build(agwn_context* ctx, const T* vertices, int64_t nv, const int32_t* indices, int64_t n_idx, T* out,
                   int64_t capacity, int64_t* n_segments)
{
    AGWN_CHECK_ARG(ctx && n_segments, "null context/count");
    AGWN_CHECK_ARG(nv >= 0 && n_idx >= 0 && n_idx % 3 == 0 && capacity >= 0, "bad sizes");
    AGWN_CHECK_ARG(n_idx == 0 || (vertices && indices), "null geometry");
    AGWN_CHECK_ARG(nv <= (int64_t(1) << 31) && n_idx / 3 < (int64_t(1) << 31), "mesh too large");
    clear_message();
    AGWN_TRY_CUDA(cudaSetDevice(ctx->device));
    *n_segments = 0;
    int64_t const m = n_idx; // one entry per triangle edge
    if (m == 0)
        return AGWN_OK;
    cudaStream_t const st = ctx->stream;
    const void *dv = nullptr, *di = nullptr;
    AGWN_TRY(stage_in(*ctx, vertices, sizeof(T) * 3 * nv, S_MISC0, &dv));
    AGWN_TRY(stage_in(*ctx, indices, sizeof(int32_t) * n_idx, S_MISC1, &di));
    int const n_rs_blocks = int((m + kRsTile - 1) / kRsTile);
    int64_t const n_sb = (m + kScanBlock - 1) / kScanBlock;
    Buf ka, kb, va, vb, hist, net, emit, pos, sums;
    AGWN_TRY(ka.alloc(sizeof(unsigned long long) * m));
    AGWN_TRY(kb.alloc(sizeof(unsigned long long) * m));
    AGWN_TRY(va.alloc(sizeof(int) * m));
    AGWN_TRY(vb.alloc(sizeof(int) * m));
    AGWN_TRY(hist.alloc(sizeof(unsigned) * 256 * size_t(n_rs_blocks)));
    Buf hsum;
    AGWN_TRY(hsum.alloc(sizeof(unsigned) * size_t(scan_sums_count(int64_t(256) * n_rs_blocks))));
    AGWN_TRY(net.alloc(sizeof(int) * m));
    AGWN_TRY(emit.alloc(sizeof(unsigned) * m));
    AGWN_TRY(pos.alloc(sizeof(unsigned) * m));
    AGWN_TRY(sums.alloc(sizeof(unsigned) * size_t(n_sb)));
    int const grid = int(std::min<int64_t>(div_up(m, 256), 8 * ctx->sm_count));
    AGWN_TRY_CUDA(cudaMemsetAsync(ctx->d_flags + FLAG_COUNT - 1, 0, sizeof(int), st));
    AGWN_TRY(ctx->launch_begin(AGWN_K_OTHER));
    k_edge_keys<<<grid, 256, 0, st>>>(static_cast<const int32_t*>(di), m / 3, nv, ka.as<unsigned long long>(),
                                      va.as<int>(), ctx->d_flags);
    // radix passes over the bits that can be set: the low `bits` of each 32-bit half
    int bits = 1;
    while ((int64_t(1) << bits) < nv)
        ++bits;
    unsigned long long *kin = ka.as<unsigned long long>(), *kout = kb.as<unsigned long long>();
    int *vin = va.as<int>(), *vout = vb.as<int>();
    for (int half = 0; half < 2; ++half)
        for (int sh = 0; sh < bits; sh += 8)
        {
            int const shift = 32 * half + sh;
            k_rs_hist<unsigned long long><<<n_rs_blocks, kRsBlock, 0, st>>>(kin, m, shift, hist.as<unsigned>(),
                                                                            n_rs_blocks);
            scan_counters(st, hist.as<unsigned>(), int64_t(256) * n_rs_blocks, hsum.as<unsigned>());
            k_rs_scatter<unsigned long long, int><<<n_rs_blocks, kRsBlock, 0, st>>>(
                kin, vin, m, shift, hist.as<unsigned>(), n_rs_blocks, kout, vout);
            std::swap(kin, kout);
            std::swap(vin, vout);
        }
    k_edge_reduce<<<grid, 256, 0, st>>>(kin, vin, m, net.as<int>(), emit.as<unsigned>());
    k_scan_sums<<<int(n_sb), kScanBlock, 0, st>>>(emit.as<unsigned>(), m, sums.as<unsigned>());
    // the block sums become block offsets; keep the total in a copy of the last sum
    unsigned last_sum = 0, last_off = 0;
    AGWN_TRY_CUDA(cudaMemcpyAsync(&last_sum, sums.as<unsigned>() + n_sb - 1, sizeof(unsigned), cudaMemcpyDeviceToHost,
                                  st));
    k_rs_scan<<<1, 1024, 0, st>>>(sums.as<unsigned>(), n_sb);
    AGWN_TRY_CUDA(cudaMemcpyAsync(&last_off, sums.as<unsigned>() + n_sb - 1, sizeof(unsigned), cudaMemcpyDeviceToHost,
                                  st));
    k_scan_apply<<<int(n_sb), kScanBlock, 0, st>>>(emit.as<unsigned>(), m, sums.as<unsigned>(), pos.as<unsigned>());
    AGWN_TRY(ctx->launch_end(AGWN_K_OTHER));
    int bad = 0;
    AGWN_TRY_CUDA(cudaMemcpyAsync(&bad, ctx->d_flags + FLAG_COUNT - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    AGWN_TRY_CUDA(cudaStreamSynchronize(st));
    if (bad)
    {
        AGWN_TRY_CUDA(cudaMemsetAsync(ctx->d_flags + FLAG_COUNT - 1, 0, sizeof(int), st));
        return fail(AGWN_ERR_INVALID, "triangle index out of range [0, %lld)", (long long)nv);
    }
    int64_t const count = int64_t(last_off) + int64_t(last_sum);
    *n_segments = count;
    if (!out || count == 0)
        return AGWN_OK;
    // all rows go to device scratch, then the first `capacity` of them to the caller
    void* dseg = nullptr;
    AGWN_TRY(ctx->scratch_reserve(S_MISC2, sizeof(T) * 7 * size_t(count), &dseg));
    AGWN_TRY(ctx->launch_begin(AGWN_K_OTHER));
    k_edge_emit<T><<<grid, 256, 0, st>>>(kin, net.as<int>(), emit.as<unsigned>(), pos.as<unsigned>(), m,
                                         static_cast<const T*>(dv), static_cast<T*>(dseg));
    AGWN_TRY(ctx->launch_end(AGWN_K_OTHER));
    int64_t const rows = std::min(count, capacity);
    if (rows > 0)
        AGWN_TRY_CUDA(cudaMemcpyAsync(out, dseg, sizeof(T) * 7 * size_t(rows), cudaMemcpyDefault, st));
    return ctx->check_flags();
}
} // namespace
} // namespace agwn

using namespace agwn;

extern "C" int agwn_build_boundary_segments_f64(agwn_context* ctx, const double* vertices, int64_t n_vertices,
                                                const int32_t* indices, int64_t n_indices, double* out,
                                                int64_t capacity, int64_t* n_segments)
{
    return boundary_build<double>(ctx, vertices, n_vertices, indices, n_indices, out, capacity, n_segments);
}
extern "C" int agwn_build_boundary_segments_f32(agwn_context* ctx, const float* vertices, int64_t n_vertices,
                                                const int32_t* indices, int64_t n_indices, float* out,
                                                int64_t capacity, int64_t* n_segments)
{
    return boundary_build<float>(ctx, vertices, n_vertices, indices, n_indices, out, capacity, n_segments);
}
