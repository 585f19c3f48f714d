// Stable LSD radix sort, 8 bits per pass, of (key, value) pairs: a per-block digit histogram, one exclusive scan of
// all (digit, block) counters, then a scatter that keeps each block's order (ranks within a warp from
// __match_any_sync, across warps from per-warp counts).  Used for the hierarchy's Morton codes (32-bit keys) and
// the boundary's edge keys (64-bit).
#pragma once

#include "agwn_internal.cuh"

namespace agwn
{
namespace
{
// ---- stable LSD radix sort, 8 bits per pass -----------------------------------------------------------------
constexpr int kRsBlock = 256;
constexpr int kRsIpt = 8;
constexpr int kRsTile = kRsBlock * kRsIpt;

template <class K>
__global__ void __launch_bounds__(kRsBlock) k_rs_hist(const K* __restrict__ keys, int64_t n, int shift,
                                                      unsigned* __restrict__ hist, int n_blocks)
{
    __shared__ unsigned cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    int64_t const base = int64_t(blockIdx.x) * kRsTile;
    for (int r = 0; r < kRsIpt; ++r)
    {
        int64_t const i = base + r * kRsBlock + threadIdx.x;
        if (i < n)
            atomicAdd(&cnt[unsigned(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[int64_t(threadIdx.x) * n_blocks + blockIdx.x] = cnt[threadIdx.x];
}

// Exclusive scan of m counters in one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_rs_scan(unsigned* __restrict__ hist, int64_t m)
{
    __shared__ unsigned part[1024];
    int64_t const per = (m + 1023) / 1024;
    int64_t const b = per * threadIdx.x;
    int64_t const e = min(b + per, m);
    unsigned s = 0;
    for (int64_t i = b; i < e; ++i)
        s += hist[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1)
    {
        unsigned const v = threadIdx.x >= unsigned(o) ? part[threadIdx.x - o] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
    for (int64_t i = b; i < e; ++i)
    {
        unsigned const v = hist[i];
        hist[i] = run;
        run += v;
    }
}

// The same exclusive scan in three parallel steps, for many counters (a sort pass's digit counters over millions of
// keys, a cell grid's offsets): block sums of 4,096 counters, one block scanning those sums (1,024 at a time, with a
// carry), and each block scanning its counters from its offset.  scan_counters launches the three; sums:
// scan_sums_count(m) unsigned of scratch.
constexpr int kScanCnt = 4096; // counters per block: 1,024 threads x 4

__device__ __forceinline__ unsigned block_exclusive(unsigned v, unsigned* warp_tot, unsigned* total)
{
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned x = v;
    for (int o = 1; o < 32; o <<= 1)
    {
        unsigned const y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o)
            x += y;
    }
    if (lane == 31)
        warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0)
    {
        unsigned w = warp_tot[lane];
        unsigned z = w;
        for (int o = 1; o < 32; o <<= 1)
        {
            unsigned const y = __shfl_up_sync(0xffffffffu, z, o);
            if (lane >= o)
                z += y;
        }
        warp_tot[lane] = z - w; // exclusive offsets of the warps
        if (lane == 31)
            *total = z;
    }
    __syncthreads();
    unsigned const r = warp_tot[warp] + x - v;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(1024) k_cnt_sums(const unsigned* __restrict__ c, int64_t m,
                                                   unsigned* __restrict__ sums)
{
    __shared__ unsigned wt[32];
    __shared__ unsigned tot;
    int64_t const i0 = int64_t(blockIdx.x) * kScanCnt + 4 * threadIdx.x;
    unsigned v = 0;
    for (int k = 0; k < 4; ++k)
        v += i0 + k < m ? c[i0 + k] : 0u;
    block_exclusive(v, wt, &tot);
    if (threadIdx.x == 0)
        sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) k_cnt_top(unsigned* __restrict__ sums, int nb)
{
    __shared__ unsigned wt[32];
    __shared__ unsigned tot;
    unsigned carry = 0;
    for (int b0 = 0; b0 < nb; b0 += 1024)
    {
        int const b = b0 + int(threadIdx.x);
        unsigned const v = b < nb ? sums[b] : 0u;
        unsigned const e = block_exclusive(v, wt, &tot);
        if (b < nb)
            sums[b] = carry + e;
        carry += tot;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(1024) k_cnt_apply(unsigned* __restrict__ c, int64_t m,
                                                    const unsigned* __restrict__ sums)
{
    __shared__ unsigned wt[32];
    __shared__ unsigned tot;
    int64_t const i0 = int64_t(blockIdx.x) * kScanCnt + 4 * threadIdx.x;
    unsigned v[4];
    unsigned t = 0;
    for (int k = 0; k < 4; ++k)
    {
        v[k] = i0 + k < m ? c[i0 + k] : 0u;
        t += v[k];
    }
    unsigned run = sums[blockIdx.x] + block_exclusive(t, wt, &tot);
    for (int k = 0; k < 4; ++k)
        if (i0 + k < m)
        {
            c[i0 + k] = run;
            run += v[k];
        }
}

inline int64_t scan_sums_count(int64_t m)
{
    return (m + kScanCnt - 1) / kScanCnt;
}

inline void scan_counters(cudaStream_t st, unsigned* c, int64_t m, unsigned* sums)
{
    int const nb = int(scan_sums_count(m));
    if (nb == 0)
        return;
    k_cnt_sums<<<nb, 1024, 0, st>>>(c, m, sums);
    k_cnt_top<<<1, 1024, 0, st>>>(sums, nb);
    k_cnt_apply<<<nb, 1024, 0, st>>>(c, m, sums);
}

template <class K, class V>
__global__ void __launch_bounds__(kRsBlock) k_rs_scatter(const K* __restrict__ kin, const V* __restrict__ vin,
                                                         int64_t n, int shift, const unsigned* __restrict__ hist,
                                                         int n_blocks, K* __restrict__ kout, V* __restrict__ vout)
{
    constexpr int W = kRsBlock / 32;
    __shared__ unsigned base[256];
    __shared__ unsigned wcnt[W][256];
    base[threadIdx.x] = hist[int64_t(threadIdx.x) * n_blocks + blockIdx.x];
    for (int w = 0; w < W; ++w)
        wcnt[w][threadIdx.x] = 0;
    __syncthreads();
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned const lt = (1u << lane) - 1u;
    int64_t const tile0 = int64_t(blockIdx.x) * kRsTile;
    for (int r = 0; r < kRsIpt; ++r)
    {
        int64_t const i = tile0 + r * kRsBlock + threadIdx.x;
        bool const valid = i < n;
        K const key = valid ? kin[i] : K(0);
        V const val = valid ? vin[i] : V(0);
        unsigned const d = valid ? (unsigned(key >> shift) & 255u) : 256u;
        unsigned const peers = __match_any_sync(0xffffffffu, d);
        unsigned const rank = __popc(peers & lt);
        bool const leader = (peers & lt) == 0;
        if (valid && leader)
            wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid)
        {
            unsigned pos = base[d] + rank;
            for (int w = 0; w < warp; ++w)
                pos += wcnt[w][d];
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
        if (valid && leader)
        {
            atomicAdd(&base[d], unsigned(__popc(peers))); // several warps may hold the same digit
            wcnt[warp][d] = 0;
        }
        __syncthreads();
    }
}
} // namespace
} // namespace agwn
