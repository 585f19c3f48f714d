// The persistent batch kernel: CTAs take work items (one mesh, a range of its queries) from a device queue
// (one atomicAdd per item) until it is empty, and evaluate RobustMeshGwn::eval for every query of the item:
// the integer count by the mesh's ray-frame hierarchy with the exact leaf test, the fractional term over the
// mesh's boundary staged through shared memory.  Per query the arithmetic and its order are those of the
// one-mesh kernels (robust.cuh), so the results equal agwn_robust_eval's bit for bit whatever the schedule.
// Included by batch_p64.cu / batch_p128.cu / batch_pf.cu, one policy each, to compile in parallel.
#pragma once

#include "batch.cuh"
#include "robust.cuh"
#include "tma.cuh"

namespace agwn
{
namespace
{
template <class P, int kStack>
__device__ __forceinline__ int batch_count(const BMesh& m, const Frame32& f, qv3<typename P::C> q, int* flags)
{
    using C = typename P::C;
    const C* const tri = static_cast<const C*>(m.tri);
    if (m.n_tri == 0)
        return 0;
    if (m.n_tri == 1)
        return robust_crossing<P>(q, tri);
    float const ox = float(P::cdbl(q.x)), oy = float(P::cdbl(q.y)), oz = float(P::cdbl(q.z));
    float const u = f.r[0] * ox + f.r[1] * oy + f.r[2] * oz;
    float const v = f.r[3] * ox + f.r[4] * oy + f.r[5] * oz;
    float const w = f.r[6] * ox + f.r[7] * oy + f.r[8] * oz;
    float const qmax = fmaxf(fmaxf(fabsf(ox), fabsf(oy)), fabsf(oz));
    float const tol = (qmax + m.scene_scale) * 3.8146973e-6f + 1e-30f;
    float const m8 = margin_permuted(qmax, m.scene_scale);
    int sum = 0;
    int cand[kRobCand];
    int nc = 0;
    // most leaves are decided in float on the exact -x frame, the rest by the exact predicate (as k_robust_cells)
    auto const decide = [&](int leaf) -> int
    {
        int const c = certain_leaf(m.leaf_uv, leaf, u, v, w, m8);
        return c != 2 ? c : robust_crossing<P>(q, tri + 9 * int64_t(leaf));
    };
    bool const ok = hier_walk<kStack>(m.nodes, m.leaf_uv, u, v, w, tol, m8,
                                      [&](int leaf)
                                      {
                                          if (nc == kRobCand)
                                          {
                                              for (int j = 0; j < kRobCand; ++j)
                                                  sum += decide(cand[j]);
                                              nc = 0;
                                          }
                                          cand[nc++] = leaf;
                                      });
    if (!ok)
        atomicOr(flags + FLAG_STACK, 1);
    for (int j = 0; j < nc; ++j)
        sum += decide(cand[j]);
    return sum;
}

// Mixed (int64_grid only): FP32 pairs on the mesh's vertex chains (robust_chain_step), TwoSum-accumulated; the rest
// in FP64.
template <class T, class P, int K, int kStack, bool Mixed>
__global__ void __launch_bounds__(256) k_batch(const BMesh* __restrict__ meshes, const BItem* __restrict__ items,
                                               int n_items, int* __restrict__ head, int tile, int* flags,
                                               float term_err, long long* counters)
{
    using C = typename P::C;
    using Seg = RSeg<C>;
    // the mixed form walks each mesh's vertex chains (RChain), the exact form its segments
    using Elem = std::conditional_t<Mixed, RChain, Seg>;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ int s_item;
    __shared__ int abort_cta;
    Elem* const buf[2] = {reinterpret_cast<Elem*>(smem), reinterpret_cast<Elem*>(smem) + tile};
    __shared__ uint32_t q_entries[Mixed ? 8 : 1][RQueue<K>::kCap];
    __shared__ double q_results[Mixed ? 8 : 1][32];
    int const lane = threadIdx.x & 31;
    RQueue<K> fq;
    fq.e = q_entries[Mixed ? threadIdx.x / 32 : 0];
    fq.res = q_results[Mixed ? threadIdx.x / 32 : 0];
    unsigned long long pairs = 0;
    if (threadIdx.x == 0)
    {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_barrier_init();
        abort_cta = 0;
    }
    __syncthreads();
    constexpr double f_norm = 2.0 / (4.0 * 3.141592653589793238462643383279502884);
    unsigned seq = 0; // tile loads this CTA issued before the current item: load g uses buffer g & 1, parity g >> 1
    for (;;)
    {
        if (threadIdx.x == 0)
            s_item = atomicAdd(head, 1);
        __syncthreads();
        int const item_idx = s_item;
        if (item_idx >= n_items)
        {
            if (Mixed && counters && lane == 0)
            {
                atomicAdd(reinterpret_cast<unsigned long long*>(counters), (unsigned long long)fq.tail);
                atomicAdd(reinterpret_cast<unsigned long long*>(counters + 1), pairs);
            }
            return;
        }
        BItem const item = items[item_idx];
        BMesh const& m = meshes[item.mesh];
        const Seg* const gseg = static_cast<const Seg*>(m.seg);
        int64_t const n_seg = m.n_seg;
        const Elem* const gel = static_cast<const Elem*>(Mixed ? m.chain : m.seg);
        int64_t const n_elem = Mixed ? m.n_entries : n_seg;
        const T* const pos = static_cast<const T*>(m.pos);
        T* const out = static_cast<T*>(m.out);
        Quant const qz{{m.qc[0], m.qc[1], m.qc[2]}, m.qs};
        Frame32 f;
#pragma unroll
        for (int k = 0; k < 9; ++k)
            f.r[k] = m.frame[k];
        int const n_tiles = n_elem > 0 ? int((n_elem + tile - 1) / tile) : 0;
        bool const single = n_tiles == 1;
        int64_t const per_sub = int64_t(blockDim.x) * K;
        int const n_sub = int((item.q1 - item.q0 + per_sub - 1) / per_sub);
        int const total = n_tiles == 0 ? 0 : (single ? 1 : n_sub * n_tiles);
        auto issue = [&](int it)
        {
            unsigned const g = seq + unsigned(it);
            int const b = int(g & 1u);
            int const st = it % n_tiles;
            int64_t const rem = n_elem - int64_t(st) * tile;
            unsigned const bytes = unsigned(rem < tile ? rem : tile) * unsigned(sizeof(Elem));
            mbar_arrive_expect_tx(&bars[b], bytes);
            bulk_copy_g2s(buf[b], gel + int64_t(st) * tile, bytes, &bars[b]);
        };
        if (threadIdx.x == 0)
        {
            if (total > 0)
                issue(0);
            if (total > 1)
                issue(1);
        }
        int it = 0;
        for (int sub = 0; sub < n_sub; ++sub)
        {
            qv3<C> q[K];
            int cnt[K];
            double half[K];
            using LV = typename RLanes<K>::V;
            LV acc[RLanes<K>::NP], comp[RLanes<K>::NP];
            int64_t idx[K];
            RVState<LV> st0[RLanes<K>::NP] = {}, st1[RLanes<K>::NP] = {};
#pragma unroll
            for (int p = 0; p < RLanes<K>::NP; ++p)
                acc[p] = comp[p] = lv_set<LV>(0.f);
#pragma unroll
            for (int k = 0; k < K; ++k)
            {
                idx[k] = item.q0 + sub * per_sub + int64_t(k) * blockDim.x + threadIdx.x;
                int64_t const ii = idx[k] < item.q1 ? idx[k] : item.q1 - 1;
                q[k] = quantize<P>(double(pos[3 * ii]), double(pos[3 * ii + 1]), double(pos[3 * ii + 2]), qz);
                cnt[k] = batch_count<P, kStack>(m, f, q[k], flags);
                half[k] = 0.0;
            }
            for (int st = 0; st < n_tiles; ++st)
            {
                unsigned const g = seq + unsigned(it);
                int const b = int(g & 1u);
                // a single tile stays in shared memory for all of the item's query sub-tiles: only the first waits for
                // it, and the warps then run the others without meeting at a barrier
                bool const landed = !single || sub == 0;
                if (landed)
                {
                    if (!mbar_wait_bounded(&bars[b], (g >> 1) & 1u, flags, 5))
                        abort_cta = 1;
                    __syncthreads();
                    if (abort_cta)
                        return;
                }
                Elem const* const sb = buf[b];
                int64_t const rem = n_elem - int64_t(st) * tile;
                int const cnt_s = int(rem < tile ? rem : tile);
                if constexpr (Mixed)
                {
                    // tiles start at even stream positions (the tile is even): the state alternation runs across them
                    for (int s = 0; s < cnt_s; s += 2)
                        robust_chain_step<P, K>(sb, s, cnt_s - s < 2 ? cnt_s - s : 2, q, st0, st1, term_err, acc, comp,
                                                fq, lane, gseg, half);
                }
                else
                {
                    for (int s = 0; s < cnt_s; ++s)
                    {
                        Seg const sgm = sb[s];
#pragma unroll
                        for (int k = 0; k < K; ++k)
                            half[k] = __dadd_rn(half[k], __dmul_rn(sgm.w, robust_contrib<P>(q[k], sgm)));
                    }
                }
                if (!single)
                {
                    __syncthreads(); // buffer b is free again
                    if (threadIdx.x == 0 && it + 2 < total)
                        issue(it + 2);
                    ++it;
                }
            }
            if constexpr (Mixed)
            {
                while (fq.tail != fq.head)
                    rq_flush<P, K>(fq, min(32u, fq.tail - fq.head), lane, gseg, q, half);
                pairs += 32ull * K * (unsigned long long)n_seg;
            }
#pragma unroll
            for (int k = 0; k < K; ++k)
                if (idx[k] < item.q1)
                {
                    if constexpr (Mixed)
                        half[k] = __dadd_rn(half[k], __dadd_rn(double(ln(acc[k / RLanes<K>::W], k % RLanes<K>::W)),
                                                               double(ln(comp[k / RLanes<K>::W], k % RLanes<K>::W))));
                    T const fr = T(__dmul_rn(half[k], f_norm));
                    out[idx[k]] = fr + T(cnt[k]);
                    if (m.counts)
                        m.counts[idx[k]] = cnt[k];
                }
        }
        seq += unsigned(total);
        __syncthreads(); // s_item and the buffers are free for the next item
    }
}

template <class T, class P>
using BatchKernel = void (*)(const BMesh*, const BItem*, int, int*, int, int*, float, long long*);

template <class T, class P>
BatchKernel<T, P> pick_batch_kernel(const BConf& c, bool mixed)
{
    if constexpr (std::is_same_v<P, P64>)
        if (mixed)
        {
            if (c.k == 1)
                return c.stack <= 32 ? k_batch<T, P, 1, 32, true> : k_batch<T, P, 1, 64, true>;
            return c.stack <= 32 ? k_batch<T, P, 2, 32, true> : k_batch<T, P, 2, 64, true>;
        }
    if (c.k == 1)
        return c.stack <= 32 ? k_batch<T, P, 1, 32, false> : k_batch<T, P, 1, 64, false>;
    return c.stack <= 32 ? k_batch<T, P, 2, 32, false> : k_batch<T, P, 2, 64, false>;
}

template <class T, class P>
int batch_occupancy_t(const BConf& c, bool mixed, size_t smem, int* per_sm)
{
    auto const kern = pick_batch_kernel<T, P>(c, mixed);
    AGWN_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    AGWN_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, kern, c.block, smem));
    return AGWN_OK;
}

template <class T, class P>
int batch_launch_t(cudaStream_t st, const BConf& c, bool mixed, float term_err, int grid, size_t smem,
                   const BMesh* meshes, const BItem* items, int n_items, int* head, int* flags, long long* counters)
{
    auto const kern = pick_batch_kernel<T, P>(c, mixed);
    kern<<<grid, c.block, smem, st>>>(meshes, items, n_items, head, c.seg_tile, flags, term_err, counters);
    AGWN_TRY_CUDA(cudaGetLastError());
    return AGWN_OK;
}

template <class P>
struct BatchOpsFor
{
    static int occupancy(int scalar_bytes, const BConf& c, bool mixed, size_t smem, int* per_sm)
    {
        return scalar_bytes == 4 ? batch_occupancy_t<float, P>(c, mixed, smem, per_sm)
                                 : batch_occupancy_t<double, P>(c, mixed, smem, per_sm);
    }
    static int launch(int scalar_bytes, cudaStream_t st, const BConf& c, bool mixed, float term_err, int grid,
                      size_t smem, const BMesh* meshes, const BItem* items, int n_items, int* head, int* flags,
                      long long* counters)
    {
        return scalar_bytes == 4 ? batch_launch_t<float, P>(st, c, mixed, term_err, grid, smem, meshes, items,
                                                            n_items, head, flags, counters)
                                 : batch_launch_t<double, P>(st, c, mixed, term_err, grid, smem, meshes, items,
                                                             n_items, head, flags, counters);
    }
};
} // namespace
} // namespace agwn
