// Batched robust evaluation of many meshes in one persistent launch (no reference counterpart: the reference
// evaluates one mesh per eval_gwnr_mesh_batch_robust call, src/antipodal/gwn_mesh_robust.hh:441-456).
// Shared declarations of the batch engine (batch.cu) and its per-policy kernel files (batch_p*.cu).
#pragma once

#include "agwn_internal.cuh"
#include "hier.cuh"

namespace agwn
{
// One mesh of a batch, as the kernel reads it (device-resident table).  The geometry pointers are the robust
// evaluator's own buffers; positions / out / counts are the caller's device arrays for this mesh.
struct BMesh
{
    const BvhNode* nodes;
    const void* tri; // predicate triangles in leaf order (P::C[9] each)
    const float4* leaf_uv;
    const void* seg;   // RSeg<P::C>
    const void* chain; // int64_grid: RChain, the vertex chains of the mixed form (nullable)
    int64_t n_entries;
    const void* pos; // n_q * 3 scalars
    void* out;       // n_q scalars
    int32_t* counts; // n_q (nullable)
    int64_t n_tri, n_seg, n_q;
    double qc[3], qs; // quantisation centre and scale
    float frame[9];
    float scene_scale;
};

// A work item: queries [q0, q1) of one mesh against all of that mesh's boundary segments and triangles.
struct BItem
{
    int32_t mesh;
    int32_t pad;
    int64_t q0, q1;
};

// Launch configuration chosen by the autotuner.
struct BConf
{
    int block;    // threads per CTA: 128 or 256
    int k;        // queries per thread: 1 or 2
    int seg_tile; // boundary segments per shared-memory tile
    int stack;    // traversal stack entries: 32 or 64
};

// Per-policy operations, defined in batch_p64.cu (int64_grid), batch_p128.cu (int128_grid) and batch_pf.cu
// (exact_float).  scalar_bytes: 4 or 8.  The queue head must be zero when the kernel starts.
// mixed selects the FP32-pair form (int64_grid only; ignored by the other policies).
struct BatchPolicyOps
{
    size_t seg_bytes; // one boundary segment in shared memory
    bool has_mixed;   // the policy has an FP32-pair form
    int (*occupancy)(int scalar_bytes, const BConf& c, bool mixed, size_t smem, int* per_sm);
    int (*launch)(int scalar_bytes, cudaStream_t st, const BConf& c, bool mixed, float term_err, int grid, size_t smem,
                  const BMesh* meshes, const BItem* items, int n_items, int* head, int* flags, long long* counters);
};
extern const BatchPolicyOps kBatchP64, kBatchP128, kBatchPF;
} // namespace agwn
