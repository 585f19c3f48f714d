// The robust evaluator's handle (agwn_robust): its geometry on the device, as robust.cu builds it and batch.cu
// reads it.
#pragma once

#include "agwn_internal.cuh"

namespace agwn
{
// The int64_grid boundary as vertex chains for the FP32 pairs (k_robust_chain, robust.cuh): per chain a start
// entry (s = -1: the first segment's p0) and then one entry per segment (s: its index in the RSeg array; p: its p1;
// w: its weight), in the order the pairs are summed.  Segment t follows s when RSeg[t].p0 == RSeg[s].p1.
struct alignas(16) RChain
{
    int32_t p[3];
    int32_t s;
    float w;
    int32_t pad[3];
};

struct Robust
{
    int device = 0;
    int scalar_bytes = 8;
    int policy = 0;
    int64_t n_tri = 0;
    int64_t n_seg = 0;
    double center[3] = {0, 0, 0};
    double scale = 1.0;
    void* tri = nullptr; // predicate triangles in leaf order
    void* seg = nullptr; // quantised, swapped boundary segments
    void* chain = nullptr; // int64_grid: the segments as vertex chains (RChain) for the FP32 pairs
    int64_t n_entries = 0;
    Hier hier;
    mutable CellGrid cells; // the integer term's cell grid over hier, built on first use
};
} // namespace agwn

struct agwn_robust : agwn::Robust
{
};
