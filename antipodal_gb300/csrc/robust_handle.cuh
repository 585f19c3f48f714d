// The robust evaluator's handle (agwn_robust): its geometry on the device, as robust.cu builds it and batch.cu
// reads it.
#pragma once

#include "agwn_internal.cuh"

namespace agwn
{
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
    Hier hier;
    mutable CellGrid cells; // the integer term's cell grid over hier, built on first use
};
} // namespace agwn

struct agwn_robust : agwn::Robust
{
};
