// cmg_seg.cuh — locate the mesh of a flattened index in a batch.
#pragma once

#include "cmg_types.h"

namespace cmg::gpu {

// Largest s with (segs[s].*field) <= idx (segments are in ascending order).
template <int64_t MeshSeg::*field>
__device__ __forceinline__ int find_seg(const MeshSeg* __restrict__ segs, int nseg, int64_t idx) {
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (segs[mid].*field <= idx) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Upper bound in a sorted int64 prefix array: the last e with off[e] <= x.
__device__ __forceinline__ int64_t last_le(const int64_t* __restrict__ off, int64_t n, int64_t x) {
    int64_t lo = 0, hi = n - 1;
    while (lo < hi) {
        int64_t mid = (lo + hi + 1) >> 1;
        if (off[mid] <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

}  // namespace cmg::gpu
