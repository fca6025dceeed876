// cmg/core/real.hpp — the coordinate type of the C++ surface of libcmg_c.so.
//
// Replaces include/cmg/core/real.hpp of the reference for the voxelization path:
// coordinates are double precision (the reference's default build). The reference's
// CMG_SINGLE build (float coordinates) has no counterpart here: the GPU path reads
// FP64 coordinates and rounds exactly as the double build does.
#pragma once

#ifdef CMG_SINGLE
#error "libcmg_c.so is built for double-precision coordinates; CMG_SINGLE is not supported"
#endif

namespace cmg {

using Real = double;

}  // namespace cmg
