// cmg/voxelize/voxelize.hpp — the C++ voxelization entry of libcmg_c.so.
//
// Drop-in for cmg::voxelize::voxelize of the reference (include/cmg/voxelize/
// voxelize.hpp:25-63, src/voxelize/voxelize.cpp:362-398): the same types, the same
// function signature (and so the same linker symbol), the same results. Occupancy is
// the exact vertical ray parity over the facets' fan triangles, the signed distance
// the nearest point-triangle distance cast to float with its sign from occupancy;
// both are computed on the GPU and equal the reference's bit for bit. A program
// written against the reference links libcmg_c.so in place of the reference's
// voxelize.cpp and includes this header (and cmg/core/*) in place of the reference's.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include "cmg/core/error.hpp"
#include "cmg/core/expected.hpp"
#include "cmg/core/geometry.hpp"
#include "cmg/core/plc.hpp"

namespace cmg::voxelize {

enum class VoxelMode { Occupancy, SignedDistance };

struct VoxelOptions {
    int resolution = 64;  // cubic cells along the longest bounding-box axis (>= 1)
    int pad = 1;          // margin cells on every side of the bounding box
    VoxelMode mode = VoxelMode::Occupancy;
};

// Cell (i, j, k) is centred at origin + (i, j, k) * spacing; its flat index is
// (k * ny + j) * nx + i. Only the selected mode's array is filled.
struct VoxelGrid {
    Point3 origin;
    double spacing = 0;
    int nx = 0, ny = 0, nz = 0;
    std::vector<std::uint8_t> occupancy;  // Occupancy: 1 inside, 0 outside
    std::vector<float> distance;          // SignedDistance: negative inside

    std::size_t index(int i, int j, int k) const {
        return (static_cast<std::size_t>(k) * ny + j) * nx + i;
    }
    std::size_t cell_count() const { return static_cast<std::size_t>(nx) * ny * nz; }
};

// Voxelizes a closed PLC on `opts.resolution` cells along its longest axis plus
// `opts.pad` cells of margin. Never throws for bad input: resolution < 1, no points,
// no boundary triangles, a zero-extent PLC and (undefined behaviour in the reference)
// a facet index outside the points return MeshErrorCode::InvalidInput with the
// reference's messages; a device failure returns MeshErrorCode::Internal with the
// CUDA error text. Reentrant; calls on one device are serialised inside the library.
expected<VoxelGrid, MeshError> voxelize(const PLC& plc, const VoxelOptions& opts = {});

}  // namespace cmg::voxelize
