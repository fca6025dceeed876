// cmg_types.h — plain data shared by the host engine and the device kernels.
#pragma once

#include <cstdint>

namespace cmg::gpu {

// Regular grid: cell (i,j,k) has its centre at corner + (i+0.5, j+0.5, k+0.5)*h
// and flat index (k*ny + j)*nx + i (include/cmg/voxelize/voxelize.hpp:36-52).
// [z0, z1) is the slab of cell layers evaluated and stored (the whole grid: 0, nz):
// the geometry stays the whole grid's (centres, occupancy columns from below the
// first layer to above the last, SDF bricks), so a slab's cells equal the whole
// grid's bit for bit; its outputs hold layers z0 .. z1-1, index ((k-z0)*ny + j)*nx + i.
struct GridDesc {
    double corner[3];
    double h;
    int nx, ny, nz;
    int z0, z1;
};

#if defined(__CUDACC__)
__host__ __device__
#endif
inline int64_t slab_cells(const GridDesc& g) {
    return static_cast<int64_t>(g.nx) * g.ny * (g.z1 - g.z0);
}

// One mesh of a batch. Every index range is global (into the concatenated
// arrays of the batch), so kernels over a flattened index space recover the mesh
// by a binary search on the corresponding *_begin field.
struct MeshSeg {
    GridDesc g;
    int64_t tri_begin, tri_end;     // triangles
    int64_t col_begin;              // xy columns (nx*ny)
    int64_t row_begin;              // occupancy work rows: ny * ceil(nx/32)
    int64_t vox_begin;              // cells (nx*ny*(z1-z0), the slab's)
    int64_t brick_begin;            // SDF bricks (also the triangle bins)
    int bnx, bny, bnz;              // bricks per axis (along z: those overlapping the slab)
    int bzo;                        // brick layer of the mesh's first brick (the slab's)
    int brick;                      // brick edge in cells
    int64_t large_begin, large_end; // always-considered triangles (global list)
    float emax;                     // max centroid-to-vertex distance of binned triangles
    float emax_all;                 // the same over all the mesh's triangles
    float scale;                    // max |coordinate| of the mesh and grid (error bounds)
};

// Counters written by the kernels (device memory, one per batch).
struct Stats {
    unsigned long long flagged_columns;    // occupancy columns sent to the exact pass
    unsigned long long nudged_columns;     // first attempt grazed
    unsigned long long exhausted_columns;  // every nudge grazed
    unsigned long long exact_calls;        // orient3d resolved in exact arithmetic
    unsigned long long height_overflow;    // columns whose crossings overflowed shared memory
    unsigned long long candidates;         // SDF candidate (brick, triangle) pairs
    unsigned long long evaluations;        // SDF (voxel, triangle) distance evaluations
    unsigned long long fp64_evaluations;   // of which in FP64
    unsigned long long band_voxels;        // mixed precision: voxels refined in FP64
    unsigned long long error_flags;        // nonzero: a kernel hit a capacity limit
    unsigned long long orient_calls;       // occupancy filter: orient3d evaluations
    unsigned long long crossings;          // occupancy filter: plane_z evaluations
    unsigned long long filtered;           // SDF: sub-brick list entries (sphere tests per cell)
};

enum : int { kPredCompat = 0, kPredExact = 1 };
enum : int { kPrecFP64 = 0, kPrecMixed = 1 };
// The evaluation kernel's own third precision: FP64 results through the FP32 pass and an
// FP64 refinement of each cell's near-ties (kPrecFP64 on 16^3 bricks unless plain FP64 is
// asked for).
enum : int { kPrecExact = 2 };

// Triangle record in the soup: 9 coordinates + 1 pad (80 bytes, 16-byte aligned).
constexpr int kSoupStride = 10;

}  // namespace cmg::gpu
