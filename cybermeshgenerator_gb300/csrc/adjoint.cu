// adjoint.cu — dL/d(vertex positions) of the unsigned distance field.
//
// For a cell p whose nearest triangle is t with closest point q on feature r
// (vertex, edge or interior: the Ericson region checkpointed by the forward pass),
// q = sum_k lambda_k V_k with the barycentrics of that feature, and by the
// envelope theorem d|p - q|/dV_k = -lambda_k (p - q) / |p - q|. With the signed
// field sdf = s |p - q| (s = -1 for occupied cells), a cell contributes
//   dL/dV_k += g_p * s * (-lambda_k (p - q) / |p - q|),   g_p = dL/dsdf(p).
// Only (t, region) per cell is kept from the forward; the backward recomputes q in
// FP64 from the current vertices. The reduction is deterministic without float
// atomics: cells are grouped by triangle with a stable radix sort (ascending cell
// order inside each triangle), each triangle's three corner gradients are summed
// in that order, and each vertex sums its (triangle, corner) entries in a fixed
// CSR order built on the host.
#include <cuda_runtime.h>

#include <cstdint>

#include "cmg_device.cuh"
#include "cmg_types.h"
#include "cmg_util.h"
#include "engine_kernels.h"

namespace cmg::gpu {

namespace {

__device__ __forceinline__ double dotd(double ax, double ay, double az, double bx, double by, double bz) {
    return ax * bx + ay * by + az * bz;
}

__device__ __forceinline__ double clamp01(double x) { return fmin(fmax(x, 0.0), 1.0); }

// Closest point barycentrics for the checkpointed feature `reg` of abc at p
// (Ericson's region formulas, src/voxelize/voxelize.cpp:212-246), FP64. Edge
// parameters are clamped to the segment, so a region taken from a forward in other
// arithmetic (mixed precision) still names a point of the triangle.
__device__ void feature_bary(const d3& p, const d3& a, const d3& b, const d3& c, int reg,
                             double* lam) {
    const double abx = b.x - a.x, aby = b.y - a.y, abz = b.z - a.z;
    const double acx = c.x - a.x, acy = c.y - a.y, acz = c.z - a.z;
    const double d1 = dotd(abx, aby, abz, p.x - a.x, p.y - a.y, p.z - a.z);
    const double d2 = dotd(acx, acy, acz, p.x - a.x, p.y - a.y, p.z - a.z);
    const double d3v = dotd(abx, aby, abz, p.x - b.x, p.y - b.y, p.z - b.z);
    const double d4 = dotd(acx, acy, acz, p.x - b.x, p.y - b.y, p.z - b.z);
    const double d5 = dotd(abx, aby, abz, p.x - c.x, p.y - c.y, p.z - c.z);
    const double d6 = dotd(acx, acy, acz, p.x - c.x, p.y - c.y, p.z - c.z);
    lam[0] = lam[1] = lam[2] = 0.0;
    switch (reg) {
    case 0: lam[0] = 1.0; break;
    case 1: lam[1] = 1.0; break;
    case 2: {
        const double den = d1 - d3v;
        const double v = den != 0.0 ? clamp01(d1 / den) : 0.0;
        lam[0] = 1.0 - v; lam[1] = v;
        break;
    }
    case 3: lam[2] = 1.0; break;
    case 4: {
        const double den = d2 - d6;
        const double w = den != 0.0 ? clamp01(d2 / den) : 0.0;
        lam[0] = 1.0 - w; lam[2] = w;
        break;
    }
    case 5: {
        const double den = (d4 - d3v) + (d5 - d6);
        const double w = den != 0.0 ? clamp01((d4 - d3v) / den) : 0.0;
        lam[1] = 1.0 - w; lam[2] = w;
        break;
    }
    default: {
        const double vc = d1 * d4 - d3v * d2, vb = d5 * d2 - d1 * d6, va = d3v * d6 - d5 * d4;
        const double s = va + vb + vc;
        const double v = s != 0.0 ? vb / s : 0.0, w = s != 0.0 ? vc / s : 0.0;
        lam[0] = 1.0 - v - w; lam[1] = v; lam[2] = w;
    }
    }
}

// The three corner gradients of one cell (9 doubles: corner k, axis a at 3k+a).
__device__ bool cell_contrib(const GridDesc& g, int64_t cell, const double* __restrict__ pts,
                             const int* __restrict__ tris, int t, int reg, bool inside,
                             double gsdf, double* out9) {
    const int64_t nxy = static_cast<int64_t>(g.nx) * g.ny;
    const int k = static_cast<int>(cell / nxy);
    const int64_t rem = cell % nxy;
    const int j = static_cast<int>(rem / g.nx), i = static_cast<int>(rem % g.nx);
    const d3 p{cell_center(g.corner[0], i, g.h), cell_center(g.corner[1], j, g.h),
               cell_center(g.corner[2], k, g.h)};
    const int ia = tris[3 * t], ib = tris[3 * t + 1], ic = tris[3 * t + 2];
    const d3 a{pts[3 * ia], pts[3 * ia + 1], pts[3 * ia + 2]};
    const d3 b{pts[3 * ib], pts[3 * ib + 1], pts[3 * ib + 2]};
    const d3 c{pts[3 * ic], pts[3 * ic + 1], pts[3 * ic + 2]};
    double lam[3];
    feature_bary(p, a, b, c, reg, lam);
    const double qx = lam[0] * a.x + lam[1] * b.x + lam[2] * c.x;
    const double qy = lam[0] * a.y + lam[1] * b.y + lam[2] * c.y;
    const double qz = lam[0] * a.z + lam[1] * b.z + lam[2] * c.z;
    const double nx = p.x - qx, ny = p.y - qy, nz = p.z - qz;
    const double d = sqrt(nx * nx + ny * ny + nz * nz);
    if (!(d > 0.0)) return false;  // on the surface: the distance is not differentiable
    const double f = -(inside ? -gsdf : gsdf) / d;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        out9[3 * q] = f * lam[q] * nx;
        out9[3 * q + 1] = f * lam[q] * ny;
        out9[3 * q + 2] = f * lam[q] * nz;
    }
    return true;
}

// Sort keys: triangle id of contributing cells, ntris (sorts last) otherwise.
__global__ void k_adj_keys(int64_t ncell, const int* __restrict__ near_tri,
                           const double* __restrict__ grad_sdf, uint32_t ntris,
                           uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                           int* __restrict__ tcount) {
    const int64_t v = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (v >= ncell) return;
    const int t = near_tri[v];
    const bool live = t >= 0 && static_cast<uint32_t>(t) < ntris && grad_sdf[v] != 0.0;
    keys[v] = live ? static_cast<uint32_t>(t) : ntris;
    vals[v] = static_cast<uint32_t>(v);
    if (live) atomicAdd(&tcount[t], 1);
}

// One thread per triangle: its cells in ascending order (the sorted segment).
__global__ void k_adj_tri(const GridDesc g, int64_t ntris, const int64_t* __restrict__ toff,
                          const uint32_t* __restrict__ sorted_cells, const double* __restrict__ pts,
                          const int* __restrict__ tris, const uint8_t* __restrict__ near_reg,
                          const uint8_t* __restrict__ occ, const double* __restrict__ grad_sdf,
                          double* __restrict__ tri_grad) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= ntris) return;
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t e = toff[t]; e < toff[t + 1]; ++e) {
        const int64_t v = sorted_cells[e];
        double c9[9];
        if (cell_contrib(g, v, pts, tris, static_cast<int>(t), near_reg[v], occ[v] != 0,
                         grad_sdf[v], c9)) {
#pragma unroll
            for (int q = 0; q < 9; ++q) acc[q] += c9[q];
        }
    }
#pragma unroll
    for (int q = 0; q < 9; ++q) tri_grad[9 * t + q] = acc[q];
}

// One thread per vertex: its (triangle, corner) entries in CSR order.
__global__ void k_adj_vertex(int64_t npts, const int64_t* __restrict__ voff,
                             const int* __restrict__ vinc, const double* __restrict__ tri_grad,
                             double* __restrict__ grad) {
    const int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    double gx = 0, gy = 0, gz = 0;
    for (int64_t e = voff[p]; e < voff[p + 1]; ++e) {
        const int code = vinc[e];  // 3 * triangle + corner
        const double* tg = tri_grad + 3 * static_cast<int64_t>(code);
        gx += tg[0];
        gy += tg[1];
        gz += tg[2];
    }
    grad[3 * p] = gx;
    grad[3 * p + 1] = gy;
    grad[3 * p + 2] = gz;
}

}  // namespace

size_t adjoint_tmp_bytes(int64_t ncell, int64_t ntris) {
    return 2 * sizeof(uint32_t) * static_cast<size_t>(ncell) + radix_sort_tmp_bytes(ncell) +
           sizeof(int) * static_cast<size_t>(ntris + 1) +
           sizeof(int64_t) * static_cast<size_t>(ntris + 2) +
           sizeof(int64_t) * scan_tmp_elems(ntris + 1) +
           sizeof(double) * 9 * static_cast<size_t>(ntris) + 8 * 256;
}

void adjoint_backward(const GridDesc& g, int64_t ncell, const double* pts, int64_t npts,
                      const int* tris, int64_t ntris, const int* near_tri, const uint8_t* near_reg,
                      const uint8_t* occ, const double* grad_sdf, const int64_t* voff,
                      const int* vinc, double* grad, void* tmp, cudaStream_t st) {
    char* p = static_cast<char*>(tmp);
    auto take = [&](size_t bytes) {
        char* q = p;
        p += (bytes + 255) & ~size_t(255);
        return q;
    };
    uint32_t* keys = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * ncell));
    uint32_t* vals = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * ncell));
    void* sort_tmp = take(radix_sort_tmp_bytes(ncell));
    int* tcount = reinterpret_cast<int*>(take(sizeof(int) * (ntris + 1)));
    int64_t* toff = reinterpret_cast<int64_t*>(take(sizeof(int64_t) * (ntris + 2)));
    int64_t* stmp = reinterpret_cast<int64_t*>(take(sizeof(int64_t) * scan_tmp_elems(ntris + 1)));
    double* tri_grad = reinterpret_cast<double*>(take(sizeof(double) * 9 * ntris));
    CMG_CUDA(cudaMemsetAsync(tcount, 0, sizeof(int) * (ntris + 1), st));
    const unsigned gc = static_cast<unsigned>((ncell + 255) / 256);
    k_adj_keys<<<gc, 256, 0, st>>>(ncell, near_tri, grad_sdf, static_cast<uint32_t>(ntris), keys,
                                   vals, tcount);
    CMG_LAUNCH();
    int bits = 1;
    while ((int64_t(1) << bits) <= ntris) ++bits;
    radix_sort_pairs(keys, vals, ncell, bits, sort_tmp, st);
    exclusive_scan(tcount, toff, ntris, stmp, st);
    const unsigned gt = static_cast<unsigned>((ntris + 127) / 128);
    k_adj_tri<<<gt, 128, 0, st>>>(g, ntris, toff, vals, pts, tris, near_reg, occ, grad_sdf, tri_grad);
    CMG_LAUNCH();
    const unsigned gp = static_cast<unsigned>((npts + 127) / 128);
    k_adj_vertex<<<gp, 128, 0, st>>>(npts, voff, vinc, tri_grad, grad);
    CMG_LAUNCH();
}

}  // namespace cmg::gpu
