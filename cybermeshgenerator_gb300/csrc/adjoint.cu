// adjoint.cu — dL/d(vertex positions) of the signed distance field.
//
// For a cell p whose nearest triangle is t with closest point q on feature r
// (vertex, edge or interior: the Ericson region checkpointed by the forward pass),
// q = sum_k lambda_k V_k with the barycentrics of that feature, and by the
// envelope theorem d|p - q|/dV_k = -lambda_k (p - q) / |p - q|. With the signed
// field sdf = s |p - q| (s = -1 for occupied cells), a cell contributes
//   dL/dV_k += g_p * s * (-lambda_k (p - q) / |p - q|),   g_p = dL/dsdf(p).
// Only (t, region) per cell is kept from the forward; the backward recomputes q in
// FP64 from the current vertices.
//
// The reduction is deterministic without float atomics:
//  1. the checkpoint is cut into runs of equal nearest triangle along each x-row
//     (head flags, a scan, emission in cell order);
//  2. the runs are sorted by triangle with a stable radix sort, so each triangle's
//     runs, and the cells in them, come in ascending cell order; the sorted runs
//     laid end to end form the "position" sequence, grouped by triangle;
//  3. one lane per position computes its cell's contribution (coalesced: a run is
//     consecutive cells); each warp sums its segments of equal triangle in lane
//     order; a segment strictly inside a warp is a whole triangle and is written
//     out, the segments at the warp's two ends are stored as partials;
//  4. one thread per triangle adds its partials in warp order;
//  5. one thread per vertex adds its (triangle, corner) entries in a fixed CSR
//     order built on the host.
// Every sum has a fixed order given the checkpoint, so results are bitwise
// reproducible.
#include <cuda_runtime.h>

#include <cstdint>

#include "cmg_device.cuh"
#include "cmg_types.h"
#include "cmg_util.h"
#include "engine_kernels.h"

namespace cmg::gpu {

namespace {

// Per-triangle FP64 data of the adjoint (192 bytes): vertices, unit normal (zero
// for a zero-area triangle), the barycentric rows of the plane projection
// (lambda_b = (p - a).mb, lambda_c = (p - a).mc with mb = (ac x N)/|N|^2,
// mc = (N x ab)/|N|^2, N = ab x ac) and 1/|e|^2 of the edges ab, ac, bc (0 for a
// zero-length edge).
struct AdjTri {
    double a[3], b[3], c[3];
    double n[3];
    double mb[3], mc[3];
    double inv_e[3];
    double pad_[3];
};
static_assert(sizeof(AdjTri) == 192, "record layout");

__global__ void k_adj_tri_rec(int64_t ntris, const double* __restrict__ pts,
                              const int* __restrict__ tris, AdjTri* __restrict__ rec) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= ntris) return;
    AdjTri r;
    const int iv[3] = {tris[3 * t], tris[3 * t + 1], tris[3 * t + 2]};
    double* V[3] = {r.a, r.b, r.c};
    for (int k = 0; k < 3; ++k)
        for (int q = 0; q < 3; ++q) V[k][q] = pts[3 * static_cast<int64_t>(iv[k]) + q];
    double e1[3], e2[3], e3[3];
    for (int q = 0; q < 3; ++q) {
        e1[q] = r.b[q] - r.a[q];
        e2[q] = r.c[q] - r.a[q];
        e3[q] = r.c[q] - r.b[q];
    }
    const double N[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                         e1[0] * e2[1] - e1[1] * e2[0]};
    const double nn = N[0] * N[0] + N[1] * N[1] + N[2] * N[2];
    const double inn = nn > 0.0 ? 1.0 / nn : 0.0;
    const double il = nn > 0.0 ? 1.0 / sqrt(nn) : 0.0;
    for (int q = 0; q < 3; ++q) r.n[q] = N[q] * il;
    r.mb[0] = (e2[1] * N[2] - e2[2] * N[1]) * inn;
    r.mb[1] = (e2[2] * N[0] - e2[0] * N[2]) * inn;
    r.mb[2] = (e2[0] * N[1] - e2[1] * N[0]) * inn;
    r.mc[0] = (N[1] * e1[2] - N[2] * e1[1]) * inn;
    r.mc[1] = (N[2] * e1[0] - N[0] * e1[2]) * inn;
    r.mc[2] = (N[0] * e1[1] - N[1] * e1[0]) * inn;
    const double* E[3] = {e1, e2, e3};
    for (int k = 0; k < 3; ++k) {
        const double ee = E[k][0] * E[k][0] + E[k][1] * E[k][1] + E[k][2] * E[k][2];
        r.inv_e[k] = ee > 0.0 ? 1.0 / ee : 0.0;
    }
    r.pad_[0] = r.pad_[1] = r.pad_[2] = 0.0;
    rec[t] = r;
}

// 1/sqrt(x) in FP64: a single-precision seed refined by two Newton-Raphson steps
// y <- y (3/2 - (x/2) y^2), each of which roughly doubles the correct bits (24 ->
// 48 -> the double's 53). Outside the seed's comfortable range, 1/sqrt.
__device__ __forceinline__ double rsqrt_nr(double x) {
    if (!(x >= 1e-30 && x <= 1e30)) return 1.0 / sqrt(x);
    double y = static_cast<double>(rsqrtf(static_cast<float>(x)));
    const double h = 0.5 * x;
    y = y * (1.5 - h * y * y);
    y = y * (1.5 - h * y * y);
    return y;
}

// Distance gradient toward the segment u + t e (t clamped to [0, 1]) for point p:
// writes the weights (1 - t, t) and r = p - q; returns |r|^2.
__device__ __forceinline__ double seg_closest(const double* p, const double* u, const double* v,
                                              double inv_e, double& t, double* r) {
    const double e0 = v[0] - u[0], e1 = v[1] - u[1], e2 = v[2] - u[2];
    const double w0 = p[0] - u[0], w1 = p[1] - u[1], w2 = p[2] - u[2];
    t = fmin(fmax((w0 * e0 + w1 * e1 + w2 * e2) * inv_e, 0.0), 1.0);
    r[0] = w0 - t * e0;
    r[1] = w1 - t * e1;
    r[2] = w2 - t * e2;
    return r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
}

// The three corner gradients of one cell (9 doubles: corner k, axis a at 3k+a),
// scaled by f = -dL/d|sdf| (the sign of the cell folded in): on the checkpointed
// feature, (p - q)/|p - q| is the unit normal (face), or r/|r| toward the edge or
// vertex, and lambda the feature's barycentrics. Edge parameters are clamped to
// the segment, so a region taken from a forward in other arithmetic (mixed
// precision) still names a point of the triangle. Returns false on the surface
// (distance 0: not differentiable) or for a zero gradient.
__device__ bool cell_contrib(const double* p, const AdjTri& R, int reg, double f, double* out9) {
#pragma unroll
    for (int q = 0; q < 9; ++q) out9[q] = 0.0;
    if (f == 0.0) return false;
    const bool flat = R.n[0] != 0.0 || R.n[1] != 0.0 || R.n[2] != 0.0;
    if (reg == 6 && flat) {
        const double w0 = p[0] - R.a[0], w1 = p[1] - R.a[1], w2 = p[2] - R.a[2];
        const double h = w0 * R.n[0] + w1 * R.n[1] + w2 * R.n[2];
        if (h == 0.0) return false;
        const double lb = w0 * R.mb[0] + w1 * R.mb[1] + w2 * R.mb[2];
        const double lc = w0 * R.mc[0] + w1 * R.mc[1] + w2 * R.mc[2];
        const double lam[3] = {1.0 - lb - lc, lb, lc};
        const double fs = h > 0.0 ? f : -f;
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int q = 0; q < 3; ++q) out9[3 * k + q] = fs * lam[k] * R.n[q];
        return true;
    }
    double r[3], d2;
    int k0 = 0, k1 = 0;
    double t = 0.0;
    if (reg == 0 || reg == 1 || reg == 3) {  // a vertex
        k0 = k1 = reg == 0 ? 0 : (reg == 1 ? 1 : 2);
        const double* v = k0 == 0 ? R.a : (k0 == 1 ? R.b : R.c);
        r[0] = p[0] - v[0];
        r[1] = p[1] - v[1];
        r[2] = p[2] - v[2];
        d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    } else if (reg == 2 || reg == 4 || reg == 5) {  // an edge
        k0 = reg == 5 ? 1 : 0;
        k1 = reg == 2 ? 1 : 2;
        const double* u = k0 == 0 ? R.a : R.b;
        const double* v = k1 == 1 ? R.b : R.c;
        d2 = seg_closest(p, u, v, R.inv_e[reg == 2 ? 0 : (reg == 4 ? 1 : 2)], t, r);
    } else {  // the face of a zero-area triangle: its nearest edge
        double rr[3], tt;
        d2 = seg_closest(p, R.a, R.b, R.inv_e[0], t, r);
        k0 = 0;
        k1 = 1;
        double e2 = seg_closest(p, R.a, R.c, R.inv_e[1], tt, rr);
        if (e2 < d2) {
            d2 = e2; t = tt; k0 = 0; k1 = 2;
            r[0] = rr[0]; r[1] = rr[1]; r[2] = rr[2];
        }
        e2 = seg_closest(p, R.b, R.c, R.inv_e[2], tt, rr);
        if (e2 < d2) {
            d2 = e2; t = tt; k0 = 1; k1 = 2;
            r[0] = rr[0]; r[1] = rr[1]; r[2] = rr[2];
        }
    }
    if (!(d2 > 0.0)) return false;
    const double s = f * rsqrt_nr(d2);
    const double l0 = k0 == k1 ? 1.0 : 1.0 - t, l1 = k0 == k1 ? 0.0 : t;
#pragma unroll
    for (int k = 0; k < 3; ++k) {  // corner weights by select: no indexed local array
        const double wk = (k == k0 ? l0 : 0.0) + (k == k1 ? l1 : 0.0);
#pragma unroll
        for (int q = 0; q < 3; ++q) out9[3 * k + q] = s * wk * r[q];
    }
    return true;
}

// Per-triangle FP32 data of the mixed-precision adjoint (96 bytes): the vertex a
// relative to the grid corner as an FP32 pair (ah + al carries ~48 bits), the edges
// e1 = b - a and e2 = c - a, the unit normal, the barycentric rows mb, mc and 1/|e|^2
// of ab, ac, bc, all rounded from FP64.
struct AdjTri32 {
    float ah[3], al[3];
    float e1[3], e2[3];
    float n[3];
    float mb[3], mc[3];
    float inv_e[3];
};
static_assert(sizeof(AdjTri32) == 96, "record layout");

__global__ void k_adj_tri_rec32(int64_t ntris, const GridDesc g, const AdjTri* __restrict__ rec,
                                AdjTri32* __restrict__ rec32) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= ntris) return;
    const AdjTri& R = rec[t];
    AdjTri32 r;
    for (int q = 0; q < 3; ++q) {
        const double A = R.a[q] - g.corner[q];
        r.ah[q] = __double2float_rn(A);
        r.al[q] = __double2float_rn(A - static_cast<double>(r.ah[q]));
        r.e1[q] = __double2float_rn(R.b[q] - R.a[q]);
        r.e2[q] = __double2float_rn(R.c[q] - R.a[q]);
        r.n[q] = __double2float_rn(R.n[q]);
        r.mb[q] = __double2float_rn(R.mb[q]);
        r.mc[q] = __double2float_rn(R.mc[q]);
        r.inv_e[q] = __double2float_rn(R.inv_e[q]);
    }
    rec32[t] = r;
}

// 1/sqrt(x) in FP32: the hardware estimate and one Newton-Raphson step.
__device__ __forceinline__ float rsqrt32(float x) {
    float y = rsqrtf(x);
    return y * (1.5f - 0.5f * x * y * y);
}

__device__ __forceinline__ float seg_closest32(const float* w, const float* e, float inv_e,
                                               float& t, float* r) {
    t = __saturatef((w[0] * e[0] + w[1] * e[1] + w[2] * e[2]) * inv_e);
    r[0] = w[0] - t * e[0];
    r[1] = w[1] - t * e[1];
    r[2] = w[2] - t * e[2];
    return r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
}

// The FP32 form of cell_contrib for cell (i, j, k). p - a is formed from the FP32
// pairs of the cell centre's offset (i + 1/2) h (h = hh + hl, the product's rounding
// error recovered exactly by an FMA) and of a - corner, so it keeps ~48 bits before
// the single rounding to FP32; the rest is FP32 on these small vectors.
__device__ void cell_contrib32(uint32_t i, uint32_t j, uint32_t k, float hh, float hl,
                               const AdjTri32& R, int reg, float f, float* out9) {
#pragma unroll
    for (int q = 0; q < 9; ++q) out9[q] = 0.f;
    if (f == 0.f) return;
    const float x[3] = {static_cast<float>(i) + 0.5f, static_cast<float>(j) + 0.5f,
                        static_cast<float>(k) + 0.5f};
    float w[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const float ph = x[q] * hh;
        const float pe = fmaf(x[q], hh, -ph);  // exact rounding error of ph
        w[q] = __fsub_rn(ph, R.ah[q]) + ((pe + x[q] * hl) - R.al[q]);
    }
    const bool flat = R.n[0] != 0.f || R.n[1] != 0.f || R.n[2] != 0.f;
    if (reg == 6 && flat) {
        const float h = w[0] * R.n[0] + w[1] * R.n[1] + w[2] * R.n[2];
        if (h == 0.f) return;
        const float lb = w[0] * R.mb[0] + w[1] * R.mb[1] + w[2] * R.mb[2];
        const float lc = w[0] * R.mc[0] + w[1] * R.mc[1] + w[2] * R.mc[2];
        const float lam[3] = {1.f - lb - lc, lb, lc};
        const float fs = h > 0.f ? f : -f;
#pragma unroll
        for (int kk = 0; kk < 3; ++kk)
#pragma unroll
            for (int q = 0; q < 3; ++q) out9[3 * kk + q] = fs * lam[kk] * R.n[q];
        return;
    }
    const float wb[3] = {w[0] - R.e1[0], w[1] - R.e1[1], w[2] - R.e1[2]};
    float r[3], d2, t = 0.f;
    int k0 = 0, k1 = 0;
    if (reg == 0) {
        r[0] = w[0]; r[1] = w[1]; r[2] = w[2];
        d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    } else if (reg == 1) {
        k0 = k1 = 1;
        r[0] = wb[0]; r[1] = wb[1]; r[2] = wb[2];
        d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    } else if (reg == 3) {
        k0 = k1 = 2;
        r[0] = w[0] - R.e2[0]; r[1] = w[1] - R.e2[1]; r[2] = w[2] - R.e2[2];
        d2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    } else {
        const float e3[3] = {R.e2[0] - R.e1[0], R.e2[1] - R.e1[1], R.e2[2] - R.e1[2]};
        if (reg == 2) {
            k1 = 1;
            d2 = seg_closest32(w, R.e1, R.inv_e[0], t, r);
        } else if (reg == 4) {
            k1 = 2;
            d2 = seg_closest32(w, R.e2, R.inv_e[1], t, r);
        } else if (reg == 5) {
            k0 = 1;
            k1 = 2;
            d2 = seg_closest32(wb, e3, R.inv_e[2], t, r);
        } else {  // the face of a zero-area triangle: its nearest edge
            float rr[3], tt;
            k1 = 1;
            d2 = seg_closest32(w, R.e1, R.inv_e[0], t, r);
            float e2v = seg_closest32(w, R.e2, R.inv_e[1], tt, rr);
            if (e2v < d2) {
                d2 = e2v; t = tt; k0 = 0; k1 = 2;
                r[0] = rr[0]; r[1] = rr[1]; r[2] = rr[2];
            }
            e2v = seg_closest32(wb, e3, R.inv_e[2], tt, rr);
            if (e2v < d2) {
                d2 = e2v; t = tt; k0 = 1; k1 = 2;
                r[0] = rr[0]; r[1] = rr[1]; r[2] = rr[2];
            }
        }
    }
    if (!(d2 > 0.f)) return;
    const float sc = f * rsqrt32(d2);
    const float l0 = k0 == k1 ? 1.f : 1.f - t, l1 = k0 == k1 ? 0.f : t;
#pragma unroll
    for (int kk = 0; kk < 3; ++kk) {
        const float wk = (kk == k0 ? l0 : 0.f) + (kk == k1 ? l1 : 0.f);
#pragma unroll
        for (int q = 0; q < 3; ++q) out9[3 * kk + q] = sc * wk * r[q];
    }
}

// 1. run heads: the first cell of a row, or a cell whose nearest triangle differs
// from its left neighbour's.
__global__ void k_run_heads(int nx, int64_t ncell, const int* __restrict__ near_tri,
                            int* __restrict__ flag) {
    const int64_t v = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (v >= ncell) return;
    flag[v] = (v % nx == 0 || near_tri[v] != near_tri[v - 1]) ? 1 : 0;
}

// Run r = runidx[v] starts at head cell v; its key is the triangle (ntris, sorting
// last, when the cell has none) and its value r. st[R] = ncell closes the last run.
__global__ void k_run_emit(int64_t ncell, const int* __restrict__ flag,
                           const int64_t* __restrict__ runidx, const int* __restrict__ near_tri,
                           uint32_t ntris, uint32_t* __restrict__ st, uint32_t* __restrict__ keys,
                           uint32_t* __restrict__ vals) {
    const int64_t v = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (v >= ncell) return;
    if (v == ncell - 1) st[runidx[ncell]] = static_cast<uint32_t>(ncell);
    if (!flag[v]) return;
    const int64_t r = runidx[v];
    const int t = near_tri[v];
    st[r] = static_cast<uint32_t>(v);
    keys[r] = (t >= 0 && static_cast<uint32_t>(t) < ntris) ? static_cast<uint32_t>(t) : ntris;
    vals[r] = static_cast<uint32_t>(r);
}

// 2. lengths of the sorted runs (0 for runs without a triangle) and runs per triangle.
__global__ void k_run_len(int64_t nrun, const uint32_t* __restrict__ keys,
                          const uint32_t* __restrict__ vals, const uint32_t* __restrict__ st,
                          uint32_t ntris, int* __restrict__ len, int* __restrict__ tcount) {
    const int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= nrun) return;
    const uint32_t t = keys[e];
    if (t >= ntris) {
        len[e] = 0;
        return;
    }
    const uint32_t r = vals[e];
    len[e] = static_cast<int>(st[r + 1] - st[r]);
    atomicAdd(&tcount[t], 1);
}

// 3. one lane per position. P (nrun + 1 entries) holds the first position of every
// sorted run; positions [0, P[nrun]) are the cells that have a triangle.
template <int PREC>
__global__ void __launch_bounds__(256) k_adj_cells(
    const GridDesc g, float hh, float hl, int64_t nrun, const int64_t* __restrict__ P,
    const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals,
    const uint32_t* __restrict__ st, const AdjTri* __restrict__ rec,
    const AdjTri32* __restrict__ rec32, const uint8_t* __restrict__ near_reg,
    const uint8_t* __restrict__ occ, const double* __restrict__ grad_sdf,
    double* __restrict__ tri_grad, double* __restrict__ wp_first, double* __restrict__ wp_last) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t ptot = P[nrun];
    const int64_t w0 = warp * 32;
    if (w0 >= ptot) return;  // whole warp past the end (warp-uniform)
    // the run holding position w0: the last e with P[e] <= w0 (binary search by
    // lane 0, broadcast)
    int64_t lo = 0;
    if (lane == 0) {
        int64_t hi = nrun - 1;
        while (lo < hi) {
            const int64_t mid = (lo + hi + 1) >> 1;
            if (P[mid] <= w0) lo = mid;
            else hi = mid - 1;
        }
    }
    const int64_t ef = __shfl_sync(0xffffffffu, lo, 0);
    // the (at most 32) runs that start after w0 inside the window
    const int64_t pk = (ef + 1 + lane <= nrun) ? P[ef + 1 + lane] : INT64_MAX;
    const int64_t pos = w0 + lane;
    const bool valid = pos < ptot;
    int off = 0;
    for (int k = 0; k < 32; ++k) off += (__shfl_sync(0xffffffffu, pk, k) <= pos) ? 1 : 0;
    const int64_t e = ef + off;
    uint32_t key = 0xffffffffu;
    double c9[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    float c9f[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (valid) {
        key = keys[e];
        const uint32_t cell = st[vals[e]] + static_cast<uint32_t>(pos - P[e]);
        const uint32_t nxy = static_cast<uint32_t>(g.nx) * static_cast<uint32_t>(g.ny);
        const uint32_t k = cell / nxy, rem = cell - k * nxy;
        const uint32_t j = rem / static_cast<uint32_t>(g.nx), i = rem - j * static_cast<uint32_t>(g.nx);
        const double gs = grad_sdf[cell];
        const int reg = near_reg[cell];
        const bool in = occ[cell] != 0;
        if (PREC == kPrecFP64) {
            const double p[3] = {cell_center(g.corner[0], static_cast<int>(i), g.h),
                                 cell_center(g.corner[1], static_cast<int>(j), g.h),
                                 cell_center(g.corner[2], static_cast<int>(k), g.h)};
            // f = -dL/d|sdf|: an occupied cell's signed distance is -|sdf|
            cell_contrib(p, rec[key], reg, in ? gs : -gs, c9);
        } else {
            const float gf = static_cast<float>(gs);
            cell_contrib32(i, j, k, hh, hl, rec32[key], reg, in ? gf : -gf, c9f);
        }
    }
    // Segments of equal key are contiguous lane ranges. A log-step tree sums each
    // segment into its first lane: at step `d` lane l adds lane l + d's partial when
    // l + d is still in its segment, so lane l ends with the sum over [l, last] in a
    // fixed order (FP32: compensated, the pair hi + lo carrying ~48 bits).
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int first = __ffs(peers) - 1;
    const int last = 31 - __clz(peers);
    double acc[9];
    if (PREC == kPrecFP64) {
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const bool take = lane + d <= last;
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                const double y = __shfl_down_sync(0xffffffffu, c9[q], d);
                if (take) c9[q] += y;
            }
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) acc[q] = c9[q];
    } else {
        float lo9[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const bool take = lane + d <= last;
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                const float yh = __shfl_down_sync(0xffffffffu, c9f[q], d);
                const float yl = __shfl_down_sync(0xffffffffu, lo9[q], d);
                if (take) {
                    const float sh = __fadd_rn(c9f[q], yh);
                    const float bp = __fsub_rn(sh, c9f[q]);
                    const float er = __fadd_rn(__fsub_rn(c9f[q], __fsub_rn(sh, bp)), __fsub_rn(yh, bp));
                    c9f[q] = sh;
                    lo9[q] = __fadd_rn(__fadd_rn(lo9[q], yl), er);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) acc[q] = static_cast<double>(c9f[q]) + static_cast<double>(lo9[q]);
    }
    if (lane != first || !valid) return;
    const bool has_lane0 = first == 0;
    const bool has_lane31 = last == 31;
    if (!has_lane0 && !has_lane31) {
#pragma unroll
        for (int q = 0; q < 9; ++q) tri_grad[9 * static_cast<int64_t>(key) + q] = acc[q];
    } else if (has_lane0) {
#pragma unroll
        for (int q = 0; q < 9; ++q) wp_first[9 * warp + q] = acc[q];
    } else {
#pragma unroll
        for (int q = 0; q < 9; ++q) wp_last[9 * warp + q] = acc[q];
    }
}

// 4. triangles whose positions reach a warp's first or last lane: add the partials
// in warp order (in warp w the triangle is the first segment when it started before
// w or at its lane 0, else the last segment); empty triangles get zeros.
__global__ void k_adj_tri_combine(int64_t ntris, const int64_t* __restrict__ toff,
                                  const int64_t* __restrict__ P,
                                  const double* __restrict__ wp_first,
                                  const double* __restrict__ wp_last,
                                  double* __restrict__ tri_grad) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= ntris) return;
    const int64_t s0 = P[toff[t]], s1 = P[toff[t + 1]] - 1;
    if (s1 < s0) {
#pragma unroll
        for (int q = 0; q < 9; ++q) tri_grad[9 * t + q] = 0.0;
        return;
    }
    const int64_t w0 = s0 >> 5, w1 = s1 >> 5;
    if (w0 == w1 && (s0 & 31) != 0 && (s1 & 31) != 31) return;  // written by k_adj_cells
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t w = w0; w <= w1; ++w) {
        const double* src = (w > w0 || (s0 & 31) == 0) ? wp_first + 9 * w : wp_last + 9 * w;
#pragma unroll
        for (int q = 0; q < 9; ++q) acc[q] += src[q];
    }
#pragma unroll
    for (int q = 0; q < 9; ++q) tri_grad[9 * t + q] = acc[q];
}

// 5. one thread per vertex: its (triangle, corner) entries in CSR order.
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

// Carves the adjoint workspace; with base == nullptr only the size is computed.
struct AdjWork {
    int* flag;
    int64_t* runidx;
    int64_t* scan_tmp;
    uint32_t *st, *keys, *vals;
    void* sort_tmp;
    int* len;
    int64_t* P;
    int* tcount;
    int64_t* toff;
    double *wp_first, *wp_last, *tri_grad;
    AdjTri* rec;
    AdjTri32* rec32;
    size_t bytes;
    AdjWork(void* base, int64_t ncell, int64_t ntris) {
        char* p = static_cast<char*>(base);
        size_t used = 0;
        auto take = [&](size_t n) {
            char* q = p ? p + used : nullptr;
            used += (n + 255) & ~size_t(255);
            return q;
        };
        const int64_t nw = (ncell + 31) / 32;
        const int64_t smax = ncell + 1 > ntris + 1 ? ncell + 1 : ntris + 1;
        flag = reinterpret_cast<int*>(take(sizeof(int) * ncell));
        runidx = reinterpret_cast<int64_t*>(take(sizeof(int64_t) * (ncell + 1)));
        scan_tmp = reinterpret_cast<int64_t*>(take(sizeof(int64_t) * scan_tmp_elems(smax)));
        st = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * (ncell + 1)));
        keys = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * ncell));
        vals = reinterpret_cast<uint32_t*>(take(sizeof(uint32_t) * ncell));
        sort_tmp = take(radix_sort_tmp_bytes(ncell));
        len = reinterpret_cast<int*>(take(sizeof(int) * ncell));
        P = reinterpret_cast<int64_t*>(take(sizeof(int64_t) * (ncell + 1)));
        tcount = reinterpret_cast<int*>(take(sizeof(int) * (ntris + 1)));
        toff = reinterpret_cast<int64_t*>(take(sizeof(int64_t) * (ntris + 2)));
        wp_first = reinterpret_cast<double*>(take(sizeof(double) * 9 * nw));
        wp_last = reinterpret_cast<double*>(take(sizeof(double) * 9 * nw));
        tri_grad = reinterpret_cast<double*>(take(sizeof(double) * 9 * ntris));
        rec = reinterpret_cast<AdjTri*>(take(sizeof(AdjTri) * ntris));
        rec32 = reinterpret_cast<AdjTri32*>(take(sizeof(AdjTri32) * ntris));
        bytes = used;
    }
};

}  // namespace

size_t adjoint_tmp_bytes(int64_t ncell, int64_t ntris) {
    return AdjWork(nullptr, ncell, ntris).bytes;
}

void adjoint_backward(int precision, const GridDesc& g, int64_t ncell, const double* pts,
                      int64_t npts, const int* tris, int64_t ntris, const int* near_tri,
                      const uint8_t* near_reg, const uint8_t* occ, const double* grad_sdf,
                      const int64_t* voff, const int* vinc, double* grad, void* tmp,
                      cudaStream_t st) {
    AdjWork w(tmp, ncell, ntris);
    const uint32_t nt = static_cast<uint32_t>(ntris);
    const unsigned gc = static_cast<unsigned>((ncell + 255) / 256);
    k_run_heads<<<gc, 256, 0, st>>>(g.nx, ncell, near_tri, w.flag);
    CMG_LAUNCH();
    exclusive_scan(w.flag, w.runidx, ncell, w.scan_tmp, st);
    k_run_emit<<<gc, 256, 0, st>>>(ncell, w.flag, w.runidx, near_tri, nt, w.st, w.keys, w.vals);
    CMG_LAUNCH();
    int64_t nrun = 0;  // the sort's length is needed on the host
    CMG_CUDA(cudaMemcpyAsync(&nrun, w.runidx + ncell, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CMG_CUDA(cudaStreamSynchronize(st));
    int bits = 1;
    while ((int64_t(1) << bits) <= ntris) ++bits;
    radix_sort_pairs(w.keys, w.vals, nrun, bits, w.sort_tmp, st);
    CMG_CUDA(cudaMemsetAsync(w.tcount, 0, sizeof(int) * (ntris + 1), st));
    const unsigned gr = static_cast<unsigned>((nrun + 255) / 256);
    k_run_len<<<gr, 256, 0, st>>>(nrun, w.keys, w.vals, w.st, nt, w.len, w.tcount);
    CMG_LAUNCH();
    exclusive_scan(w.len, w.P, nrun, w.scan_tmp, st);
    exclusive_scan(w.tcount, w.toff, ntris, w.scan_tmp, st);
    const unsigned gt = static_cast<unsigned>((ntris + 127) / 128);
    k_adj_tri_rec<<<gt, 128, 0, st>>>(ntris, pts, tris, w.rec);
    CMG_LAUNCH();
    if (precision == kPrecMixed) {
        k_adj_tri_rec32<<<gt, 128, 0, st>>>(ntris, g, w.rec, w.rec32);
        CMG_LAUNCH();
        const float hh = static_cast<float>(g.h);
        const float hl = static_cast<float>(g.h - static_cast<double>(hh));
        k_adj_cells<kPrecMixed><<<gc, 256, 0, st>>>(g, hh, hl, nrun, w.P, w.keys, w.vals, w.st,
                                                    w.rec, w.rec32, near_reg, occ, grad_sdf,
                                                    w.tri_grad, w.wp_first, w.wp_last);
    } else {
        k_adj_cells<kPrecFP64><<<gc, 256, 0, st>>>(g, 0.f, 0.f, nrun, w.P, w.keys, w.vals, w.st,
                                                   w.rec, w.rec32, near_reg, occ, grad_sdf,
                                                   w.tri_grad, w.wp_first, w.wp_last);
    }
    CMG_LAUNCH();
    k_adj_tri_combine<<<gt, 128, 0, st>>>(ntris, w.toff, w.P, w.wp_first, w.wp_last, w.tri_grad);
    CMG_LAUNCH();
    const unsigned gp = static_cast<unsigned>((npts + 127) / 128);
    k_adj_vertex<<<gp, 128, 0, st>>>(npts, voff, vinc, w.tri_grad, grad);
    CMG_LAUNCH();
}

}  // namespace cmg::gpu
