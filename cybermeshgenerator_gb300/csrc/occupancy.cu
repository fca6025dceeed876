// occupancy.cu — inside/outside bytes by exact vertical ray parity.
//
// Restates the reference's classify_occupancy (src/voxelize/voxelize.cpp:121-196)
// for the GPU:
//   k_tri_prep     triangle soup (80-byte records) + the reference's xy cell box of
//                  each triangle (floor((x-corner)/h), clamped; voxelize.cpp:82-100)
//   k_col_pairs    (triangle, column) pairs of those boxes -> per-column buckets (CSR)
//   k_occ_filter   one warp per column, lanes over the column's bucket: orient3d in
//                  reference operation order (FP64, no FMA); every column whose
//                  evaluations are all decided by the rounded determinant is finished
//                  here (crossings in shared memory, parity, coalesced byte rows);
//                  the rest are appended to a compact list
//   k_occ_exact    one warp per listed column: the same walk with exact signs for the
//                  undecided evaluations, the reference's six nudges on a graze, and
//                  its keep-the-last-partial-result rule when every nudge grazes.
// Bucket order in the reference is ascending triangle id; here buckets are
// unordered and "the first graze" is the graze with the smallest triangle id, so
// the partial heights are exactly the crossings of smaller ids.
#include <cuda_runtime.h>

#include <climits>

#include "cmg_device.cuh"
#include "cmg_exact.cuh"
#include "cmg_seg.cuh"
#include "cmg_types.h"
#include "cmg_util.h"
#include "engine_kernels.h"

namespace cmg::gpu {

namespace {

constexpr int kRowCols = 32;   // columns per CTA row segment
constexpr int kOccThreads = 128;
constexpr int kHCap = 32;      // crossings kept in shared memory per column

__constant__ double c_nudge[6][2] = {
    {1.0e-6, 3.0e-7},  {-7.0e-7, 5.0e-7}, {4.0e-7, -9.0e-7},
    {-2.0e-6, -1.0e-6}, {8.0e-7, 6.0e-7}, {-5.0e-7, -4.0e-6},
};  // voxelize.cpp:148-151

__device__ __forceinline__ void load_tri(const double* __restrict__ soup, int64_t t, d3& a, d3& b,
                                         d3& c) {
    const double2* r = reinterpret_cast<const double2*>(soup + t * kSoupStride);
    double2 v0 = __ldg(r), v1 = __ldg(r + 1), v2 = __ldg(r + 2), v3 = __ldg(r + 3), v4 = __ldg(r + 4);
    a = {v0.x, v0.y, v1.x};
    b = {v1.y, v2.x, v2.y};
    c = {v3.x, v3.y, v4.x};
}

// plane_z (voxelize.cpp:107-114) in reference order.
__device__ __forceinline__ double plane_z(const d3& a, const d3& b, const d3& c, double x, double y) {
    double ux = dsub(b.x, a.x), uy = dsub(b.y, a.y), uz = dsub(b.z, a.z);
    double vx = dsub(c.x, a.x), vy = dsub(c.y, a.y), vz = dsub(c.z, a.z);
    double nx = dsub(dmul(uy, vz), dmul(uz, vy));
    double ny = dsub(dmul(uz, vx), dmul(ux, vz));
    double nz = dsub(dmul(ux, vy), dmul(uy, vx));
    return dsub(a.z, ddiv(dadd(dmul(nx, dsub(x, a.x)), dmul(ny, dsub(y, a.y))), nz));
}

// Sign of orient3d under the chosen semantics. FULL=false: returns 2 when the
// rounded determinant does not decide (COMPAT: it is exactly zero; EXACT: it is
// within the error bound). FULL=true: falls back to exact arithmetic.
template <bool FULL, int MODE>
__device__ __forceinline__ int o3d_sign(const d3& a, const d3& b, const d3& c, const d3& d,
                                        unsigned* exact_calls) {
    double perm;
    double det = o3d_fast(a, b, c, d, MODE == kPredExact ? &perm : nullptr);
    bool decided;
    if (MODE == kPredCompat) decided = det != 0.0;
    else decided = det > kO3dErrA * perm || -det > kO3dErrA * perm;
    if (decided) return sgn(det);
    if (!FULL) return 2;
    ++*exact_calls;
    return exact::orient3d_sign(a, b, c, d);
}

// One bucket triangle against the vertical segment P..Q (voxelize.cpp:127-141).
// Returns 0: no crossing, 1: crossing (height in *h), 2: graze (FULL) or
// undecided (filter).
template <bool FULL, int MODE>
__device__ __forceinline__ int column_tri(const d3& P, const d3& Q, const d3& a, const d3& b,
                                          const d3& c, double* h, unsigned* exact_calls,
                                          unsigned* orients = nullptr) {
    int sa = o3d_sign<FULL, MODE>(P, a, b, c, exact_calls);
    if (sa == 2 || sa == 0) return 2;
    int sb = o3d_sign<FULL, MODE>(Q, a, b, c, exact_calls);
    if (sb == 2 || sb == 0) return 2;
    if (orients) *orients += 2;
    if (sa == sb) return 0;
    if (orients) *orients += 3;
    int s1 = o3d_sign<FULL, MODE>(P, Q, a, b, exact_calls);
    if (s1 == 2 || s1 == 0) return 2;
    int s2 = o3d_sign<FULL, MODE>(P, Q, b, c, exact_calls);
    if (s2 == 2 || s2 == 0) return 2;
    int s3 = o3d_sign<FULL, MODE>(P, Q, c, a, exact_calls);
    if (s3 == 2 || s3 == 0) return 2;
    if (s1 != s2 || s2 != s3) return 0;
    *h = plane_z(a, b, c, P.x, P.y);
    return 1;
}

// Number of cell centres strictly below h: #{k : zc_k < h}. zc_k is
// non-decreasing in k, so {k : zc_k < h} is a prefix [0, n).
__device__ __forceinline__ int centres_below(double hgt, double cz, double sp, int nz) {
    int lo = 0, hi = nz;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (cell_center(cz, mid, sp) < hgt) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__global__ void k_tri_prep(const MeshSeg* __restrict__ segs, int nseg, int64_t ntris,
                           const double* __restrict__ pts, const int* __restrict__ tris,
                           double* __restrict__ soup, int4* __restrict__ xybox,
                           int64_t* __restrict__ pairs) {
    int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= ntris) return;
    const MeshSeg& s = segs[find_seg<&MeshSeg::tri_begin>(segs, nseg, t)];
    double v[9];
    for (int k = 0; k < 3; ++k) {
        int64_t vi = tris[3 * t + k];
        v[3 * k] = pts[3 * vi];
        v[3 * k + 1] = pts[3 * vi + 1];
        v[3 * k + 2] = pts[3 * vi + 2];
    }
    double2* r = reinterpret_cast<double2*>(soup + t * kSoupStride);
    r[0] = make_double2(v[0], v[1]);
    r[1] = make_double2(v[2], v[3]);
    r[2] = make_double2(v[4], v[5]);
    r[3] = make_double2(v[6], v[7]);
    r[4] = make_double2(v[8], 0.0);
    int i0 = s.g.nx, i1 = 0, j0 = s.g.ny, j1 = 0;
    for (int k = 0; k < 3; ++k) {
        int i = cell_clamped(v[3 * k], s.g.corner[0], s.g.h, s.g.nx);
        int j = cell_clamped(v[3 * k + 1], s.g.corner[1], s.g.h, s.g.ny);
        i0 = min(i0, i); i1 = max(i1, i);
        j0 = min(j0, j); j1 = max(j1, j);
    }
    xybox[t] = make_int4(i0, i1, j0, j1);
    pairs[t] = static_cast<int64_t>(i1 - i0 + 1) * (j1 - j0 + 1);
}

// FILL=false: count bucket sizes; FILL=true: write bucket entries.
template <bool FILL>
__global__ void k_col_pairs(const MeshSeg* __restrict__ segs, int nseg, int64_t ntris,
                            const int4* __restrict__ xybox, const int64_t* __restrict__ pair_off,
                            int* __restrict__ colcnt, const int64_t* __restrict__ col_off,
                            int* __restrict__ col_list) {
    const int64_t npairs = pair_off[ntris];
    for (int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; p < npairs;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t t = last_le(pair_off, ntris, p);
        while (t + 1 < ntris && pair_off[t + 1] <= p) ++t;  // skip empty predecessors
        const MeshSeg& s = segs[find_seg<&MeshSeg::tri_begin>(segs, nseg, t)];
        int4 bx = xybox[t];
        int64_t local = p - pair_off[t];
        int w = bx.y - bx.x + 1;
        int i = bx.x + static_cast<int>(local % w);
        int j = bx.z + static_cast<int>(local / w);
        int64_t col = s.col_begin + static_cast<int64_t>(j) * s.g.nx + i;
        int slot = atomicAdd(&colcnt[col], 1);
        if (FILL) col_list[col_off[col] + slot] = static_cast<int>(t);
    }
}

template <int MODE>
__global__ void __launch_bounds__(kOccThreads)
k_occ_filter(const MeshSeg* __restrict__ segs, int nseg, const double* __restrict__ soup,
             const int64_t* __restrict__ col_off, const int* __restrict__ col_list,
             uint8_t* __restrict__ occ, int64_t* __restrict__ flagged, Stats* __restrict__ st) {
    __shared__ double hts[kRowCols][kHCap];
    __shared__ int nbelow[kRowCols][kHCap];
    __shared__ int hcnt[kRowCols];
    __shared__ int cflag[kRowCols];
    __shared__ unsigned long long* flag_count;

    const int64_t row = blockIdx.x;
    const int si = find_seg<&MeshSeg::row_begin>(segs, nseg, row);
    const MeshSeg& s = segs[si];
    const GridDesc g = s.g;
    const int rows_per_j = (g.nx + kRowCols - 1) / kRowCols;
    const int64_t lrow = row - s.row_begin;
    const int j = static_cast<int>(lrow / rows_per_j);
    const int i0 = static_cast<int>(lrow % rows_per_j) * kRowCols;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x < kRowCols) {
        hcnt[threadIdx.x] = 0;
        cflag[threadIdx.x] = 0;
    }
    __syncthreads();

    const double zmin = dsub(g.corner[2], g.h);
    const double zmax = dadd(g.corner[2], dmul(static_cast<double>(g.nz + 1), g.h));
    const double cy = cell_center(g.corner[1], j, g.h);
    unsigned dummy = 0, orients = 0, crossings = 0;
    for (int c = warp; c < kRowCols; c += kOccThreads / 32) {
        const int i = i0 + c;
        if (i >= g.nx) break;
        const int64_t col = s.col_begin + static_cast<int64_t>(j) * g.nx + i;
        const double cx = cell_center(g.corner[0], i, g.h);
        const d3 P{cx, cy, zmin}, Q{cx, cy, zmax};
        int undecided = 0;
        for (int64_t e = col_off[col] + lane; e < col_off[col + 1]; e += 32) {
            d3 a, b, cc;
            load_tri(soup, col_list[e], a, b, cc);
            double hgt;
            int r = column_tri<false, MODE>(P, Q, a, b, cc, &hgt, &dummy, &orients);
            if (r == 2) {
                undecided = 1;
            } else if (r == 1) {
                ++crossings;
                int slot = atomicAdd(&hcnt[c], 1);
                if (slot < kHCap) hts[c][slot] = hgt;
                else undecided = 1;
            }
        }
        if (__any_sync(0xffffffffu, undecided) && lane == 0) cflag[c] = 1;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < kRowCols * kHCap; q += kOccThreads) {
        int c = q / kHCap, k = q % kHCap;
        if (k < min(hcnt[c], kHCap)) nbelow[c][k] = centres_below(hts[c][k], g.corner[2], g.h, g.nz);
    }
    __syncthreads();
    // parity bytes: lane = column, warps stride k; one warp writes 32 consecutive bytes
    // (the layers of the slab [z0, z1) only; the column spans the whole grid)
    {
        const int c = lane, i = i0 + lane;
        const bool live = i < g.nx && !cflag[c];
        const int m = min(hcnt[c], kHCap);
        uint8_t* base = occ + s.vox_begin + static_cast<int64_t>(j) * g.nx + i;
        const int64_t kstride = static_cast<int64_t>(g.nx) * g.ny;
        for (int k = g.z0 + warp; k < g.z1; k += kOccThreads / 32) {
            if (!live) continue;
            int par = 0;
            for (int q = 0; q < m; ++q) par ^= (nbelow[c][q] > k);
            base[(k - g.z0) * kstride] = static_cast<uint8_t>(par);
        }
    }
    {
        long long o = warp_sum(static_cast<long long>(orients));
        long long x = warp_sum(static_cast<long long>(crossings));
        if (lane == 0 && o) atomicAdd(&st->orient_calls, static_cast<unsigned long long>(o));
        if (lane == 0 && x) atomicAdd(&st->crossings, static_cast<unsigned long long>(x));
    }
    if (warp == 0) {
        const int i = i0 + lane;
        bool f = i < g.nx && cflag[lane];
        unsigned mask = __ballot_sync(0xffffffffu, f);
        int n = __popc(mask);
        unsigned long long base = 0;
        if (lane == 0 && n) base = atomicAdd(&st->flagged_columns, static_cast<unsigned long long>(n));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (f) {
            int rank = __popc(mask & ((1u << lane) - 1u));
            flagged[base + rank] = s.col_begin + static_cast<int64_t>(j) * g.nx + i;
        }
    }
    (void)flag_count;
}

// One warp per listed column (grid-stride); scratch hs[e] holds the crossing height
// of bucket entry e (NaN-free flag in hv[e]) of the attempt being kept.
template <int MODE>
__global__ void __launch_bounds__(128)
k_occ_exact(const MeshSeg* __restrict__ segs, int nseg, const double* __restrict__ soup,
            const int64_t* __restrict__ col_off, const int* __restrict__ col_list,
            const int64_t* __restrict__ flagged, double* __restrict__ hs, uint8_t* __restrict__ hv,
            uint8_t* __restrict__ occ, Stats* __restrict__ st) {
    const int lane = threadIdx.x & 31;
    const int64_t nflag = static_cast<int64_t>(st->flagged_columns);
    const int64_t wstride = static_cast<int64_t>(gridDim.x) * (blockDim.x / 32);
    for (int64_t w = static_cast<int64_t>(blockIdx.x) * (blockDim.x / 32) + (threadIdx.x >> 5);
         w < nflag; w += wstride) {
        const int64_t col = flagged[w];
        const int si = find_seg<&MeshSeg::col_begin>(segs, nseg, col);
        const MeshSeg& s = segs[si];
        const GridDesc g = s.g;
        const int64_t lc = col - s.col_begin;
        const int i = static_cast<int>(lc % g.nx), j = static_cast<int>(lc / g.nx);
        const double zmin = dsub(g.corner[2], g.h);
        const double zmax = dadd(g.corner[2], dmul(static_cast<double>(g.nz + 1), g.h));
        const double cx = cell_center(g.corner[0], i, g.h);
        const double cy = cell_center(g.corner[1], j, g.h);
        const int64_t e0 = col_off[col], e1 = col_off[col + 1];
        unsigned exact_calls = 0;
        int limit = INT_MAX;  // crossings of triangles with id < limit are kept
        for (int attempt = 0; attempt < 7; ++attempt) {
            double x = cx, y = cy;
            if (attempt > 0) {
                x = dadd(cx, dmul(c_nudge[attempt - 1][0], g.h));
                y = dadd(cy, dmul(c_nudge[attempt - 1][1], g.h));
            }
            const d3 P{x, y, zmin}, Q{x, y, zmax};
            int first_graze = INT_MAX;
            for (int64_t e = e0 + lane; e < e1; e += 32) {
                d3 a, b, cc;
                const int t = col_list[e];
                load_tri(soup, t, a, b, cc);
                double hgt = 0.0;
                int r = column_tri<true, MODE>(P, Q, a, b, cc, &hgt, &exact_calls);
                if (r == 2) first_graze = min(first_graze, t);
                hs[e] = hgt;
                hv[e] = static_cast<uint8_t>(r == 1);
            }
            first_graze = warp_min(first_graze);
            if (first_graze == INT_MAX) {
                limit = INT_MAX;
                if (attempt > 0 && lane == 0) atomicAdd(&st->nudged_columns, 1ull);
                break;
            }
            limit = first_graze;  // if this is the last attempt, its partial result stays
            if (attempt == 6 && lane == 0) {
                atomicAdd(&st->nudged_columns, 1ull);
                atomicAdd(&st->exhausted_columns, 1ull);
            }
        }
        __syncwarp();
        long long ec = warp_sum(static_cast<long long>(exact_calls));
        if (lane == 0 && ec) atomicAdd(&st->exact_calls, static_cast<unsigned long long>(ec));
        // parity per cell: crossings of ids < limit strictly above the cell centre
        uint8_t* base = occ + s.vox_begin + static_cast<int64_t>(j) * g.nx + i;
        const int64_t kstride = static_cast<int64_t>(g.nx) * g.ny;
        for (int k = g.z0 + lane; k < g.z1; k += 32) {  // the slab's layers
            const double zc = cell_center(g.corner[2], k, g.h);
            int par = 0;
            for (int64_t e = e0; e < e1; ++e)
                if (hv[e] && col_list[e] < limit && hs[e] > zc) par ^= 1;
            base[(k - g.z0) * kstride] = static_cast<uint8_t>(par);
        }
    }
}

}  // namespace

void launch_tri_prep(const MeshSeg* segs, int nseg, int64_t ntris, const double* pts,
                     const int* tris, double* soup, int4* xybox, int64_t* pairs, cudaStream_t st) {
    if (ntris == 0) return;
    k_tri_prep<<<static_cast<unsigned>((ntris + 255) / 256), 256, 0, st>>>(segs, nseg, ntris, pts,
                                                                          tris, soup, xybox, pairs);
    CMG_LAUNCH();
}

void launch_col_pairs(bool fill, const MeshSeg* segs, int nseg, int64_t ntris, const int4* xybox,
                      const int64_t* pair_off, int* colcnt, const int64_t* col_off, int* col_list,
                      int grid, cudaStream_t st) {
    if (ntris == 0) return;
    if (fill)
        k_col_pairs<true><<<grid, 256, 0, st>>>(segs, nseg, ntris, xybox, pair_off, colcnt, col_off,
                                                col_list);
    else
        k_col_pairs<false><<<grid, 256, 0, st>>>(segs, nseg, ntris, xybox, pair_off, colcnt, col_off,
                                                 col_list);
    CMG_LAUNCH();
}

void launch_occ_filter(int mode, const MeshSeg* segs, int nseg, int64_t nrows, const double* soup,
                       const int64_t* col_off, const int* col_list, uint8_t* occ, int64_t* flagged,
                       Stats* stats, cudaStream_t st) {
    if (nrows == 0) return;
    if (mode == kPredExact)
        k_occ_filter<kPredExact><<<static_cast<unsigned>(nrows), kOccThreads, 0, st>>>(
            segs, nseg, soup, col_off, col_list, occ, flagged, stats);
    else
        k_occ_filter<kPredCompat><<<static_cast<unsigned>(nrows), kOccThreads, 0, st>>>(
            segs, nseg, soup, col_off, col_list, occ, flagged, stats);
    CMG_LAUNCH();
}

void launch_occ_exact(int mode, const MeshSeg* segs, int nseg, const double* soup,
                      const int64_t* col_off, const int* col_list, const int64_t* flagged,
                      double* hs, uint8_t* hv, uint8_t* occ, Stats* stats, int grid,
                      cudaStream_t st) {
    if (mode == kPredExact)
        k_occ_exact<kPredExact><<<grid, 128, 0, st>>>(segs, nseg, soup, col_off, col_list, flagged,
                                                      hs, hv, occ, stats);
    else
        k_occ_exact<kPredCompat><<<grid, 128, 0, st>>>(segs, nseg, soup, col_off, col_list, flagged,
                                                       hs, hv, occ, stats);
    CMG_LAUNCH();
}

int occ_row_cols() { return kRowCols; }

}  // namespace cmg::gpu
