// detect.cu — self-intersections of a triangulated PLC surface on the GPU.
//
// Replaces cmg::detect::self_intersections (src/detect/self_intersection.cpp:150-188),
// which tests every pair of fan triangles i < j that share no vertex index with the
// Guigue-Devillers orientation test (O. Devillers, P. Guigue, INRIA RR-4488, 2002),
// every decision a sign of the reference's robust::orient3d (the rounded determinant
// unless exactly zero, then the exact sign; coplanar pairs do not cross). Here:
//   1. broad phase: two triangles that cross share a point, so their bounding boxes
//      (exact double min/max) overlap; triangles are binned on a uniform grid by box,
//      and a pair is examined only in the cell that holds the low corner of the
//      intersection of the two boxes, so each candidate pair is seen exactly once;
//   2. narrow phase: the same orientation decisions on the device (o3d_fast in the
//      reference order, the exact sign when it is zero);
//   3. the crossing pairs are sorted to the reference's (i, j) order on the host, and
//      their rows (facets, corners) gathered on the device.
// The facets are fanned on the device and the surface's extent reduced there, each
// stage's buffers sized once its sizes are known (nothing is uploaded twice).
// The pair set does not depend on the grid, so the result is deterministic.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <vector>

#include "cmg_device.cuh"
#include "cmg_exact.cuh"
#include "cmg_util.h"
#include "engine_kernels.h"

namespace cmg::gpu {

namespace {

struct DetGrid {
    double lo[3];
    double cs;
    int n[3];
};

__device__ __forceinline__ int cell_of(double x, double lo, double cs, int n) {
    const double f = floor((x - lo) / cs);
    const int c = f < 0.0 ? 0 : (f >= n ? n - 1 : static_cast<int>(f));
    return c;
}

__device__ __forceinline__ int osign(const d3& a, const d3& b, const d3& c, const d3& d) {
    const double v = o3d_fast(a, b, c, d, nullptr);
    if (v != 0.0) return v > 0.0 ? 1 : -1;
    return exact::orient3d_sign(a, b, c, d);
}

__device__ bool gd_interval(const d3& p1, const d3& q1, const d3& r1, const d3& p2, const d3& q2,
                            const d3& r2) {
    if (osign(q2, p2, p1, q1) > 0) return false;
    if (osign(r2, p2, r1, p1) > 0) return false;
    return true;
}

// Triangle 2's vertex signs (sp, sq, sr) with respect to triangle 1's plane; p1 alone
// on its side of plane 2 after the caller's rotation.
__device__ bool gd_core(const d3& p1, const d3& q1, const d3& r1, const d3& p2, const d3& q2,
                        const d3& r2, int sp, int sq, int sr) {
    if (sp > 0) {
        if (sq > 0) return gd_interval(p1, r1, q1, r2, p2, q2);
        if (sr > 0) return gd_interval(p1, r1, q1, q2, r2, p2);
        return gd_interval(p1, q1, r1, p2, q2, r2);
    }
    if (sp < 0) {
        if (sq < 0) return gd_interval(p1, q1, r1, r2, p2, q2);
        if (sr < 0) return gd_interval(p1, q1, r1, q2, r2, p2);
        return gd_interval(p1, r1, q1, p2, q2, r2);
    }
    if (sq > 0) {
        if (sr >= 0) return gd_interval(p1, r1, q1, q2, r2, p2);
        return gd_interval(p1, q1, r1, p2, q2, r2);
    }
    if (sq < 0) {
        if (sr > 0) return gd_interval(p1, q1, r1, q2, r2, p2);
        return gd_interval(p1, r1, q1, p2, q2, r2);
    }
    if (sr > 0) return gd_interval(p1, q1, r1, r2, p2, q2);
    if (sr < 0) return gd_interval(p1, r1, q1, r2, p2, q2);
    return false;  // coplanar
}

__device__ bool tri_tri_cross(const d3& p1, const d3& q1, const d3& r1, const d3& p2, const d3& q2,
                              const d3& r2) {
    const int a = osign(p1, p2, q2, r2), b = osign(q1, p2, q2, r2), c = osign(r1, p2, q2, r2);
    if (a * b > 0 && a * c > 0) return false;
    const int d = osign(p2, q1, r1, p1), e = osign(q2, q1, r1, p1), f = osign(r2, q1, r1, p1);
    if (d * e > 0 && d * f > 0) return false;
    if (a > 0) {
        if (b > 0) return gd_core(r1, p1, q1, p2, r2, q2, d, f, e);
        if (c > 0) return gd_core(q1, r1, p1, p2, r2, q2, d, f, e);
        return gd_core(p1, q1, r1, p2, q2, r2, d, e, f);
    }
    if (a < 0) {
        if (b < 0) return gd_core(r1, p1, q1, p2, q2, r2, d, e, f);
        if (c < 0) return gd_core(q1, r1, p1, p2, q2, r2, d, e, f);
        return gd_core(p1, q1, r1, p2, r2, q2, d, f, e);
    }
    if (b < 0) {
        if (c >= 0) return gd_core(q1, r1, p1, p2, r2, q2, d, f, e);
        return gd_core(p1, q1, r1, p2, q2, r2, d, e, f);
    }
    if (b > 0) {
        if (c > 0) return gd_core(p1, q1, r1, p2, r2, q2, d, f, e);
        return gd_core(q1, r1, p1, p2, q2, r2, d, e, f);
    }
    if (c > 0) return gd_core(r1, p1, q1, p2, q2, r2, d, e, f);
    if (c < 0) return gd_core(r1, p1, q1, p2, r2, q2, d, f, e);
    return false;  // coplanar
}

// Boxes of the valid triangles (an index outside [0, npts) marks a triangle the
// reference skips) and their cell counts.
__global__ void k_det_boxes(int64_t ntris, const int* __restrict__ tris, const double* __restrict__ pts,
                            int64_t npts, DetGrid G, double* __restrict__ box, int* __restrict__ cnt) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= ntris) return;
    const int i0 = tris[3 * t], i1 = tris[3 * t + 1], i2 = tris[3 * t + 2];
    if (i0 < 0 || i0 >= npts || i1 < 0 || i1 >= npts || i2 < 0 || i2 >= npts) {
        cnt[t] = 0;
        return;
    }
    int64_t c = 1;
    for (int q = 0; q < 3; ++q) {
        const double a = pts[3 * i0 + q], b = pts[3 * i1 + q], d = pts[3 * i2 + q];
        const double lo = fmin(a, fmin(b, d)), hi = fmax(a, fmax(b, d));
        box[6 * t + q] = lo;
        box[6 * t + 3 + q] = hi;
        c *= cell_of(hi, G.lo[q], G.cs, G.n[q]) - cell_of(lo, G.lo[q], G.cs, G.n[q]) + 1;
    }
    cnt[t] = static_cast<int>(c);
}

// (cell, triangle) entries: count per cell (FILL = false) or write (FILL = true).
template <bool FILL>
__global__ void k_det_bin(int64_t ntris, const int* __restrict__ cnt, const double* __restrict__ box,
                          DetGrid G, int* __restrict__ cellcnt, const int64_t* __restrict__ celloff,
                          int* __restrict__ list) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= ntris || cnt[t] == 0) return;
    int c0[3], c1[3];
    for (int q = 0; q < 3; ++q) {
        c0[q] = cell_of(box[6 * t + q], G.lo[q], G.cs, G.n[q]);
        c1[q] = cell_of(box[6 * t + 3 + q], G.lo[q], G.cs, G.n[q]);
    }
    for (int z = c0[2]; z <= c1[2]; ++z)
        for (int y = c0[1]; y <= c1[1]; ++y)
            for (int x = c0[0]; x <= c1[0]; ++x) {
                const int64_t cell = (static_cast<int64_t>(z) * G.n[1] + y) * G.n[0] + x;
                const int slot = atomicAdd(&cellcnt[cell], 1);
                if (FILL) list[celloff[cell] + slot] = static_cast<int>(t);
            }
}

// One thread per (cell, entry): the pairs with the cell's later entries.
__global__ void k_det_pairs(int64_t nentries, const int* __restrict__ list, const int64_t* __restrict__ celloff,
                            int64_t ncell, const double* __restrict__ box, DetGrid G,
                            const int* __restrict__ tris, const double* __restrict__ pts,
                            long long* __restrict__ out, unsigned long long* __restrict__ nout,
                            unsigned long long cap) {
    const int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= nentries) return;
    // the cell of entry e: the last c with celloff[c] <= e
    int64_t lo = 0, hi = ncell - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (celloff[mid] <= e) lo = mid;
        else hi = mid - 1;
    }
    const int64_t cell = lo, end = celloff[cell + 1];
    const int cx = static_cast<int>(cell % G.n[0]);
    const int cy = static_cast<int>((cell / G.n[0]) % G.n[1]);
    const int cz = static_cast<int>(cell / (static_cast<int64_t>(G.n[0]) * G.n[1]));
    const int t0 = list[e];
    for (int64_t f = e + 1; f < end; ++f) {
        const int t1 = list[f];
        const int a = min(t0, t1), b = max(t0, t1);
        const double* A = box + 6 * static_cast<int64_t>(a);
        const double* B = box + 6 * static_cast<int64_t>(b);
        bool overlap = true;
        int cc[3];
        for (int q = 0; q < 3; ++q) {
            overlap = overlap && A[q] <= B[3 + q] && B[q] <= A[3 + q];
            cc[q] = cell_of(fmax(A[q], B[q]), G.lo[q], G.cs, G.n[q]);
        }
        if (!overlap || cc[0] != cx || cc[1] != cy || cc[2] != cz) continue;
        const int* U = tris + 3 * static_cast<int64_t>(a);
        const int* V = tris + 3 * static_cast<int64_t>(b);
        bool shared = false;
        for (int x = 0; x < 3; ++x)
            for (int y = 0; y < 3; ++y) shared = shared || U[x] == V[y];
        if (shared) continue;
        auto P = [&](int i) { return d3{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]}; };
        if (tri_tri_cross(P(U[0]), P(U[1]), P(U[2]), P(V[0]), P(V[1]), P(V[2]))) {
            const unsigned long long k = atomicAdd(nout, 1ull);
            if (k < cap) out[k] = (static_cast<long long>(a) << 32) | static_cast<long long>(b);
        }
    }
}

// ---- fan triangulation of the facets, extent of the surface, result rows ----------

__global__ void k_det_fan_count(const size_t* __restrict__ foff, int64_t nf, int64_t* __restrict__ cnt) {
    const int64_t f = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int64_t n = static_cast<int64_t>(foff[f + 1] - foff[f]);
    cnt[f] = n >= 3 ? n - 2 : 0;
}

// Fan triangles (v0, v[i-1], v[i]) of facet f at toff[f] + i - 2, with their facet.
__global__ void k_det_fan_emit(const size_t* __restrict__ foff, const int* __restrict__ fidx, int64_t nf,
                               const int64_t* __restrict__ toff, int* __restrict__ tris,
                               int* __restrict__ facet) {
    const int64_t f = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const size_t o = foff[f];
    const int64_t n = static_cast<int64_t>(foff[f + 1] - o);
    for (int64_t i = 2; i < n; ++i) {
        const int64_t t = toff[f] + i - 2;
        tris[3 * t] = fidx[o];
        tris[3 * t + 1] = fidx[o + i - 1];
        tris[3 * t + 2] = fidx[o + i];
        facet[t] = static_cast<int>(f);
    }
}

// Order-preserving integer image of a double (min / max commute with it).
__device__ __forceinline__ unsigned long long ord_of(double x) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ inline double from_ord(unsigned long long o) {
    const unsigned long long b = (o >> 63) ? (o & 0x7fffffffffffffffull) : ~o;
    double d;
    memcpy(&d, &b, sizeof(d));
    return d;
}

struct Extent {
    unsigned long long lo[3], hi[3];  // ord_of images
    double ext_sum;                   // sum of the valid triangles' largest box extents
    unsigned long long nvalid;
    int nonfinite;
};

// Boxes of the valid triangles (indices inside the points), and the surface's extent.
__global__ void __launch_bounds__(256) k_det_extent(int64_t ntris, const int* __restrict__ tris,
                                                    const double* __restrict__ pts, int64_t npts,
                                                    double* __restrict__ box, int* __restrict__ valid,
                                                    Extent* __restrict__ ext) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0ull, 0ull, 0ull};
    double es = 0.0;
    bool ok = false, bad = false;
    if (t < ntris) {
        const int i0 = tris[3 * t], i1 = tris[3 * t + 1], i2 = tris[3 * t + 2];
        ok = i0 >= 0 && i0 < npts && i1 >= 0 && i1 < npts && i2 >= 0 && i2 < npts;
        valid[t] = ok ? 1 : 0;
        if (ok) {
            for (int q = 0; q < 3; ++q) {
                const double a = pts[3 * static_cast<int64_t>(i0) + q], b = pts[3 * static_cast<int64_t>(i1) + q],
                             d = pts[3 * static_cast<int64_t>(i2) + q];
                bad = bad || !isfinite(a) || !isfinite(b) || !isfinite(d);
                const double l = fmin(a, fmin(b, d)), h = fmax(a, fmax(b, d));
                box[6 * t + q] = l;
                box[6 * t + 3 + q] = h;
                lo[q] = ord_of(l);
                hi[q] = ord_of(h);
                es = fmax(es, h - l);
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        for (int q = 0; q < 3; ++q) {
            const unsigned long long l = __shfl_xor_sync(0xffffffffu, lo[q], o);
            const unsigned long long h = __shfl_xor_sync(0xffffffffu, hi[q], o);
            lo[q] = l < lo[q] ? l : lo[q];
            hi[q] = h > hi[q] ? h : hi[q];
        }
        es += __shfl_xor_sync(0xffffffffu, es, o);
    }
    const unsigned nv = __popc(__ballot_sync(0xffffffffu, ok));
    const bool anybad = __any_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0 && nv) {
        for (int q = 0; q < 3; ++q) {
            atomicMin(&ext->lo[q], lo[q]);
            atomicMax(&ext->hi[q], hi[q]);
        }
        atomicAdd(&ext->ext_sum, es);
        atomicAdd(&ext->nvalid, static_cast<unsigned long long>(nv));
        if (anybad) atomicExch(&ext->nonfinite, 1);
    }
}

__global__ void k_det_count(int64_t ntris, const int* __restrict__ valid, const double* __restrict__ box,
                            DetGrid G, int* __restrict__ cnt) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= ntris) return;
    if (!valid[t]) {
        cnt[t] = 0;
        return;
    }
    int64_t c = 1;
    for (int q = 0; q < 3; ++q)
        c *= cell_of(box[6 * t + 3 + q], G.lo[q], G.cs, G.n[q]) - cell_of(box[6 * t + q], G.lo[q], G.cs, G.n[q]) + 1;
    cnt[t] = static_cast<int>(c);
}

// Rows of the sorted pairs: facet_a, facet_b, triangle a's corners, triangle b's.
__global__ void k_det_rows(int64_t np, const long long* __restrict__ keys, const int* __restrict__ tris,
                           const int* __restrict__ facet, int* __restrict__ rows) {
    const int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const int64_t a = keys[p] >> 32, b = keys[p] & 0xffffffffll;
    int* r = rows + 8 * p;
    r[0] = facet[a];
    r[1] = facet[b];
    for (int k = 0; k < 3; ++k) {
        r[2 + k] = tris[3 * a + k];
        r[5 + k] = tris[3 * b + k];
    }
}

}  // namespace

namespace {
float g_last_ms = 0.f;  // device time of the last call's broad + narrow phase
}

float self_intersections_last_ms() { return g_last_ms; }

// Sizes one arena for a plan (the plan's pointers are taken again after a growth).
template <typename Plan>
void size_arena(Arena& A, Plan&& plan) {
    A.clear_need();
    plan();
    if (A.overflowed()) {
        A.reserve(A.need());
        plan();
    }
}

void self_intersections(const double* h_pts, int64_t npts, const int* h_fidx, int64_t nidx,
                        const size_t* h_foff, int64_t nfacets, std::vector<int>& rows,
                        cudaStream_t st) {
    rows.clear();
    g_last_ms = 0.f;
    if (nfacets <= 0 || npts <= 0) return;
    if (nidx >= (int64_t(1) << 31)) throw std::invalid_argument("self_intersections: too many facet vertices");
    static std::mutex mu;
    // one arena per stage, each sized when its sizes are known, so that no earlier
    // stage's buffers move: inputs, triangles, cells, entries, output, rows
    static Arena A_in, A_tri, A_cell, A_list, A_out, A_rows;
    static cudaEvent_t ev[2] = {nullptr, nullptr};
    std::lock_guard<std::mutex> lk(mu);
    if (!ev[0])
        for (cudaEvent_t& e : ev) CMG_CUDA(cudaEventCreate(&e));
    const int64_t nf = nfacets;
    double* d_pts;
    int* d_fidx;
    size_t* d_foff;
    int64_t *fcnt, *toff, *stmp_f;
    Extent* ext;
    size_arena(A_in, [&]() {
        A_in.reset();
        d_pts = A_in.take<double>(3 * npts);
        d_fidx = A_in.take<int>(std::max<int64_t>(nidx, 1));
        d_foff = A_in.take<size_t>(nf + 1);
        fcnt = A_in.take<int64_t>(nf);
        toff = A_in.take<int64_t>(nf + 1);
        stmp_f = A_in.take<int64_t>(scan_tmp_elems(nf));
        ext = A_in.take<Extent>(1);
    });
    CMG_CUDA(cudaMemcpyAsync(d_pts, h_pts, sizeof(double) * 3 * npts, cudaMemcpyHostToDevice, st));
    if (nidx) CMG_CUDA(cudaMemcpyAsync(d_fidx, h_fidx, sizeof(int) * nidx, cudaMemcpyHostToDevice, st));
    CMG_CUDA(cudaMemcpyAsync(d_foff, h_foff, sizeof(size_t) * (nf + 1), cudaMemcpyHostToDevice, st));
    CMG_CUDA(cudaEventRecord(ev[0], st));
    const unsigned gf = static_cast<unsigned>((nf + 255) / 256);
    k_det_fan_count<<<gf, 256, 0, st>>>(d_foff, nf, fcnt);
    CMG_LAUNCH();
    exclusive_scan(fcnt, toff, nf, stmp_f, st);
    int64_t ntris = 0;
    CMG_CUDA(cudaMemcpyAsync(&ntris, toff + nf, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CMG_CUDA(cudaStreamSynchronize(st));
    if (ntris < 2) return;
    if (ntris >= (int64_t(1) << 31)) throw std::invalid_argument("self_intersections: too many triangles");

    int *tris, *facet, *valid, *cnt;
    double* box;
    size_arena(A_tri, [&]() {
        A_tri.reset();
        tris = A_tri.take<int>(3 * ntris);
        facet = A_tri.take<int>(ntris);
        valid = A_tri.take<int>(ntris);
        cnt = A_tri.take<int>(ntris);
        box = A_tri.take<double>(6 * ntris);
    });
    const unsigned gt = static_cast<unsigned>((ntris + 255) / 256);
    k_det_fan_emit<<<gf, 256, 0, st>>>(d_foff, d_fidx, nf, toff, tris, facet);
    CMG_LAUNCH();
    CMG_CUDA(cudaMemsetAsync(ext, 0, sizeof(Extent), st));
    CMG_CUDA(cudaMemsetAsync(ext->lo, 0xff, sizeof(ext->lo), st));
    k_det_extent<<<gt, 256, 0, st>>>(ntris, tris, d_pts, npts, box, valid, ext);
    CMG_LAUNCH();
    Extent h{};
    CMG_CUDA(cudaMemcpyAsync(&h, ext, sizeof(Extent), cudaMemcpyDeviceToHost, st));
    CMG_CUDA(cudaStreamSynchronize(st));
    if (h.nvalid < 2) return;
    if (h.nonfinite) throw std::invalid_argument("self_intersections: non-finite coordinate");
    // grid over the valid triangles' points: cell edge ~ twice the mean box extent
    double lo[3], hi[3];
    for (int q = 0; q < 3; ++q) {
        lo[q] = from_ord(h.lo[q]);
        hi[q] = from_ord(h.hi[q]);
    }
    DetGrid G{};
    double span = 0.0;
    for (int q = 0; q < 3; ++q) span = std::max(span, hi[q] - lo[q]);
    double cs = std::max(2.0 * h.ext_sum / static_cast<double>(h.nvalid), span / 2048.0);
    if (!(cs > 0.0)) cs = 1.0;
    for (;;) {
        int64_t total = 1;
        for (int q = 0; q < 3; ++q) {
            G.n[q] = std::max(1, static_cast<int>(std::ceil((hi[q] - lo[q]) / cs)));
            total *= G.n[q];
        }
        if (total <= (int64_t(1) << 24)) break;
        cs *= 1.5;
    }
    for (int q = 0; q < 3; ++q) G.lo[q] = lo[q];
    G.cs = cs;
    const int64_t ncell = static_cast<int64_t>(G.n[0]) * G.n[1] * G.n[2];

    int* cellcnt;
    int64_t *celloff, *stmp;
    size_arena(A_cell, [&]() {
        A_cell.reset();
        cellcnt = A_cell.take<int>(ncell);
        celloff = A_cell.take<int64_t>(ncell + 1);
        stmp = A_cell.take<int64_t>(scan_tmp_elems(ncell + 1));
    });
    k_det_count<<<gt, 256, 0, st>>>(ntris, valid, box, G, cnt);
    CMG_LAUNCH();
    CMG_CUDA(cudaMemsetAsync(cellcnt, 0, sizeof(int) * ncell, st));
    k_det_bin<false><<<gt, 256, 0, st>>>(ntris, cnt, box, G, cellcnt, nullptr, nullptr);
    CMG_LAUNCH();
    exclusive_scan(cellcnt, celloff, ncell, stmp, st);
    int64_t nent = 0;
    CMG_CUDA(cudaMemcpyAsync(&nent, celloff + ncell, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CMG_CUDA(cudaStreamSynchronize(st));
    int* list;
    size_arena(A_list, [&]() {
        A_list.reset();
        list = A_list.take<int>(std::max<int64_t>(nent, 1));
    });
    CMG_CUDA(cudaMemsetAsync(cellcnt, 0, sizeof(int) * ncell, st));
    k_det_bin<true><<<gt, 256, 0, st>>>(ntris, cnt, box, G, cellcnt, celloff, list);
    CMG_LAUNCH();
    unsigned long long cap = 1 << 16;
    for (int attempt = 0; attempt < 2; ++attempt) {
        long long* out;
        unsigned long long* nout;
        size_arena(A_out, [&]() {
            A_out.reset();
            out = A_out.take<long long>(cap);
            nout = A_out.take<unsigned long long>(1);
        });
        CMG_CUDA(cudaMemsetAsync(nout, 0, sizeof(unsigned long long), st));
        if (nent > 0) {
            k_det_pairs<<<static_cast<unsigned>((nent + 127) / 128), 128, 0, st>>>(
                nent, list, celloff, ncell, box, G, tris, d_pts, out, nout, cap);
            CMG_LAUNCH();
        }
        CMG_CUDA(cudaEventRecord(ev[1], st));
        unsigned long long found = 0;
        CMG_CUDA(cudaMemcpyAsync(&found, nout, sizeof(found), cudaMemcpyDeviceToHost, st));
        CMG_CUDA(cudaStreamSynchronize(st));
        CMG_CUDA(cudaEventElapsedTime(&g_last_ms, ev[0], ev[1]));
        if (found <= cap) {
            if (found == 0) return;
            // the reference's (i, j) order, then the rows gathered on the device
            std::vector<long long> keys(found);
            CMG_CUDA(cudaMemcpy(keys.data(), out, sizeof(long long) * found, cudaMemcpyDeviceToHost));
            std::sort(keys.begin(), keys.end());
            long long* dkeys;
            int* drows;
            size_arena(A_rows, [&]() {
                A_rows.reset();
                dkeys = A_rows.take<long long>(found);
                drows = A_rows.take<int>(8 * found);
            });
            CMG_CUDA(cudaMemcpyAsync(dkeys, keys.data(), sizeof(long long) * found, cudaMemcpyHostToDevice, st));
            k_det_rows<<<static_cast<unsigned>((found + 255) / 256), 256, 0, st>>>(
                static_cast<int64_t>(found), dkeys, tris, facet, drows);
            CMG_LAUNCH();
            rows.resize(8 * found);
            CMG_CUDA(cudaMemcpyAsync(rows.data(), drows, sizeof(int) * 8 * found, cudaMemcpyDeviceToHost, st));
            CMG_CUDA(cudaStreamSynchronize(st));
            return;
        }
        cap = found;  // exact count known: one more pass with room for every pair
    }
    throw std::runtime_error("self_intersections: output sizing failed");
}

}  // namespace cmg::gpu
