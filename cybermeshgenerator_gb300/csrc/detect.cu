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
//   3. the crossing pairs are sorted to the reference's (i, j) order on the host.
// The pair set does not depend on the grid, so the result is deterministic.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
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

}  // namespace

namespace {
float g_last_ms = 0.f;  // device time of the last call's broad + narrow phase
}

float self_intersections_last_ms() { return g_last_ms; }

void self_intersections(const double* h_pts, int64_t npts, const int* h_tris, int64_t ntris,
                        std::vector<std::pair<int, int>>& pairs, cudaStream_t st) {
    pairs.clear();
    g_last_ms = 0.f;
    if (ntris < 2) return;
    if (ntris >= (int64_t(1) << 31)) throw std::invalid_argument("self_intersections: too many triangles");
    // grid over the valid triangles' points: cell edge ~ twice the mean box extent
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    double ext_sum = 0.0;
    int64_t nvalid = 0;
    for (int64_t t = 0; t < ntris; ++t) {
        const int* T = h_tris + 3 * t;
        if (T[0] < 0 || T[0] >= npts || T[1] < 0 || T[1] >= npts || T[2] < 0 || T[2] >= npts) continue;
        double e = 0.0;
        for (int q = 0; q < 3; ++q) {
            const double a = h_pts[3 * T[0] + q], b = h_pts[3 * T[1] + q], c = h_pts[3 * T[2] + q];
            const double l = std::min(a, std::min(b, c)), h = std::max(a, std::max(b, c));
            lo[q] = std::min(lo[q], l);
            hi[q] = std::max(hi[q], h);
            e = std::max(e, h - l);
        }
        ext_sum += e;
        ++nvalid;
    }
    if (nvalid < 2) return;
    for (int q = 0; q < 3; ++q)
        if (!std::isfinite(lo[q]) || !std::isfinite(hi[q]))
            throw std::invalid_argument("self_intersections: non-finite coordinate");
    DetGrid G{};
    double span = 0.0;
    for (int q = 0; q < 3; ++q) span = std::max(span, hi[q] - lo[q]);
    double cs = std::max(2.0 * ext_sum / nvalid, span / 2048.0);
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

    static std::mutex mu;
    static Arena arena;  // grows; the calls are serialised
    std::lock_guard<std::mutex> lk(mu);
    Arena& A = arena;
    double *d_pts, *box;
    int *d_tris, *cnt, *cellcnt, *list;
    int64_t *celloff, *stmp;
    long long* out;
    unsigned long long* nout;
    int64_t nent = 0;
    unsigned long long cap = 1 << 16;
    auto plan = [&](int64_t ent) {
        A.reset();
        d_pts = A.take<double>(3 * npts);
        d_tris = A.take<int>(3 * ntris);
        box = A.take<double>(6 * ntris);
        cnt = A.take<int>(ntris);
        cellcnt = A.take<int>(ncell);
        celloff = A.take<int64_t>(ncell + 1);
        stmp = A.take<int64_t>(scan_tmp_elems(std::max(ncell, ntris) + 1));
        list = A.take<int>(std::max<int64_t>(ent, 1));
        out = A.take<long long>(cap);
        nout = A.take<unsigned long long>(1);
    };
    auto sized = [&](int64_t ent) {
        A.clear_need();
        plan(ent);
        if (A.overflowed()) {
            A.reserve(A.need());
            plan(ent);
        }
    };
    sized(0);
    CMG_CUDA(cudaMemcpyAsync(d_pts, h_pts, sizeof(double) * 3 * npts, cudaMemcpyHostToDevice, st));
    CMG_CUDA(cudaMemcpyAsync(d_tris, h_tris, sizeof(int) * 3 * ntris, cudaMemcpyHostToDevice, st));
    const unsigned gt = static_cast<unsigned>((ntris + 255) / 256);
    k_det_boxes<<<gt, 256, 0, st>>>(ntris, d_tris, d_pts, npts, G, box, cnt);
    CMG_LAUNCH();
    CMG_CUDA(cudaMemsetAsync(cellcnt, 0, sizeof(int) * ncell, st));
    k_det_bin<false><<<gt, 256, 0, st>>>(ntris, cnt, box, G, cellcnt, nullptr, nullptr);
    CMG_LAUNCH();
    exclusive_scan(cellcnt, celloff, ncell, stmp, st);
    CMG_CUDA(cudaMemcpyAsync(&nent, celloff + ncell, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CMG_CUDA(cudaStreamSynchronize(st));
    cudaEvent_t e0, e1;
    CMG_CUDA(cudaEventCreate(&e0));
    CMG_CUDA(cudaEventCreate(&e1));
    struct Ev {
        cudaEvent_t a, b;
        ~Ev() {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } ev{e0, e1};
    for (int attempt = 0; attempt < 2; ++attempt) {
        // the entry list (and, on a second attempt, the output) sized; inputs re-uploaded
        // because a grown arena moved them
        sized(nent);
        CMG_CUDA(cudaMemcpyAsync(d_pts, h_pts, sizeof(double) * 3 * npts, cudaMemcpyHostToDevice, st));
        CMG_CUDA(cudaMemcpyAsync(d_tris, h_tris, sizeof(int) * 3 * ntris, cudaMemcpyHostToDevice, st));
        CMG_CUDA(cudaEventRecord(e0, st));
        k_det_boxes<<<gt, 256, 0, st>>>(ntris, d_tris, d_pts, npts, G, box, cnt);
        CMG_LAUNCH();
        CMG_CUDA(cudaMemsetAsync(cellcnt, 0, sizeof(int) * ncell, st));
        k_det_bin<false><<<gt, 256, 0, st>>>(ntris, cnt, box, G, cellcnt, nullptr, nullptr);
        CMG_LAUNCH();
        exclusive_scan(cellcnt, celloff, ncell, stmp, st);
        CMG_CUDA(cudaMemsetAsync(cellcnt, 0, sizeof(int) * ncell, st));
        k_det_bin<true><<<gt, 256, 0, st>>>(ntris, cnt, box, G, cellcnt, celloff, list);
        CMG_LAUNCH();
        CMG_CUDA(cudaMemsetAsync(nout, 0, sizeof(unsigned long long), st));
        if (nent > 0) {
            k_det_pairs<<<static_cast<unsigned>((nent + 127) / 128), 128, 0, st>>>(
                nent, list, celloff, ncell, box, G, d_tris, d_pts, out, nout, cap);
            CMG_LAUNCH();
        }
        CMG_CUDA(cudaEventRecord(e1, st));
        unsigned long long found = 0;
        CMG_CUDA(cudaMemcpyAsync(&found, nout, sizeof(found), cudaMemcpyDeviceToHost, st));
        CMG_CUDA(cudaStreamSynchronize(st));
        CMG_CUDA(cudaEventElapsedTime(&g_last_ms, e0, e1));
        if (found <= cap) {
            std::vector<long long> h(found);
            if (found)
                CMG_CUDA(cudaMemcpy(h.data(), out, sizeof(long long) * found, cudaMemcpyDeviceToHost));
            std::sort(h.begin(), h.end());
            pairs.reserve(found);
            for (long long k : h) pairs.emplace_back(static_cast<int>(k >> 32), static_cast<int>(k & 0xffffffff));
            return;
        }
        cap = found;  // exact count known: one more pass with room for every pair
    }
    throw std::runtime_error("self_intersections: output sizing failed");
}

}  // namespace cmg::gpu
