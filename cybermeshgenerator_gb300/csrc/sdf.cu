// sdf.cu — signed distance field: nearest boundary triangle per cell.
//
// The reference computes, per cell centre, the minimum of point_tri_dist2
// (Ericson, src/voxelize/voxelize.cpp:202-247) over the triangles found by a
// Chebyshev ring search of 3-D buckets (:251-326); its pruning is exact, so the
// result equals the brute-force minimum over all triangles. Here:
//
//   k_sdf_tri_prep   centroid c_t, radius e_t = max |v - c_t| (rounded up), bin of
//                    c_t in the brick grid; triangles larger than two bricks (or
//                    degenerate) go to a per-mesh "always considered" list
//   k_bin_fill       bin -> triangle CSR
//   k_brick_walk     one CTA per brick: a ring walk over bins gives an upper bound
//                    U on the distance from the brick centre to the surface, then
//                    the candidate list = every triangle whose lower bound
//                    |c - c_t| - e_t - r_B can be <= U + r_B (r_B = brick radius),
//                    with margins far above FP32 and FP64 rounding
//   k_sdf_fp64       one CTA per brick, candidates staged through shared memory;
//                    each thread owns voxels and evaluates Ericson in the reference
//                    operation order (FP64, no FMA): bit-identical to the reference
//   k_sdf_mixed      same walk in FP32 on brick-recentred coordinates (normals from
//                    FP64) with a stated error bound; cells within a band of the
//                    surface are re-evaluated in FP64 over the candidates whose
//                    FP32 distance is within twice the bound of the best, which
//                    reproduces the FP64 minimum exactly there.
// Both evaluation kernels skip a candidate for a whole warp when no lane's cells
// can reach it (bounding sphere of the triangle vs the current best).
#include <cuda_runtime.h>

#include <cfloat>
#include <climits>
#include <type_traits>

#include "cmg_device.cuh"
#include "cmg_sdf.cuh"
#include "cmg_seg.cuh"
#include "cmg_types.h"
#include "cmg_util.h"
#include "engine_kernels.h"

namespace cmg::gpu {

namespace {

using namespace sdf;
static_assert(sizeof(TriRec) == kTriRecBytes, "the workspace carves kTriRecBytes per record");

__device__ __forceinline__ float round_up_f(double x) { return __double2float_ru(x); }

// ------------------------------------------------------------------ triangle prep
// tinfo (float4 per triangle): centroid relative to the mesh grid corner (FP32,
// nearest) and the radius e_t rounded up (plus the rounding of the centroid).
__global__ void k_sdf_tri_prep(const MeshSeg* __restrict__ segs, int nseg, int64_t ntris,
                               const double* __restrict__ soup, float4* __restrict__ tinfo,
                               float4* __restrict__ tinfo_lo, TriRec* __restrict__ trec,
                               float4* __restrict__ tnorm,
                               float4* __restrict__ tlo, float4* __restrict__ thi,
                               int64_t* __restrict__ tbin, int* __restrict__ bincnt,
                               int* __restrict__ large_cnt, unsigned* __restrict__ emax_bits) {
    int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= ntris) return;
    const int si = find_seg<&MeshSeg::tri_begin>(segs, nseg, t);
    const MeshSeg& s = segs[si];
    d3 a, b, c;
    load_soup(soup, t, a, b, c);
    const double* K = s.g.corner;
    // centroid in FP64 (any rounding is covered by the radius padding below)
    double cx = (a.x + b.x + c.x) / 3.0, cy = (a.y + b.y + c.y) / 3.0, cz = (a.z + b.z + c.z) / 3.0;
    double r2 = 0.0;
    const d3 V[3] = {a, b, c};
    double lo[3] = {a.x, a.y, a.z}, hi[3] = {a.x, a.y, a.z};
    for (int k = 0; k < 3; ++k) {
        double dx = V[k].x - cx, dy = V[k].y - cy, dz = V[k].z - cz;
        r2 = fmax(r2, dx * dx + dy * dy + dz * dz);
        lo[0] = fmin(lo[0], V[k].x); hi[0] = fmax(hi[0], V[k].x);
        lo[1] = fmin(lo[1], V[k].y); hi[1] = fmax(hi[1], V[k].y);
        lo[2] = fmin(lo[2], V[k].z); hi[2] = fmax(hi[2], V[k].z);
    }
    float4 ci, cl;
    split2(cx - K[0], ci.x, cl.x);
    split2(cy - K[1], ci.y, cl.y);
    split2(cz - K[2], ci.z, cl.z);
    cl.w = 0.f;
    tinfo_lo[t] = cl;
    // radius: sqrt rounded up, padded for the FP32 centroid (|err| <= u*|c - K|*sqrt3)
    double pad = 2.0 * kU32 * (fabs(cx - K[0]) + fabs(cy - K[1]) + fabs(cz - K[2])) + 1e-300;
    ci.w = round_up_f(sqrt(r2) * (1.0 + 1e-12) + pad);
    tinfo[t] = ci;
    tlo[t] = make_float4(__double2float_rd(lo[0] - K[0]), __double2float_rd(lo[1] - K[1]),
                         __double2float_rd(lo[2] - K[2]), 0.f);
    thi[t] = make_float4(__double2float_ru(hi[0] - K[0]), __double2float_ru(hi[1] - K[1]),
                         __double2float_ru(hi[2] - K[2]), 0.f);
    // translation-invariant FP32 record (from FP64)
    double ux = b.x - a.x, uy = b.y - a.y, uz = b.z - a.z;
    double vx = c.x - a.x, vy = c.y - a.y, vz = c.z - a.z;
    double nx = uy * vz - uz * vy, ny = uz * vx - ux * vz, nz = ux * vy - uy * vx;
    bool degenerate = !(nx * nx + ny * ny + nz * nz > 0.0);
    {
        double nl = sqrt(nx * nx + ny * ny + nz * nz);
        double n3[3] = {0.0, 0.0, 0.0};
        if (nl > 0.0) { n3[0] = nx / nl; n3[1] = ny / nl; n3[2] = nz / nl; }
        // the FP64 path's plane bound: the unit normal in FP32 and a bound on its distance
        // from the exact one: the cross product of rounded edges errs by at most
        // 21 u |u| |v| (as a vector), which turns its direction by at most twice that
        // over |u x v|; then the normalisation and the FP32 rounding of the components
        const double lu = sqrt(ux * ux + uy * uy + uz * uz), lv = sqrt(vx * vx + vy * vy + vz * vz);
        const double en = nl > 0.0 ? 50.0 * kU64 * lu * lv / nl + 1.2e-7 : 0.0;
        if (tnorm)
            tnorm[t] = make_float4(static_cast<float>(n3[0]), static_cast<float>(n3[1]),
                                   static_cast<float>(n3[2]), round_up_f(en));
        // the mixed path's record in the triangle's frame: u along b - a (else along
        // c - a, else x), v from c - a by two Gram-Schmidt passes (so c = a + cx u +
        // cy v to FP64 rounding however thin the triangle), n = u x v
        double U[3], Vv[3], bx;
        const double lab = lu, lac = lv;
        if (lab > 0.0) { U[0] = ux / lab; U[1] = uy / lab; U[2] = uz / lab; bx = lab; }
        else if (lac > 0.0) { U[0] = vx / lac; U[1] = vy / lac; U[2] = vz / lac; bx = 0.0; }
        else { U[0] = 1.0; U[1] = 0.0; U[2] = 0.0; bx = 0.0; }
        double ccx = vx * U[0] + vy * U[1] + vz * U[2];
        double rx = vx - ccx * U[0], ry = vy - ccx * U[1], rz = vz - ccx * U[2];
        const double kk = rx * U[0] + ry * U[1] + rz * U[2];
        ccx += kk;
        rx -= kk * U[0]; ry -= kk * U[1]; rz -= kk * U[2];
        // a residual at the rounding level (exactly collinear vertices leave one along u)
        // carries no direction: the triangle is taken as collinear, which moves c by at
        // most 1e-9 of the triangle's size (far inside the stated FP32 error)
        double ccy = sqrt(rx * rx + ry * ry + rz * rz);
        if (!(ccy > 1e-9 * fmax(lab, lac))) ccy = 0.0;
        if (ccy > 0.0) {
            Vv[0] = rx / ccy; Vv[1] = ry / ccy; Vv[2] = rz / ccy;
        } else {
            // collinear: any unit vector across u (u x the axis least aligned with u)
            const int ax = fabs(U[0]) <= fabs(U[1]) && fabs(U[0]) <= fabs(U[2]) ? 0 : (fabs(U[1]) <= fabs(U[2]) ? 1 : 2);
            const double A[3] = {ax == 0 ? 1.0 : 0.0, ax == 1 ? 1.0 : 0.0, ax == 2 ? 1.0 : 0.0};
            double wx = A[1] * U[2] - A[2] * U[1], wy = A[2] * U[0] - A[0] * U[2], wz = A[0] * U[1] - A[1] * U[0];
            const double wl = sqrt(wx * wx + wy * wy + wz * wz);
            Vv[0] = wx / wl; Vv[1] = wy / wl; Vv[2] = wz / wl;
        }
        const double N[3] = {U[1] * Vv[2] - U[2] * Vv[1], U[2] * Vv[0] - U[0] * Vv[2], U[0] * Vv[1] - U[1] * Vv[0]};
        TriRec r;
        r.o0[0] = static_cast<float>(a.x - cx);
        r.o0[1] = static_cast<float>(a.y - cy);
        r.o0[2] = static_cast<float>(a.z - cz);
        for (int q = 0; q < 3; ++q) {
            r.nn[q] = static_cast<float>(N[q]);
            r.uu[q] = static_cast<float>(U[q]);
            r.vv[q] = static_cast<float>(Vv[q]);
        }
        // the triangle lies in the frame's plane (to FP64 rounding), every triangle has
        // one, and its FP32 normal is within the rounding of a unit vector (sqrt(3) u)
        r.nerr = 2.4e-7f;
        r.bx = static_cast<float>(bx);
        r.cx = static_cast<float>(ccx);
        r.cy = static_cast<float>(ccy);
        r.e1x = static_cast<float>(ccx - bx);
        r.ib = bx > 0.0 ? static_cast<float>(1.0 / bx) : 0.f;
        const double l1 = (ccx - bx) * (ccx - bx) + ccy * ccy, l2 = ccx * ccx + ccy * ccy;
        r.inv1 = l1 > 0.0 ? static_cast<float>(1.0 / l1) : 0.f;
        r.inv2 = l2 > 0.0 ? static_cast<float>(1.0 / l2) : 0.f;
        r.ok = bx > 0.0 && ccy > 0.0 ? 1.f : 0.f;
        r.pad_[0] = r.pad_[1] = r.pad_[2] = 0.f;
        trec[t] = r;
    }
    // the mesh's coordinate scale max |v - K| (rounded up), per segment, for the
    // FP32 tolerances; k_seg_finish folds in the grid extent
    {
        double m = 0.0;
        for (int k = 0; k < 3; ++k)
            m = fmax(m, fmax(fabs(V[k].x - K[0]), fmax(fabs(V[k].y - K[1]), fabs(V[k].z - K[2]))));
        const unsigned bits = __float_as_uint(round_up_f(m));
        const unsigned grp = __match_any_sync(__activemask(), si);
        const unsigned mx = __reduce_max_sync(grp, bits);
        if ((threadIdx.x & 31) == __ffs(grp) - 1) atomicMax(&emax_bits[nseg + si], mx);
    }
    // the largest radius of all the mesh's triangles (the mixed path's error bounds)
    atomicMax(&emax_bits[2 * nseg + si], __float_as_uint(ci.w));
    // degenerate (zero-area) or larger than two bricks: always considered
    const double bw = static_cast<double>(s.brick) * s.g.h;
    bool large = degenerate || sqrt(r2) > 2.0 * bw;
    if (large) {
        tbin[t] = -1;
        atomicAdd(&large_cnt[si], 1);
        return;
    }
    atomicMax(&emax_bits[si], __float_as_uint(ci.w));
    // the bin of the centroid among the mesh's bricks (along z those of its slab, from
    // brick layer bzo), clamped: a clamped triangle lies outside the bins' box, and no
    // point inside the box is nearer its clamped position than its own
    int bx = static_cast<int>(floor((cx - K[0]) / bw));
    int by = static_cast<int>(floor((cy - K[1]) / bw));
    int bz = static_cast<int>(floor((cz - K[2]) / bw)) - s.bzo;
    bx = min(max(bx, 0), s.bnx - 1);
    by = min(max(by, 0), s.bny - 1);
    bz = min(max(bz, 0), s.bnz - 1);
    int64_t bin = s.brick_begin + (static_cast<int64_t>(bz) * s.bny + by) * s.bnx + bx;
    tbin[t] = bin;
    atomicAdd(&bincnt[bin], 1);
}

__global__ void k_bin_fill(int64_t ntris, const int64_t* __restrict__ tbin,
                           const int64_t* __restrict__ bin_off, int* __restrict__ bincur,
                           int* __restrict__ bin_list, const MeshSeg* __restrict__ segs, int nseg,
                           int* __restrict__ large_cur, int* __restrict__ large_list) {
    int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= ntris) return;
    int64_t b = tbin[t];
    if (b >= 0) {
        int slot = atomicAdd(&bincur[b], 1);
        bin_list[bin_off[b] + slot] = static_cast<int>(t);
    } else {
        const int si = find_seg<&MeshSeg::tri_begin>(segs, nseg, t);
        int slot = atomicAdd(&large_cur[si], 1);
        large_list[segs[si].large_begin + slot] = static_cast<int>(t);
    }
}

// Writes each mesh's always-considered range, emax and coordinate scale (the
// larger of max |v - K| over its points and the grid extent, with 1e-4 slack)
// into its segment.
__global__ void k_seg_finish(MeshSeg* segs, int nseg, const int64_t* __restrict__ large_off,
                             const unsigned* __restrict__ emax_bits) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nseg) return;
    segs[i].large_begin = large_off[i];
    segs[i].large_end = large_off[i + 1];
    segs[i].emax = __uint_as_float(emax_bits[i]);
    segs[i].emax_all = __uint_as_float(emax_bits[2 * nseg + i]);
    const GridDesc& g = segs[i].g;
    const double ext = g.h * static_cast<double>(max(g.nx, max(g.ny, g.nz)));
    const double sc = fmax(static_cast<double>(__uint_as_float(emax_bits[nseg + i])), ext);
    segs[i].scale = __double2float_ru(sc * 1.0001);
}

// ------------------------------------------------------------------ brick geometry
struct BrickGeo {
    int bx, by, bz;
    int x0, y0, z0, x1, y1, z1;  // cell range [x0, x1)
    float cx, cy, cz;            // centre of the cell-centre box, relative to the corner
    float rb;                    // half-diagonal of that box (rounded up)
};

__device__ __forceinline__ BrickGeo brick_geo(const MeshSeg& s, int64_t lb) {
    BrickGeo q;
    q.bx = static_cast<int>(lb % s.bnx);
    q.by = static_cast<int>((lb / s.bnx) % s.bny);
    q.bz = static_cast<int>(lb / (static_cast<int64_t>(s.bnx) * s.bny));
    const int B = s.brick;
    q.x0 = q.bx * B; q.x1 = min(q.x0 + B, s.g.nx);
    q.y0 = q.by * B; q.y1 = min(q.y0 + B, s.g.ny);
    q.z0 = (q.bz + s.bzo) * B; q.z1 = min(q.z0 + B, s.g.nz);  // bz counts from the slab's bricks
    const float h = static_cast<float>(s.g.h);
    q.cx = 0.5f * (q.x0 + q.x1) * h;
    q.cy = 0.5f * (q.y0 + q.y1) * h;
    q.cz = 0.5f * (q.z0 + q.z1) * h;
    double hx = 0.5 * (q.x1 - q.x0 - 1) * s.g.h, hy = 0.5 * (q.y1 - q.y0 - 1) * s.g.h,
           hz = 0.5 * (q.z1 - q.z0 - 1) * s.g.h;
    q.rb = __double2float_ru(sqrt(hx * hx + hy * hy + hz * hz) * (1.0 + 1e-9));
    return q;
}

// Shell q of Chebyshev radius r -> offset (dx, dy, dz).
__device__ __forceinline__ void shell_offset(int r, int q, int& dx, int& dy, int& dz) {
    if (r == 0) { dx = dy = dz = 0; return; }
    const int w = 2 * r + 1, v = 2 * r - 1;
    const int A = w * w, Bn = w * v;
    if (q < 2 * A) {
        dz = (q / A) ? r : -r;
        int rem = q % A;
        dy = rem / w - r;
        dx = rem % w - r;
        return;
    }
    q -= 2 * A;
    if (q < 2 * Bn) {
        dy = (q / Bn) ? r : -r;
        int rem = q % Bn;
        dz = rem / w - (r - 1);
        dx = rem % w - r;
        return;
    }
    q -= 2 * Bn;
    const int C = v * v;
    dx = (q / C) ? r : -r;
    int rem = q % C;
    dz = rem / v - (r - 1);
    dy = rem % v - (r - 1);
}

__device__ __forceinline__ int shell_count(int r) { return r == 0 ? 1 : 24 * r * r + 2; }

// Bin k of the Chebyshev shell r around the brick (if in the grid): its entry
// range [b0, b1) in the bin CSR; `inside` is set when the bin lies in the grid.
__device__ __forceinline__ void shell_bin(const MeshSeg& s, const BrickGeo& q,
                                          const int64_t* __restrict__ bin_off, int r, int k, int n,
                                          bool& inside, int64_t& b0, int64_t& b1) {
    if (k >= n) return;
    int dx, dy, dz;
    shell_offset(r, k, dx, dy, dz);
    const int x = q.bx + dx, y = q.by + dy, z = q.bz + dz;
    if (x < 0 || y < 0 || z < 0 || x >= s.bnx || y >= s.bny || z >= s.bnz) return;
    inside = true;
    const int64_t bin = s.brick_begin + (static_cast<int64_t>(z) * s.bny + y) * s.bnx + x;
    b0 = bin_off[bin];
    b1 = bin_off[bin + 1];
}

// Upper bound on the distance from point c (corner-relative) to a large triangle:
// the distance to its nearest edge point (segments), plus rounding margin.
__device__ __forceinline__ float seg_dist(float px, float py, float pz, float ax, float ay, float az,
                                          float bx, float by, float bz) {
    float ex = bx - ax, ey = by - ay, ez = bz - az;
    float qx = px - ax, qy = py - ay, qz = pz - az;
    float ee = ex * ex + ey * ey + ez * ez;
    float t = ee > 0.f ? __saturatef((qx * ex + qy * ey + qz * ez) / ee) : 0.f;
    qx -= t * ex; qy -= t * ey; qz -= t * ez;
    return sqrtf(qx * qx + qy * qy + qz * qz);
}

__device__ __forceinline__ float large_upper(const double* __restrict__ soup, int64_t t,
                                             const double* K, float cx, float cy, float cz,
                                             float tol) {
    d3 a, b, c;
    load_soup(soup, t, a, b, c);
    float ax = static_cast<float>(a.x - K[0]), ay = static_cast<float>(a.y - K[1]),
          az = static_cast<float>(a.z - K[2]);
    float bx = static_cast<float>(b.x - K[0]), by = static_cast<float>(b.y - K[1]),
          bz = static_cast<float>(b.z - K[2]);
    float qx = static_cast<float>(c.x - K[0]), qy = static_cast<float>(c.y - K[1]),
          qz = static_cast<float>(c.z - K[2]);
    float d = fminf(seg_dist(cx, cy, cz, ax, ay, az, bx, by, bz),
                    fminf(seg_dist(cx, cy, cz, bx, by, bz, qx, qy, qz),
                          seg_dist(cx, cy, cz, qx, qy, qz, ax, ay, az)));
    return d * (1.f + 16.f * kU32) + tol;
}

__device__ __forceinline__ float aabb_dist(float cx, float cy, float cz, float4 lo, float4 hi) {
    float dx = fmaxf(0.f, fmaxf(lo.x - cx, cx - hi.x));
    float dy = fmaxf(0.f, fmaxf(lo.y - cy, cy - hi.y));
    float dz = fmaxf(0.f, fmaxf(lo.z - cz, cz - hi.z));
    return sqrtf(dx * dx + dy * dy + dz * dz) * (1.f - 8.f * kU32);
}

// The entries of a group of 32 bins (lane L holds bin L's range [b0, b1)) as one
// list, in bin order and then entry order: the order of a loop over the bins. The
// warp takes 32 x R entries per round (R loads in flight per lane, across bin
// boundaries); f(e, ok) gets the R entry positions of this lane and whether each
// exists. The trip count is warp-uniform, so f may use warp votes.
constexpr int kWalkRounds = 4;

template <class F>
__device__ __forceinline__ void for_group_entries(int64_t b0, int64_t b1, int lane, F&& f) {
    const int len = static_cast<int>(b1 - b0);
    int inc = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    const int total = __shfl_sync(0xffffffffu, inc, 31);
    const int excl = inc - len;
    for (int base = 0; base < total; base += 32 * kWalkRounds) {
        int64_t e[kWalkRounds];
        bool ok[kWalkRounds];
#pragma unroll
        for (int j = 0; j < kWalkRounds; ++j) {
            const int v = base + 32 * j + lane;
            // owner bin: the number of bins whose inclusive end is <= v
            int lo = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1)
                if (__shfl_sync(0xffffffffu, inc, lo + step - 1) <= v) lo += step;
            const int L = min(lo, 31);
            const int s0 = __shfl_sync(0xffffffffu, excl, L);
            const int64_t bb = __shfl_sync(0xffffffffu, b0, L);
            ok[j] = v < total;
            e[j] = bb + (v - s0);
        }
        f(e, ok);
    }
}

// W warps per brick, 4 / W bricks per CTA of 128 threads. With few bricks the walks of
// the bricks deep inside a closed surface set the kernel's time (tens of thousands of
// candidates each: every triangle within U + 2 r_B), and W = 4 splits them; with
// many bricks the GPU is full anyway and W = 1 walks each with one warp. Each
// shell's 32-bin groups are split into contiguous ranges, one per warp, range w
// before range w + 1, so the walk order is that of a single walker; the bound U, the
// stopping rules and the counts are reduced over the brick's warps after each shell
// (a named barrier per brick). FILL=false: computes U (stored) and the candidate
// count. FILL=true: per shell each warp counts its candidates, the brick's warps take
// prefix sums, and each writes its own at its offset, in walk order.
constexpr int kWalkThreads = 128;

template <bool FILL, int W>
__global__ void __launch_bounds__(kWalkThreads)
k_brick_walk(const MeshSeg* __restrict__ segs, int nseg, int64_t nbricks,
             const double* __restrict__ soup, const float4* __restrict__ tinfo,
             const float4* __restrict__ tlo, const float4* __restrict__ thi,
             const int64_t* __restrict__ bin_off, const int* __restrict__ bin_list,
             const int* __restrict__ large_list, float* __restrict__ bound,
             int* __restrict__ cand_cnt, const int64_t* __restrict__ cand_off,
             int* __restrict__ cand, float* __restrict__ brick_emax,
             Stats* __restrict__ st) {
    constexpr int kWarps = kWalkThreads / 32;
    __shared__ float s_f[kWarps];
    __shared__ int s_i[kWarps];
    __shared__ int s_c[kWarps];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int slot = wid / W, sub = wid % W;  // brick within the CTA, warp within the brick
    const int first = slot * W;               // the brick's first warp
    const int64_t gb = static_cast<int64_t>(blockIdx.x) * (kWarps / W) + slot;
    if (gb >= nbricks) return;  // uniform over the brick's warps
    auto brick_sync = [&]() {
        if (W == 1) __syncwarp();
        else asm volatile("bar.sync %0, %1;" ::"r"(1 + slot), "r"(32 * W) : "memory");
    };
    const int si = find_seg<&MeshSeg::brick_begin>(segs, nseg, gb);
    const MeshSeg& s = segs[si];
    const BrickGeo q = brick_geo(s, gb - s.brick_begin);
    const float bw = static_cast<float>(s.brick * s.g.h);
    const float tol = 8.f * kU32 * s.scale + 1e-30f;
    const float emax = s.emax;
    const int rmax = max(s.bnx, max(s.bny, s.bnz));
    // reductions over the brick's warps (each of its threads calls them, at points
    // uniform over the brick)
    auto brick_min = [&](float v) {
        v = warp_min(v);
        if (W == 1) return v;
        if (lane == 0) s_f[wid] = v;
        brick_sync();
        float m = s_f[first];
#pragma unroll
        for (int w = 1; w < W; ++w) m = fminf(m, s_f[first + w]);
        brick_sync();
        return m;
    };
    auto brick_any = [&](bool v) {
        const bool wv = __any_sync(0xffffffffu, v);
        if (W == 1) return wv;
        if (lane == 0) s_i[wid] = wv ? 1 : 0;
        brick_sync();
        int a = 0;
#pragma unroll
        for (int w = 0; w < W; ++w) a |= s_i[first + w];
        brick_sync();
        return a != 0;
    };
    // this warp's contiguous range [g0, g1) of the 32-bin groups of a shell of n bins
    auto range = [&](int n, int& g0, int& g1) {
        const int ng = (n + 31) / 32;
        g0 = static_cast<int>(static_cast<int64_t>(ng) * sub / W);
        g1 = static_cast<int>(static_cast<int64_t>(ng) * (sub + 1) / W);
    };
    float U;
    if (!FILL) {
        // ---- upper bound on the distance from the brick centre to the surface
        U = FLT_MAX;
        for (int64_t e = s.large_begin + 32 * sub + lane; e < s.large_end; e += 32 * W)
            U = fminf(U, large_upper(soup, large_list[e], s.g.corner, q.cx, q.cy, q.cz, tol));
        for (int r = 0; r <= rmax; ++r) {
            U = brick_min(U);
            if (r > 0 && (r - 1) * bw > U) break;  // farther bins cannot lower U
            const int n = shell_count(r);
            int g0, g1;
            range(n, g0, g1);
            bool inside = false;
            for (int g = g0; g < g1; ++g) {
                int64_t b0 = 0, b1 = 0;
                shell_bin(s, q, bin_off, r, 32 * g + lane, n, inside, b0, b1);
                for_group_entries(b0, b1, lane, [&](const int64_t* e, const bool* ok) {
                    int t[kWalkRounds];
#pragma unroll
                    for (int j = 0; j < kWalkRounds; ++j) t[j] = ok[j] ? bin_list[e[j]] : -1;
#pragma unroll
                    for (int j = 0; j < kWalkRounds; ++j) {
                        if (t[j] < 0) continue;
                        float4 ti = tinfo[t[j]];
                        float dx2 = ti.x - q.cx, dy2 = ti.y - q.cy, dz2 = ti.z - q.cz;
                        float d = sqrtf(dx2 * dx2 + dy2 * dy2 + dz2 * dz2) * (1.f + 4.f * kU32);
                        U = fminf(U, d + ti.w + tol);
                    }
                });
            }
            if (r > 0 && !brick_any(inside)) {
                U = brick_min(U);
                break;
            }
        }
        U = brick_min(U);
        if (sub == 0 && lane == 0) bound[gb] = U;
    } else {
        U = bound[gb];
    }
    // ---- candidates: lower bound <= U + 2 r_B (+ margins). The relative margin (4e-5,
    // about 670 u) covers four stated FP32 errors 48u (d + 2e + 2r) beyond any cell's
    // distance (e at most two bricks here; larger triangles are always considered): the
    // exact FP64 path's near-ties and its band pass need them, the mixed path two
    const float lim = (U + 2.f * q.rb) * (1.f + 4e-5f) + 2.f * tol;
    const int64_t out = FILL ? cand_off[gb] : 0;
    const unsigned below = (1u << lane) - 1u;
    float bemax = 0.f;
    // walks this warp's groups of shell r; f(take, t, e_t) per entry, in walk order,
    // called by the whole warp
    auto walk = [&](int r, int n, int g0, int g1, bool& inside, auto&& f) {
        for (int g = g0; g < g1; ++g) {
            int64_t b0 = 0, b1 = 0;
            shell_bin(s, q, bin_off, r, 32 * g + lane, n, inside, b0, b1);
            for_group_entries(b0, b1, lane, [&](const int64_t* e, const bool* ok) {
                int t[kWalkRounds];
#pragma unroll
                for (int j = 0; j < kWalkRounds; ++j) t[j] = ok[j] ? bin_list[e[j]] : -1;
                float4 ti[kWalkRounds];
#pragma unroll
                for (int j = 0; j < kWalkRounds; ++j)
                    if (t[j] >= 0) ti[j] = tinfo[t[j]];
#pragma unroll
                for (int j = 0; j < kWalkRounds; ++j) {
                    bool take = false;
                    float et = 0.f;
                    if (t[j] >= 0) {
                        float dx2 = ti[j].x - q.cx, dy2 = ti[j].y - q.cy, dz2 = ti[j].z - q.cz;
                        float d = sqrtf(dx2 * dx2 + dy2 * dy2 + dz2 * dz2) * (1.f - 4.f * kU32);
                        take = d - ti[j].w <= lim;  // |v - c_t| - e_t >= d - r_B - e_t
                        et = ti[j].w;
                    }
                    f(take, t[j], et);
                }
            });
        }
    };
    // the always-considered large triangles first, by the brick's first warp
    if (sub == 0) {
        int c = 0;
        for (int64_t e0 = s.large_begin; e0 < s.large_end; e0 += 32) {
            const int64_t e = e0 + lane;
            bool take = false;
            int t = 0;
            float et = 0.f;
            if (e < s.large_end) {
                t = large_list[e];
                float4 lo = tlo[t], hi = thi[t];
                float d = aabb_dist(q.cx, q.cy, q.cz, lo, hi);
                take = d <= lim;  // d(v,t) >= d - r_B must reach U + r_B
                et = tinfo[t].w;
            }
            const unsigned m = __ballot_sync(0xffffffffu, take);
            if (FILL && take) cand[out + c + __popc(m & below)] = t;
            if (take) bemax = fmaxf(bemax, et);
            c += __popc(m);
        }
        if (lane == 0) s_c[first] = c;
    }
    brick_sync();
    int64_t base = s_c[first];  // entries before the current shell
    brick_sync();
    int mine = 0;           // count pass: this warp's entries over all shells
    for (int r = 0; r <= rmax; ++r) {
        if (r > 0 && (r - 1) * bw - emax > lim) break;
        const int n = shell_count(r);
        int g0, g1;
        range(n, g0, g1);
        bool any_inside = false;
        int c = 0;
        if (FILL && W == 1) {
            // one warp per brick: written in the one walk, at a running offset
            walk(r, n, g0, g1, any_inside, [&](bool take, int t, float et) {
                const unsigned m = __ballot_sync(0xffffffffu, take);
                if (take) {
                    cand[out + base + c + __popc(m & below)] = t;
                    bemax = fmaxf(bemax, et);
                }
                c += __popc(m);
            });
            base += c;
        } else {
            walk(r, n, g0, g1, any_inside,
                 [&](bool take, int, float) { c += __popc(__ballot_sync(0xffffffffu, take)); });
        }
        if (FILL && W > 1) {
            // several warps: prefix sums of this shell's counts, then the writing walk
            if (lane == 0) s_c[wid] = c;
            brick_sync();
            int64_t off = base;
            int tot = 0;
#pragma unroll
            for (int w = 0; w < W; ++w) {
                if (w < sub) off += s_c[first + w];
                tot += s_c[first + w];
            }
            brick_sync();
            int k = 0;
            bool again = false;
            walk(r, n, g0, g1, again, [&](bool take, int t, float et) {
                const unsigned m = __ballot_sync(0xffffffffu, take);
                if (take) {
                    cand[out + off + k + __popc(m & below)] = t;
                    bemax = fmaxf(bemax, et);
                }
                k += __popc(m);
            });
            base += tot;
        } else if (!FILL) {
            mine += c;
        }
        if (r > 0 && !brick_any(any_inside)) break;
    }
    if (!FILL) {
        if (lane == 0) s_c[wid] = mine;
        brick_sync();
        if (sub == 0 && lane == 0) {
            int64_t total = base;
#pragma unroll
            for (int w = 0; w < W; ++w) total += s_c[first + w];
            cand_cnt[gb] = static_cast<int>(total);
            atomicAdd(&st->candidates, static_cast<unsigned long long>(total));
        }
    } else {
        bemax = -brick_min(-bemax);
        if (sub == 0 && lane == 0) brick_emax[gb] = bemax;
    }
}

// ------------------------------------------------------------------ evaluation
constexpr int kChunk = 64;  // candidates staged per round

// Cell owned by (thread, slot) inside a brick of edge B.
template <int B, int THREADS>
struct CellMap {
    static constexpr int VPT = B * B * B / THREADS;
    __device__ static void cell(int tid, int v, int& x, int& y, int& z) {
        // threads tile x (fastest), then y, then z-slabs; each thread owns VPT cells in z
        x = tid % B;
        y = (tid / B) % B;
        int zslab = tid / (B * B);
        z = zslab * VPT + v;
    }
};

// Plain FP64: CTA per brick (persistent over a work list), THREADS threads.
template <int B, int THREADS>
__global__ void __launch_bounds__(THREADS)
k_sdf_fp64(const MeshSeg* __restrict__ segs, int nseg, const uint32_t* __restrict__ work,
           int64_t nwork, unsigned long long* __restrict__ queue, const double* __restrict__ soup,
           const float4* __restrict__ tinfo, const int64_t* __restrict__ cand_off,
           const int* __restrict__ cand, Out o, Stats* __restrict__ st) {
    using M = CellMap<B, THREADS>;
    constexpr int VPT = M::VPT;
    __shared__ double sv[kChunk][12];  // a, b, c, centroid (FP64)
    __shared__ double srad[kChunk];
    __shared__ int sid[kChunk];
    __shared__ int64_t s_item;
    const int tid = threadIdx.x;
    unsigned long long evals = 0;
    for (;;) {
        if (tid == 0) s_item = static_cast<int64_t>(atomicAdd(queue, 1ull));
        __syncthreads();
        const int64_t item = s_item;
        __syncthreads();
        if (item >= nwork) break;
        const int64_t gb = static_cast<int64_t>(work[item]);
        const int si = find_seg<&MeshSeg::brick_begin>(segs, nseg, gb);
        const MeshSeg& s = segs[si];
        const BrickGeo q = brick_geo(s, gb - s.brick_begin);
        const GridDesc g = s.g;
        d3 p[VPT];
        bool valid[VPT];
        double best[VPT], bestd[VPT];
        int bt[VPT], br[VPT];
#pragma unroll
        for (int v = 0; v < VPT; ++v) {
            int x, y, z;
            M::cell(tid, v, x, y, z);
            x += q.x0; y += q.y0; z += q.z0;
            valid[v] = x < q.x1 && y < q.y1 && z < q.z1;
            p[v] = {cell_center(g.corner[0], x, g.h), cell_center(g.corner[1], y, g.h),
                    cell_center(g.corner[2], z, g.h)};
            best[v] = DBL_MAX;
            bestd[v] = DBL_MAX;
            bt[v] = INT_MAX;
            br[v] = 0;
        }
        const int64_t c0 = cand_off[gb], c1 = cand_off[gb + 1];
        for (int64_t base = c0; base < c1; base += kChunk) {
            const int n = static_cast<int>(c1 - base < kChunk ? c1 - base : kChunk);
            __syncthreads();
            for (int k = tid; k < n; k += THREADS) {
                int t = cand[base + k];
                d3 a, b, c;
                load_soup(soup, t, a, b, c);
                sv[k][0] = a.x; sv[k][1] = a.y; sv[k][2] = a.z;
                sv[k][3] = b.x; sv[k][4] = b.y; sv[k][5] = b.z;
                sv[k][6] = c.x; sv[k][7] = c.y; sv[k][8] = c.z;
                float4 ti = tinfo[t];
                sv[k][9] = g.corner[0] + ti.x;
                sv[k][10] = g.corner[1] + ti.y;
                sv[k][11] = g.corner[2] + ti.z;
                srad[k] = static_cast<double>(ti.w) * (1.0 + 1e-6) + 1e-9 * s.scale;
                sid[k] = t;
            }
            __syncthreads();
            for (int k = 0; k < n; ++k) {
                // warp-uniform skip: the bounding sphere is beyond every lane's best
                bool need = false;
#pragma unroll
                for (int v = 0; v < VPT; ++v) {
                    double dx = p[v].x - sv[k][9], dy = p[v].y - sv[k][10], dz = p[v].z - sv[k][11];
                    double lim = bestd[v] + srad[k];
                    need |= valid[v] && (bestd[v] == DBL_MAX || dx * dx + dy * dy + dz * dz <= lim * lim);
                }
                if (!__any_sync(0xffffffffu, need)) continue;
                const d3 a{sv[k][0], sv[k][1], sv[k][2]}, b{sv[k][3], sv[k][4], sv[k][5]},
                    c{sv[k][6], sv[k][7], sv[k][8]};
                const int t = sid[k];
#pragma unroll
                for (int v = 0; v < VPT; ++v) {
                    if (!valid[v]) continue;
                    int reg;
                    double d2 = ericson(p[v], a, b, c, &reg);
                    ++evals;
                    if (d2 < best[v] || (d2 == best[v] && t < bt[v])) {
                        best[v] = d2;
                        bt[v] = t;
                        br[v] = reg;
                        bestd[v] = sqrt(d2) * (1.0 + 1e-9);
                    }
                }
            }
        }
#pragma unroll
        for (int v = 0; v < VPT; ++v) {
            if (!valid[v]) continue;
            int x, y, z;
            M::cell(tid, v, x, y, z);
            x += q.x0; y += q.y0; z += q.z0;
            int64_t idx = s.vox_begin + (static_cast<int64_t>(z) * g.ny + y) * g.nx + x;
            write_cell(o, idx, __dsqrt_rn(best[v]), bt[v], br[v]);
        }
    }
    long long ev = warp_sum(static_cast<long long>(evals));
    if ((tid & 31) == 0 && ev) {
        atomicAdd(&st->evaluations, static_cast<unsigned long long>(ev));
        atomicAdd(&st->fp64_evaluations, static_cast<unsigned long long>(ev));
    }
}

// FP32 record of a candidate, recentred on the brick centre.
struct alignas(16) Rec32 {
    float v0[3], v1[3], v2[3];   // vertices
    float e0[3], e1[3], e2[3];   // edges v1-v0, v2-v1, v0-v2
    float nn[3];                 // unit normal (from FP64)
    float m0[3], m1[3], m2[3];   // in-plane inward edge normals
    float inv[3];                // 1 / |e_k|^2 (0 for a degenerate edge)
    float cen[3], rad;           // bounding sphere
    float ok;                    // 1: plane branch allowed (non-degenerate)
    int tid;
    float pad_[1];
};
static_assert(sizeof(Rec32) == 160, "record layout");

__device__ __forceinline__ void make_rec(Rec32& r, const d3& a, const d3& b, const d3& c,
                                         const double* cb, float rad, int t) {
    float v[9] = {static_cast<float>(a.x - cb[0]), static_cast<float>(a.y - cb[1]),
                  static_cast<float>(a.z - cb[2]), static_cast<float>(b.x - cb[0]),
                  static_cast<float>(b.y - cb[1]), static_cast<float>(b.z - cb[2]),
                  static_cast<float>(c.x - cb[0]), static_cast<float>(c.y - cb[1]),
                  static_cast<float>(c.z - cb[2])};
    for (int k = 0; k < 3; ++k) {
        r.v0[k] = v[k]; r.v1[k] = v[3 + k]; r.v2[k] = v[6 + k];
        r.e0[k] = v[3 + k] - v[k];
        r.e1[k] = v[6 + k] - v[3 + k];
        r.e2[k] = v[k] - v[6 + k];
    }
    // normal in FP64 from the FP64 vertices, then normalised in FP32
    double ux = b.x - a.x, uy = b.y - a.y, uz = b.z - a.z;
    double wx = c.x - a.x, wy = c.y - a.y, wz = c.z - a.z;
    double nx = uy * wz - uz * wy, ny = uz * wx - ux * wz, nz = ux * wy - uy * wx;
    double nl = sqrt(nx * nx + ny * ny + nz * nz);
    float ok = nl > 0.0 ? 1.f : 0.f;
    float n3[3] = {0.f, 0.f, 0.f};
    if (nl > 0.0) {
        n3[0] = static_cast<float>(nx / nl);
        n3[1] = static_cast<float>(ny / nl);
        n3[2] = static_cast<float>(nz / nl);
    }
    r.nn[0] = n3[0]; r.nn[1] = n3[1]; r.nn[2] = n3[2];
    const float* E[3] = {r.e0, r.e1, r.e2};
    float* Mv[3] = {r.m0, r.m1, r.m2};
    for (int k = 0; k < 3; ++k) {
        const float* e = E[k];
        // n x e points into the triangle for a counter-clockwise (about n) edge
        Mv[k][0] = n3[1] * e[2] - n3[2] * e[1];
        Mv[k][1] = n3[2] * e[0] - n3[0] * e[2];
        Mv[k][2] = n3[0] * e[1] - n3[1] * e[0];
        float ee = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
        r.inv[k] = ee > 0.f ? 1.f / ee : 0.f;
    }
    r.cen[0] = (v[0] + v[3] + v[6]) * (1.f / 3.f);
    r.cen[1] = (v[1] + v[4] + v[7]) * (1.f / 3.f);
    r.cen[2] = (v[2] + v[5] + v[8]) * (1.f / 3.f);
    r.rad = rad * (1.f + 64.f * kU32);
    r.ok = ok;
    r.tid = t;
}

// FP32 squared distance from p to the recorded triangle; region in Ericson's
// numbering (0 a, 1 b, 2 ab, 3 c, 4 ac, 5 bc, 6 interior).
__device__ __forceinline__ float dist32(const Rec32& r, float px, float py, float pz, int* reg) {
    float pax = px - r.v0[0], pay = py - r.v0[1], paz = pz - r.v0[2];
    float pbx = px - r.v1[0], pby = py - r.v1[1], pbz = pz - r.v1[2];
    float pcx = px - r.v2[0], pcy = py - r.v2[1], pcz = pz - r.v2[2];
    float s0 = r.m0[0] * pax + r.m0[1] * pay + r.m0[2] * paz;
    float s1 = r.m1[0] * pbx + r.m1[1] * pby + r.m1[2] * pbz;
    float s2 = r.m2[0] * pcx + r.m2[1] * pcy + r.m2[2] * pcz;
    if (r.ok > 0.f && s0 >= 0.f && s1 >= 0.f && s2 >= 0.f) {
        float dp = r.nn[0] * pax + r.nn[1] * pay + r.nn[2] * paz;
        *reg = 6;
        return dp * dp;
    }
    float t0 = __saturatef((pax * r.e0[0] + pay * r.e0[1] + paz * r.e0[2]) * r.inv[0]);
    float qx = pax - t0 * r.e0[0], qy = pay - t0 * r.e0[1], qz = paz - t0 * r.e0[2];
    float d0 = qx * qx + qy * qy + qz * qz;
    float t1 = __saturatef((pbx * r.e1[0] + pby * r.e1[1] + pbz * r.e1[2]) * r.inv[1]);
    qx = pbx - t1 * r.e1[0]; qy = pby - t1 * r.e1[1]; qz = pbz - t1 * r.e1[2];
    float d1 = qx * qx + qy * qy + qz * qz;
    float t2 = __saturatef((pcx * r.e2[0] + pcy * r.e2[1] + pcz * r.e2[2]) * r.inv[2]);
    qx = pcx - t2 * r.e2[0]; qy = pcy - t2 * r.e2[1]; qz = pcz - t2 * r.e2[2];
    float d2 = qx * qx + qy * qy + qz * qz;
    float d = d0;
    int g = t0 <= 0.f ? 0 : (t0 >= 1.f ? 1 : 2);
    if (d1 < d) { d = d1; g = t1 <= 0.f ? 1 : (t1 >= 1.f ? 3 : 5); }
    if (d2 < d) { d = d2; g = t2 <= 0.f ? 3 : (t2 >= 1.f ? 0 : 4); }
    *reg = g;
    return d;
}

template <int B, int THREADS>
__global__ void __launch_bounds__(THREADS)
k_sdf_mixed(const MeshSeg* __restrict__ segs, int nseg, const uint32_t* __restrict__ work,
            int64_t nwork, unsigned long long* __restrict__ queue, const double* __restrict__ soup,
            const float4* __restrict__ tinfo, const int64_t* __restrict__ cand_off,
            const int* __restrict__ cand, const float* __restrict__ brick_emax, float band_cells,
            Out o, Stats* __restrict__ st) {
    using M = CellMap<B, THREADS>;
    constexpr int VPT = M::VPT;
    __shared__ Rec32 rec[kChunk];
    __shared__ int64_t s_item;
    __shared__ int s_band;
    const int tid = threadIdx.x;
    unsigned long long evals = 0, evals64 = 0, bandc = 0;
    for (;;) {
        if (tid == 0) {
            s_item = static_cast<int64_t>(atomicAdd(queue, 1ull));
            s_band = 0;
        }
        __syncthreads();
        const int64_t item = s_item;
        if (item >= nwork) break;
        const int64_t gb = static_cast<int64_t>(work[item]);
        const int si = find_seg<&MeshSeg::brick_begin>(segs, nseg, gb);
        const MeshSeg& s = segs[si];
        const BrickGeo q = brick_geo(s, gb - s.brick_begin);
        const GridDesc g = s.g;
        // brick centre in FP64 (the recentring origin)
        const double cb[3] = {g.corner[0] + 0.5 * (q.x0 + q.x1) * g.h,
                              g.corner[1] + 0.5 * (q.y0 + q.y1) * g.h,
                              g.corner[2] + 0.5 * (q.z0 + q.z1) * g.h};
        float px[VPT], py[VPT], pz[VPT], best[VPT], bestd[VPT];
        int bt[VPT], br[VPT];
        bool valid[VPT];
#pragma unroll
        for (int v = 0; v < VPT; ++v) {
            int x, y, z;
            M::cell(tid, v, x, y, z);
            x += q.x0; y += q.y0; z += q.z0;
            valid[v] = x < q.x1 && y < q.y1 && z < q.z1;
            px[v] = static_cast<float>(cell_center(g.corner[0], x, g.h) - cb[0]);
            py[v] = static_cast<float>(cell_center(g.corner[1], y, g.h) - cb[1]);
            pz[v] = static_cast<float>(cell_center(g.corner[2], z, g.h) - cb[2]);
            best[v] = FLT_MAX;
            bestd[v] = FLT_MAX;
            bt[v] = INT_MAX;
            br[v] = 0;
        }
        const int64_t c0 = cand_off[gb], c1 = cand_off[gb + 1];
        for (int64_t base = c0; base < c1; base += kChunk) {
            const int n = static_cast<int>(c1 - base < kChunk ? c1 - base : kChunk);
            __syncthreads();
            for (int k = tid; k < n; k += THREADS) {
                int t = cand[base + k];
                d3 a, b, c;
                load_soup(soup, t, a, b, c);
                make_rec(rec[k], a, b, c, cb, tinfo[t].w, t);
            }
            __syncthreads();
            for (int k = 0; k < n; ++k) {
                const Rec32& r = rec[k];
                bool need = false;
#pragma unroll
                for (int v = 0; v < VPT; ++v) {
                    float dx = px[v] - r.cen[0], dy = py[v] - r.cen[1], dz = pz[v] - r.cen[2];
                    float lim = bestd[v] + r.rad;
                    need |= valid[v] && dx * dx + dy * dy + dz * dz <= lim * lim;
                }
                if (!__any_sync(0xffffffffu, need)) continue;
#pragma unroll
                for (int v = 0; v < VPT; ++v) {
                    if (!valid[v]) continue;
                    int reg;
                    float d2 = dist32(r, px[v], py[v], pz[v], &reg);
                    ++evals;
                    if (d2 < best[v] || (d2 == best[v] && r.tid < bt[v])) {
                        best[v] = d2;
                        bt[v] = r.tid;
                        br[v] = reg;
                        bestd[v] = sqrtf(d2) * (1.f + 4.f * kU32) + 1e-30f;
                    }
                }
            }
        }
        // stated FP32 error bound per cell and the FP64 band
        const float emx = brick_emax[gb];
        const float bandw = band_cells * static_cast<float>(g.h);
        float eb[VPT];
        bool inband[VPT];
        bool any_band = false;
#pragma unroll
        for (int v = 0; v < VPT; ++v) {
            float d = sqrtf(best[v]);
            eb[v] = 48.f * kU32 * (d + 2.f * emx + 2.f * q.rb) + 1e-30f;
            inband[v] = valid[v] && d <= bandw + eb[v];
            any_band |= inband[v];
        }
        if (any_band) s_band = 1;
        __syncthreads();
        double best64[VPT];
        int bt64[VPT], br64[VPT];
#pragma unroll
        for (int v = 0; v < VPT; ++v) {
            best64[v] = DBL_MAX;
            bt64[v] = INT_MAX;
            br64[v] = 0;
        }
        if (s_band) {
            // FP64 refinement over candidates within 2*eb of the FP32 best
            for (int64_t base = c0; base < c1; base += kChunk) {
                const int n = static_cast<int>(c1 - base < kChunk ? c1 - base : kChunk);
                __syncthreads();
                for (int k = tid; k < n; k += THREADS) {
                    int t = cand[base + k];
                    d3 a, b, c;
                    load_soup(soup, t, a, b, c);
                    make_rec(rec[k], a, b, c, cb, tinfo[t].w, t);
                }
                __syncthreads();
                for (int k = 0; k < n; ++k) {
                    const Rec32& r = rec[k];
#pragma unroll
                    for (int v = 0; v < VPT; ++v) {
                        if (!inband[v]) continue;
                        int reg;
                        float d2 = dist32(r, px[v], py[v], pz[v], &reg);
                        float lim = sqrtf(best[v]) + 2.f * eb[v];
                        if (sqrtf(d2) > lim * (1.f + 1e-6f)) continue;
                        d3 a, b, c;
                        load_soup(soup, r.tid, a, b, c);
                        int x, y, z;
                        M::cell(tid, v, x, y, z);
                        x += q.x0; y += q.y0; z += q.z0;
                        const d3 P{cell_center(g.corner[0], x, g.h), cell_center(g.corner[1], y, g.h),
                                   cell_center(g.corner[2], z, g.h)};
                        int r64;
                        double e2 = ericson(P, a, b, c, &r64);
                        ++evals64;
                        if (e2 < best64[v] || (e2 == best64[v] && r.tid < bt64[v])) {
                            best64[v] = e2;
                            bt64[v] = r.tid;
                            br64[v] = r64;
                        }
                    }
                }
            }
        }
#pragma unroll
        for (int v = 0; v < VPT; ++v) {
            if (!valid[v]) continue;
            int x, y, z;
            M::cell(tid, v, x, y, z);
            x += q.x0; y += q.y0; z += q.z0;
            int64_t idx = s.vox_begin + (static_cast<int64_t>(z) * g.ny + y) * g.nx + x;
            if (inband[v]) {
                ++bandc;
                write_cell(o, idx, __dsqrt_rn(best64[v]), bt64[v], br64[v]);
                if (o.errbound) o.errbound[idx] = 0.f;
            } else {
                write_cell(o, idx, static_cast<double>(sqrtf(best[v])), bt[v], br[v]);
                if (o.errbound) o.errbound[idx] = eb[v];
            }
        }
        __syncthreads();
    }
    long long ev = warp_sum(static_cast<long long>(evals));
    long long ev64 = warp_sum(static_cast<long long>(evals64));
    long long bc = warp_sum(static_cast<long long>(bandc));
    if ((tid & 31) == 0) {
        if (ev) atomicAdd(&st->evaluations, static_cast<unsigned long long>(ev));
        if (ev64) atomicAdd(&st->fp64_evaluations, static_cast<unsigned long long>(ev64));
        if (bc) atomicAdd(&st->band_voxels, static_cast<unsigned long long>(bc));
    }
}

// Work model: per cell, K(v) = #{t : |p - c_t| - e_t <= |sdf(v)|}, the triangles
// whose bounding sphere reaches the distance sphere of the cell -- the minimal
// candidate set of any bounding-sphere-pruned exact search. out[0] = sum K over
// all cells, out[1] = sum K over cells with |sdf| <= band, out[2] = those cells.
template <int B, int THREADS>
__global__ void __launch_bounds__(THREADS)
k_count_K(const MeshSeg* __restrict__ segs, int nseg, int64_t nbricks,
          const float4* __restrict__ tinfo, const int64_t* __restrict__ cand_off,
          const int* __restrict__ cand, const double* __restrict__ sdf64,
          const float* __restrict__ sdf32, float band_cells, unsigned long long* __restrict__ out) {
    using M = CellMap<B, THREADS>;
    constexpr int VPT = M::VPT;
    const int64_t gb = blockIdx.x;
    if (gb >= nbricks) return;
    const int si = find_seg<&MeshSeg::brick_begin>(segs, nseg, gb);
    const MeshSeg& s = segs[si];
    const BrickGeo q = brick_geo(s, gb - s.brick_begin);
    const GridDesc g = s.g;
    const float h = static_cast<float>(g.h);
    unsigned long long k_all = 0, k_band = 0, n_band = 0;
    for (int v = 0; v < VPT; ++v) {
        int x, y, z;
        M::cell(threadIdx.x, v, x, y, z);
        x += q.x0; y += q.y0; z += q.z0;
        if (!(x < q.x1 && y < q.y1 && z < q.z1 && z >= g.z0 && z < g.z1)) continue;
        int64_t idx = s.vox_begin + (static_cast<int64_t>(z - g.z0) * g.ny + y) * g.nx + x;
        float d = sdf64 ? static_cast<float>(fabs(sdf64[idx])) : fabsf(sdf32[idx]);
        float px = (x + 0.5f) * h, py = (y + 0.5f) * h, pz = (z + 0.5f) * h;
        unsigned kk = 0;
        for (int64_t e = cand_off[gb]; e < cand_off[gb + 1]; ++e) {
            float4 ti = tinfo[cand[e]];
            float dx = px - ti.x, dy = py - ti.y, dz = pz - ti.z;
            kk += sqrtf(dx * dx + dy * dy + dz * dz) - ti.w <= d;
        }
        kk = max(kk, 1u);
        k_all += kk;
        if (d <= band_cells * h) {
            k_band += kk;
            ++n_band;
        }
    }
    long long a = warp_sum(static_cast<long long>(k_all));
    long long b = warp_sum(static_cast<long long>(k_band));
    long long c = warp_sum(static_cast<long long>(n_band));
    if ((threadIdx.x & 31) == 0) {
        if (a) atomicAdd(&out[0], static_cast<unsigned long long>(a));
        if (b) atomicAdd(&out[1], static_cast<unsigned long long>(b));
        if (c) atomicAdd(&out[2], static_cast<unsigned long long>(c));
    }
}

// LPT order of the bricks: key = ~count so an ascending sort puts the most
// expensive bricks first.
__global__ void k_work_keys(const int* __restrict__ cand_cnt, int64_t n, uint32_t* __restrict__ keys,
                            uint32_t* __restrict__ vals) {
    int64_t b = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (b >= n) return;
    keys[b] = ~static_cast<uint32_t>(cand_cnt[b]);
    vals[b] = static_cast<uint32_t>(b);
}

}  // namespace

// ------------------------------------------------------------------ launchers
void launch_sdf_tri_prep(const MeshSeg* segs, int nseg, int64_t ntris, const double* soup,
                         float4* tinfo, float4* tinfo_lo, void* trec, float4* tnorm, float4* tlo,
                         float4* thi,
                         int64_t* tbin, int* bincnt, int* large_cnt, unsigned* emax_bits,
                         cudaStream_t st) {
    if (ntris == 0) return;
    k_sdf_tri_prep<<<static_cast<unsigned>((ntris + 255) / 256), 256, 0, st>>>(
        segs, nseg, ntris, soup, tinfo, tinfo_lo, static_cast<TriRec*>(trec), tnorm, tlo, thi, tbin,
        bincnt, large_cnt, emax_bits);
    CMG_LAUNCH();
}

void launch_bin_fill(int64_t ntris, const int64_t* tbin, const int64_t* bin_off, int* bincur,
                     int* bin_list, const MeshSeg* segs, int nseg, int* large_cur, int* large_list,
                     cudaStream_t st) {
    if (ntris == 0) return;
    k_bin_fill<<<static_cast<unsigned>((ntris + 255) / 256), 256, 0, st>>>(
        ntris, tbin, bin_off, bincur, bin_list, segs, nseg, large_cur, large_list);
    CMG_LAUNCH();
}

void launch_seg_finish(MeshSeg* segs, int nseg, const int64_t* large_off, const unsigned* emax_bits,
                       cudaStream_t st) {
    k_seg_finish<<<(nseg + 127) / 128, 128, 0, st>>>(segs, nseg, large_off, emax_bits);
    CMG_LAUNCH();
}

int brick_walk_warps(int64_t nbricks, int walk_warps) {
    if (walk_warps == 1 || walk_warps == 2 || walk_warps == 4) return walk_warps;
    // 4 while 4-warp bricks fit about twice in the GPU's warp slots (a few heavy bricks
    // set the time), 2 up to twice that, then 1
    const int64_t sms = device_sms();
    return nbricks <= 32 * sms ? 4 : (nbricks <= 64 * sms ? 2 : 1);
}

void launch_brick_walk(bool fill, const MeshSeg* segs, int nseg, int64_t nbricks, const double* soup,
                       const float4* tinfo, const float4* tlo, const float4* thi,
                       const int64_t* bin_off, const int* bin_list, const int* large_list,
                       float* bound, int* cand_cnt, const int64_t* cand_off, int* cand,
                       float* brick_emax, Stats* stats, int walk_warps, cudaStream_t st) {
    if (nbricks == 0) return;
    const int W = brick_walk_warps(nbricks, walk_warps);
    const unsigned grid = static_cast<unsigned>((nbricks * W + 3) / 4);
    auto go = [&](auto fill_tag, auto w_tag) {
        constexpr bool F = decltype(fill_tag)::value;
        constexpr int WW = decltype(w_tag)::value;
        k_brick_walk<F, WW><<<grid, kWalkThreads, 0, st>>>(segs, nseg, nbricks, soup, tinfo, tlo, thi,
                                                           bin_off, bin_list, large_list, bound,
                                                           cand_cnt, cand_off, cand, brick_emax, stats);
    };
    using T = std::true_type;
    using Fa = std::false_type;
    using W1 = std::integral_constant<int, 1>;
    using W2 = std::integral_constant<int, 2>;
    using W4 = std::integral_constant<int, 4>;
    if (fill) {
        if (W == 4) go(T{}, W4{});
        else if (W == 2) go(T{}, W2{});
        else go(T{}, W1{});
    } else {
        if (W == 4) go(Fa{}, W4{});
        else if (W == 2) go(Fa{}, W2{});
        else go(Fa{}, W1{});
    }
    CMG_LAUNCH();
}

void launch_count_K(int brick, const MeshSeg* segs, int nseg, int64_t nbricks, const float4* tinfo,
                    const int64_t* cand_off, const int* cand, const double* sdf64,
                    const float* sdf32, float band_cells, unsigned long long* out,
                    cudaStream_t st) {
    if (nbricks == 0) return;
    if (brick == 4)
        k_count_K<4, 64><<<static_cast<unsigned>(nbricks), 64, 0, st>>>(
            segs, nseg, nbricks, tinfo, cand_off, cand, sdf64, sdf32, band_cells, out);
    else if (brick == 16)
        k_count_K<16, 256><<<static_cast<unsigned>(nbricks), 256, 0, st>>>(
            segs, nseg, nbricks, tinfo, cand_off, cand, sdf64, sdf32, band_cells, out);
    else
        k_count_K<8, 128><<<static_cast<unsigned>(nbricks), 128, 0, st>>>(
            segs, nseg, nbricks, tinfo, cand_off, cand, sdf64, sdf32, band_cells, out);
    CMG_LAUNCH();
}

void launch_work_keys(const int* cand_cnt, int64_t n, uint32_t* keys, uint32_t* vals,
                      cudaStream_t st) {
    if (n == 0) return;
    k_work_keys<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(cand_cnt, n, keys, vals);
    CMG_LAUNCH();
}

void launch_sdf_eval(int precision, int brick, const MeshSeg* segs, int nseg, const uint32_t* work,
                     int64_t nwork, unsigned long long* queue, const double* soup,
                     const float4* tinfo, const int64_t* cand_off, const int* cand,
                     const float* brick_emax, float band_cells, const uint8_t* occ, float* sdf32,
                     double* sdf64, int* near_tri, uint8_t* near_reg, float* errbound, Stats* stats,
                     int grid, cudaStream_t st) {
    if (nwork == 0) return;
    Out o{occ, sdf32, sdf64, near_tri, near_reg, errbound};
    if (precision == kPrecMixed) {
        if (brick == 4)
            k_sdf_mixed<4, 64><<<grid, 64, 0, st>>>(segs, nseg, work, nwork, queue, soup, tinfo,
                                                    cand_off, cand, brick_emax, band_cells, o, stats);
        else
            k_sdf_mixed<8, 128><<<grid, 128, 0, st>>>(segs, nseg, work, nwork, queue, soup, tinfo,
                                                      cand_off, cand, brick_emax, band_cells, o,
                                                      stats);
    } else {
        if (brick == 4)
            k_sdf_fp64<4, 64><<<grid, 64, 0, st>>>(segs, nseg, work, nwork, queue, soup, tinfo,
                                                   cand_off, cand, o, stats);
        else
            k_sdf_fp64<8, 128><<<grid, 128, 0, st>>>(segs, nseg, work, nwork, queue, soup, tinfo,
                                                     cand_off, cand, o, stats);
    }
    CMG_LAUNCH();
}

}  // namespace cmg::gpu
