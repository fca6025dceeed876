// cmg_sdf.cuh — device pieces shared by the signed-distance kernels.
#pragma once

#include <cfloat>
#include <climits>

#include "cmg_device.cuh"
#include "cmg_types.h"

namespace cmg::gpu {
namespace sdf {

constexpr float kU32 = 5.9604645e-8f;  // 2^-24
constexpr double kU64 = 1.1102230246251565e-16;  // 2^-53

// ------------------------------------------------------------------ FP64 Ericson
// Squared distance and region, reference operation order (src/voxelize/
// voxelize.cpp:202-247); regions 0 a, 1 b, 2 ab, 3 c, 4 ac, 5 bc, 6 interior.
__device__ __forceinline__ double dot3r(double ax, double ay, double az, double bx, double by,
                                        double bz) {
    return dadd(dadd(dmul(ax, bx), dmul(ay, by)), dmul(az, bz));
}
__device__ __forceinline__ double d2r(const d3& p, double qx, double qy, double qz) {
    double dx = dsub(p.x, qx), dy = dsub(p.y, qy), dz = dsub(p.z, qz);
    return dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
}

static __device__ __noinline__ double ericson(const d3& p, const d3& a, const d3& b, const d3& c,
                                              int* region) {
    double abx = dsub(b.x, a.x), aby = dsub(b.y, a.y), abz = dsub(b.z, a.z);
    double acx = dsub(c.x, a.x), acy = dsub(c.y, a.y), acz = dsub(c.z, a.z);
    double apx = dsub(p.x, a.x), apy = dsub(p.y, a.y), apz = dsub(p.z, a.z);
    double d1 = dot3r(abx, aby, abz, apx, apy, apz), d2 = dot3r(acx, acy, acz, apx, apy, apz);
    if (d1 <= 0 && d2 <= 0) { *region = 0; return d2r(p, a.x, a.y, a.z); }
    double bpx = dsub(p.x, b.x), bpy = dsub(p.y, b.y), bpz = dsub(p.z, b.z);
    double d3v = dot3r(abx, aby, abz, bpx, bpy, bpz), d4 = dot3r(acx, acy, acz, bpx, bpy, bpz);
    if (d3v >= 0 && d4 <= d3v) { *region = 1; return d2r(p, b.x, b.y, b.z); }
    double vc = dsub(dmul(d1, d4), dmul(d3v, d2));
    if (vc <= 0 && d1 >= 0 && d3v <= 0) {
        double v = ddiv(d1, dsub(d1, d3v));
        *region = 2;
        return d2r(p, dadd(a.x, dmul(v, abx)), dadd(a.y, dmul(v, aby)), dadd(a.z, dmul(v, abz)));
    }
    double cpx = dsub(p.x, c.x), cpy = dsub(p.y, c.y), cpz = dsub(p.z, c.z);
    double d5 = dot3r(abx, aby, abz, cpx, cpy, cpz), d6 = dot3r(acx, acy, acz, cpx, cpy, cpz);
    if (d6 >= 0 && d5 <= d6) { *region = 3; return d2r(p, c.x, c.y, c.z); }
    double vb = dsub(dmul(d5, d2), dmul(d1, d6));
    if (vb <= 0 && d2 >= 0 && d6 <= 0) {
        double w = ddiv(d2, dsub(d2, d6));
        *region = 4;
        return d2r(p, dadd(a.x, dmul(w, acx)), dadd(a.y, dmul(w, acy)), dadd(a.z, dmul(w, acz)));
    }
    double va = dsub(dmul(d3v, d6), dmul(d5, d4));
    double d43 = dsub(d4, d3v), d56 = dsub(d5, d6);
    if (va <= 0 && d43 >= 0 && d56 >= 0) {
        double w = ddiv(d43, dadd(d43, d56));
        *region = 5;
        return d2r(p, dadd(b.x, dmul(w, dsub(c.x, b.x))), dadd(b.y, dmul(w, dsub(c.y, b.y))),
                   dadd(b.z, dmul(w, dsub(c.z, b.z))));
    }
    double denom = ddiv(1.0, dadd(dadd(va, vb), vc));
    double v = dmul(vb, denom), w = dmul(vc, denom);
    *region = 6;
    return d2r(p, dadd(dadd(a.x, dmul(abx, v)), dmul(acx, w)),
               dadd(dadd(a.y, dmul(aby, v)), dmul(acy, w)),
               dadd(dadd(a.z, dmul(abz, v)), dmul(acz, w)));
}

__device__ __forceinline__ void load_soup(const double* __restrict__ soup, int64_t t, d3& a, d3& b,
                                          d3& c) {
    const double2* r = reinterpret_cast<const double2*>(soup + t * kSoupStride);
    double2 v0 = __ldg(r), v1 = __ldg(r + 1), v2 = __ldg(r + 2), v3 = __ldg(r + 3), v4 = __ldg(r + 4);
    a = {v0.x, v0.y, v1.x};
    b = {v1.y, v2.x, v2.y};
    c = {v3.x, v3.y, v4.x};
}

// ------------------------------------------------------------------ FP32 record
// Translation-invariant FP32 data of a triangle, computed once from FP64: vertex
// offsets from the centroid, edges (v1-v0, v2-v1, v0-v2), unit normal, in-plane
// inward edge normals (n x e_k), 1/|e_k|^2 (0 for a degenerate edge), a flag
// that allows the plane branch (nonzero area), and a bound on the distance of the
// FP32 unit normal from the exact one (0 for a degenerate triangle).
struct alignas(16) TriRec {
    float o0[3], o1[3], o2[3];
    float e0[3], e1[3], e2[3];
    float nn[3];
    float m0[3], m1[3], m2[3];
    float inv[3];
    float ok;
    float nerr;
    float pad_;
};
static_assert(sizeof(TriRec) == 144, "record layout");

__device__ __forceinline__ void load_rec(const TriRec* __restrict__ recs, int t, TriRec& r) {
    const float4* s = reinterpret_cast<const float4*>(recs + t);
    float4* d = reinterpret_cast<float4*>(&r);
#pragma unroll
    for (int i = 0; i < 9; ++i) d[i] = __ldg(s + i);
}

// Squared FP32 distance from a point to the triangle, given (dx,dy,dz) = point -
// centroid; region numbered as the FP64 Ericson regions. A point that projects inside
// a non-degenerate triangle (every in-plane edge function >= 0) is at its plane
// distance; otherwise its nearest point lies on the boundary, and the distance is the
// smallest of the three segment distances (the segment of a satisfied edge is never
// nearer than the triangle, so the minimum is the boundary distance up to rounding,
// within the same bound as each segment distance). Every lane measures all three
// segments: no branch splits a warp whose cells lie in different regions.
// Explicit intrinsics fix the operation sequence, so the value does not depend on
// whether the region is wanted (REG) or on the inlining context.
__device__ __forceinline__ float dot3f(float ax, float ay, float az, const float* b) {
    return fmaf(ax, b[0], fmaf(ay, b[1], __fmul_rn(az, b[2])));
}

__device__ __forceinline__ void seg2(float px, float py, float pz, const float* e, float inv,
                                     float& d, float& t) {
    t = __saturatef(__fmul_rn(dot3f(px, py, pz, e), inv));
    const float qx = fmaf(-t, e[0], px), qy = fmaf(-t, e[1], py), qz = fmaf(-t, e[2], pz);
    d = fmaf(qx, qx, fmaf(qy, qy, __fmul_rn(qz, qz)));
}

template <bool REG>
__device__ __forceinline__ float dist_rec_t(const TriRec& r, float dx, float dy, float dz, int* reg) {
    const float pax = __fsub_rn(dx, r.o0[0]), pay = __fsub_rn(dy, r.o0[1]), paz = __fsub_rn(dz, r.o0[2]);
    const float pbx = __fsub_rn(dx, r.o1[0]), pby = __fsub_rn(dy, r.o1[1]), pbz = __fsub_rn(dz, r.o1[2]);
    const float pcx = __fsub_rn(dx, r.o2[0]), pcy = __fsub_rn(dy, r.o2[1]), pcz = __fsub_rn(dz, r.o2[2]);
    const float s0 = dot3f(pax, pay, paz, r.m0);
    const float s1 = dot3f(pbx, pby, pbz, r.m1);
    const float s2 = dot3f(pcx, pcy, pcz, r.m2);
    const float dp = dot3f(pax, pay, paz, r.nn);
    float d0, t0, d1, t1, d2, t2;
    seg2(pax, pay, paz, r.e0, r.inv[0], d0, t0);
    seg2(pbx, pby, pbz, r.e1, r.inv[1], d1, t1);
    seg2(pcx, pcy, pcz, r.e2, r.inv[2], d2, t2);
    const bool face = r.ok > 0.f && s0 >= 0.f && s1 >= 0.f && s2 >= 0.f;
    float d = d0;
    int g = 0;
    if (REG) g = t0 <= 0.f ? 0 : (t0 >= 1.f ? 1 : 2);
    if (d1 < d) {
        d = d1;
        if (REG) g = t1 <= 0.f ? 1 : (t1 >= 1.f ? 3 : 5);
    }
    if (d2 < d) {
        d = d2;
        if (REG) g = t2 <= 0.f ? 3 : (t2 >= 1.f ? 0 : 4);
    }
    if (face) {
        d = __fmul_rn(dp, dp);
        g = 6;
    }
    if (REG) *reg = g;
    return d;
}

// The distance and its region.
__device__ __forceinline__ float dist_rec(const TriRec& r, float dx, float dy, float dz, int* reg) {
    return dist_rec_t<true>(r, dx, dy, dz, reg);
}
// The distance alone (the same value as dist_rec).
__device__ __forceinline__ float dist_rec_val(const TriRec& r, float dx, float dy, float dz) {
    return dist_rec_t<false>(r, dx, dy, dz, nullptr);
}

// ------------------------------------------------------------------ outputs
struct Out {
    const uint8_t* occ;
    float* sdf32;
    double* sdf64;
    int* near_tri;
    uint8_t* near_reg;
    float* errbound;  // mixed: per-cell stated FP32 error bound (nullable)
};

__device__ __forceinline__ void write_cell(const Out& o, int64_t idx, double d, int tri, int reg) {
    const bool in = o.occ[idx] != 0;
    const double sd = in ? -d : d;
    if (o.sdf64) o.sdf64[idx] = sd;
    if (o.sdf32) o.sdf32[idx] = __double2float_rn(sd);
    if (o.near_tri) o.near_tri[idx] = tri;
    if (o.near_reg) o.near_reg[idx] = static_cast<uint8_t>(reg);
}

// Splits x (FP64) into hi = fl32(x) and lo = fl32(x - hi): hi + lo carries ~48
// bits, so differences of nearby points can be formed in FP32 without losing
// the bits that an FP32 subtraction of far-from-zero coordinates would drop.
__device__ __forceinline__ void split2(double x, float& hi, float& lo) {
    hi = __double2float_rn(x);
    lo = __double2float_rn(x - static_cast<double>(hi));
}

}  // namespace sdf
}  // namespace cmg::gpu
