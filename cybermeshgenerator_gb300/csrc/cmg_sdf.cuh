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
// Translation-invariant FP32 data of a triangle (a, b, c), computed once from FP64, in
// the triangle's own orthonormal frame (u, v, n): u along b - a, v in the triangle's
// plane toward c, n = u x v. In that frame a = (0, 0), b = (bx, 0), c = (cx, cy) with
// cy >= 0, the triangle lies in the plane n = 0, and a point's squared distance is its
// squared in-plane distance to the 2-D triangle plus its squared n component. The frame
// is built by two Gram-Schmidt passes, so b and c lie in it to FP64 rounding even for
// slivers and collinear or repeated vertices (then v is any unit vector across u).
struct alignas(16) TriRec {
    float o0[3];       // a - centroid
    float nn[3];       // n
    float nerr;        // bound on |n (FP32) - n| (the plane test's normal error)
    float uu[3];       // u
    float vv[3];       // v
    float bx;          // |b - a|
    float cx, cy;      // c - a in the frame
    float e1x;         // (c - b) . u
    float ib;          // 1 / bx (0 if a == b)
    float inv1, inv2;  // 1 / |c - b|^2, 1 / |c - a|^2 (0 for a zero edge)
    float ok;          // 1: the face branch is allowed (bx > 0 and cy > 0)
    float pad_[3];
};
static_assert(sizeof(TriRec) == 96, "record layout");
constexpr int kRecVec = static_cast<int>(sizeof(TriRec) / 16);  // float4 words per record

__device__ __forceinline__ void load_rec(const TriRec* __restrict__ recs, int t, TriRec& r) {
    const float4* s = reinterpret_cast<const float4*>(recs + t);
    float4* d = reinterpret_cast<float4*>(&r);
#pragma unroll
    for (int i = 0; i < kRecVec; ++i) d[i] = __ldg(s + i);
}

__device__ __forceinline__ float dot3f(float ax, float ay, float az, const float* b) {
    return fmaf(ax, b[0], fmaf(ay, b[1], __fmul_rn(az, b[2])));
}

// The point's offset from a, pa = (point - centroid) - (a - centroid), and its n
// component: the first steps of the distance, shared with the plane test.
struct PaN {
    float x, y, z, n;
};
__device__ __forceinline__ PaN pa_n(const TriRec& r, float dx, float dy, float dz) {
    PaN p;
    p.x = __fsub_rn(dx, r.o0[0]);
    p.y = __fsub_rn(dy, r.o0[1]);
    p.z = __fsub_rn(dz, r.o0[2]);
    p.n = dot3f(p.x, p.y, p.z, r.nn);
    return p;
}

// Squared FP32 distance from a point to the triangle, from pa_n; region numbered as the
// FP64 Ericson regions (0 a, 1 b, 2 ab, 3 c, 4 ac, 5 bc, 6 face). In the frame the
// point is (pu, pv, pn); it projects inside when the three 2-D edge functions
// (pv, (c - b) x (p - b), (a - c) x (p - c)) are >= 0 and the triangle has area, and
// is then at |pn|; otherwise its nearest point is on the boundary, at the smallest of
// the three 2-D segment distances (each with pn^2 added once at the end). Every lane
// measures all three segments: no branch splits a warp whose cells lie in different
// regions. Explicit intrinsics fix the operation sequence, so the value does not depend
// on whether the region is wanted (REG) or on the inlining context.
// Error (u = 2^-24, d the distance, e the largest centroid-to-vertex distance, r the
// sub-brick radius): pa errs by at most u (3 r + 4 d + 6 e) (the recentring, as
// before), |pa| <= d + 2 e; the frame rounded to FP32 and the three dots move the
// point by at most 7 u |pa|, the FP32 2-D vertices the triangle by 3 u e; the segment
// parameter, the residual and the sums add at most 7 u (d + 2 e), a face decision on
// the wrong side of an edge 4 u (d + 2 e): together below u (22 d + 39 e + 3 r), well
// inside the stated 48 u (d + 2 e + 2 r).
template <bool REG>
__device__ __forceinline__ float dist_rec_t(const TriRec& r, const PaN& p, int* reg) {
    const float pu = dot3f(p.x, p.y, p.z, r.uu), pv = dot3f(p.x, p.y, p.z, r.vv);
    const float qu1 = __fsub_rn(pu, r.bx);
    const float qu2 = __fsub_rn(pu, r.cx), qv2 = __fsub_rn(pv, r.cy);
    const float s1 = fmaf(r.e1x, pv, -__fmul_rn(r.cy, qu1));
    const float s2 = fmaf(r.cy, qu2, -__fmul_rn(r.cx, qv2));
    // a -> b along u
    const float t0 = __saturatef(__fmul_rn(pu, r.ib));
    const float r0u = fmaf(-t0, r.bx, pu);
    const float d0 = fmaf(r0u, r0u, __fmul_rn(pv, pv));
    // b -> c, direction (e1x, cy)
    const float t1 = __saturatef(__fmul_rn(fmaf(qu1, r.e1x, __fmul_rn(pv, r.cy)), r.inv1));
    const float r1u = fmaf(-t1, r.e1x, qu1), r1v = fmaf(-t1, r.cy, pv);
    const float d1 = fmaf(r1u, r1u, __fmul_rn(r1v, r1v));
    // c -> a, direction (-cx, -cy)
    const float t2 = __saturatef(__fmul_rn(-fmaf(qu2, r.cx, __fmul_rn(qv2, r.cy)), r.inv2));
    const float r2u = fmaf(t2, r.cx, qu2), r2v = fmaf(t2, r.cy, qv2);
    const float d2 = fmaf(r2u, r2u, __fmul_rn(r2v, r2v));
    const bool face = r.ok > 0.f && pv >= 0.f && s1 >= 0.f && s2 >= 0.f;
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
        d = 0.f;
        g = 6;
    }
    if (REG) *reg = g;
    return fmaf(p.n, p.n, d);
}

// The distance and its region.
__device__ __forceinline__ float dist_rec(const TriRec& r, float dx, float dy, float dz, int* reg) {
    return dist_rec_t<true>(r, pa_n(r, dx, dy, dz), reg);
}
// The distance alone (the same value as dist_rec).
__device__ __forceinline__ float dist_rec_val(const TriRec& r, float dx, float dy, float dz) {
    return dist_rec_t<false>(r, pa_n(r, dx, dy, dz), nullptr);
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
