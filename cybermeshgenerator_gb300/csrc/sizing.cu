// sizing.cu — the background-mesh sizing field evaluated for batches of query points.
//
// Semantics of the reference (src/sizing/background.cpp:29-74): node sizes padded with
// 0 or truncated to the node count; for a query p, the first tetrahedron in order
// whose determinant value D = orient3d(v0, v1, v2, v3) is not zero and whose four
// weights w_i = orient3d(.. p in place of v_i ..) / D are all >= -1e-9 gives
// (w0 s0 + w1 s1 + w2 s2 + w3 s3) * scale; otherwise the size of the nearest node
// (smallest rounded squared distance from DBL_MAX, first index on ties) times scale.
// orient3d is the reference's VALUE (src/predicates/robust.cpp:36-42): the rounded
// determinant when it is not zero (the predicates run with a zero static filter), else
// the adaptive routine's answer (o3_adapt below). This file compiles with -fmad=false:
// every product and sum rounds separately, as the reference's x86-64 build does;
// exact products use __fma_rn explicitly.
//
// Device plan. The reference scans every tetrahedron per query. Here each
// tetrahedron with D != 0 is binned into the cells of a uniform grid over the domain
// Dom (the nodes' box grown by half its extent) that meet its bounding box inflated by
// a margin m outside which the reference's rounded test provably fails for every
// query in Dom:
//   * if all exact barycentrics of p are >= -eta, p lies within the box inflated by
//     3 eta L (L its largest extent), so min_i lambda_i(p) <= -delta(p) / (3 L), delta
//     the distance (max-norm) from p to the box;
//   * |w_i - lambda_i| <= c (delta + L)^3 with c from the orient3d error bound
//     (16 u times the permanent, the permanent at most 6 (delta + L)^3), the error of D
//     and of the division;
//   * so a passing p has g(delta) = delta / (3 L) - 1e-9 - c (delta + L)^3 <= 0; g is
//     concave, so g > 0 at m and at the farthest point of Dom means g > 0 in between
//     and nothing beyond m passes.
// Tetrahedra for which no such m exists (slivers, or tiny ones far from Dom's
// corners) are tested by every query (the global list). A query tests the merged
// ascending candidates of its cell and the global list and stops at the first pass
// (the smallest passing index, as the reference's scan). Queries outside Dom or not
// finite take the reference's scan itself (one warp per query). The nearest node comes
// from a ring search over a second grid on the nodes' box, with a lower bound on the
// rounded squared distance of every unvisited node.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "cmg_util.h"
#include "engine_kernels.h"

namespace cmg::gpu {

namespace {

constexpr int kThreads = 256;
constexpr double kU = 1.1102230246251565e-16;  // 2^-53
constexpr double kEps = -1e-9;                  // background.cpp:39

// ------------------------------------------------------------ orient3d value

struct P3 {
    double x, y, z;
};

__device__ __forceinline__ void two_sum(double a, double b, double& x, double& y) {
    x = a + b;
    const double bv = x - a, av = x - bv;
    y = (a - av) + (b - bv);
}
__device__ __forceinline__ void fast_two_sum(double a, double b, double& x, double& y) {
    x = a + b;
    y = b - (x - a);
}
__device__ __forceinline__ double diff_tail(double a, double b, double x) {
    const double bv = a - x, av = x + bv;
    return (a - av) + (bv - b);
}
__device__ __forceinline__ void two_prod(double a, double b, double& x, double& y) {
    x = a * b;
    y = __fma_rn(a, b, -x);  // the exact error of the product
}
// (a1, a0) - (b1, b0) -> x[0..3], x[3] the largest
__device__ __forceinline__ void two_two_diff(double a1, double a0, double b1, double b0, double* x) {
    double i, j, z;
    i = a0 - b0;
    x[0] = diff_tail(a0, b0, i);
    two_sum(a1, i, j, z);
    i = z - b1;
    x[1] = diff_tail(z, b1, i);
    two_sum(j, i, x[3], x[2]);
}
// (a1, a0) * b -> x[0..3]
__device__ __forceinline__ void two_one_prod(double a1, double a0, double b, double* x) {
    double i, j, z, k;
    two_prod(a0, b, i, x[0]);
    two_prod(a1, b, j, z);
    two_sum(i, z, k, x[1]);
    fast_two_sum(j, k, x[3], x[2]);
}
__device__ __forceinline__ bool take_e(double e, double f) { return (f > e) == (f > -e); }

// Zero-eliminating sum of two expansions, merged smallest magnitude first.
static __device__ __noinline__ int xsum(int elen, const double* e, int flen, const double* f,
                                        double* h) {
    int ei = 0, fi = 0, hi = 0;
    double en = e[0], fn = f[0], q, qn, hh;
    if (take_e(en, fn)) {
        q = en;
        en = ++ei < elen ? e[ei] : 0.0;
    } else {
        q = fn;
        fn = ++fi < flen ? f[fi] : 0.0;
    }
    if (ei < elen && fi < flen) {
        if (take_e(en, fn)) {
            fast_two_sum(en, q, qn, hh);
            en = ++ei < elen ? e[ei] : 0.0;
        } else {
            fast_two_sum(fn, q, qn, hh);
            fn = ++fi < flen ? f[fi] : 0.0;
        }
        q = qn;
        if (hh != 0.0) h[hi++] = hh;
        while (ei < elen && fi < flen) {
            if (take_e(en, fn)) {
                two_sum(q, en, qn, hh);
                en = ++ei < elen ? e[ei] : 0.0;
            } else {
                two_sum(q, fn, qn, hh);
                fn = ++fi < flen ? f[fi] : 0.0;
            }
            q = qn;
            if (hh != 0.0) h[hi++] = hh;
        }
    }
    for (; ei < elen;) {
        two_sum(q, en, qn, hh);
        en = ++ei < elen ? e[ei] : 0.0;
        q = qn;
        if (hh != 0.0) h[hi++] = hh;
    }
    for (; fi < flen;) {
        two_sum(q, fn, qn, hh);
        fn = ++fi < flen ? f[fi] : 0.0;
        q = qn;
        if (hh != 0.0) h[hi++] = hh;
    }
    if (q != 0.0 || hi == 0) h[hi++] = q;
    return hi;
}

// Zero-eliminating product of an expansion and a double.
static __device__ __noinline__ int xscale(int elen, const double* e, double b, double* h) {
    double q, hh, p1, p0, s;
    int hi = 0;
    two_prod(e[0], b, q, hh);
    if (hh != 0.0) h[hi++] = hh;
    for (int i = 1; i < elen; ++i) {
        two_prod(e[i], b, p1, p0);
        two_sum(q, p0, s, hh);
        if (hh != 0.0) h[hi++] = hh;
        fast_two_sum(p1, s, q, hh);
        if (hh != 0.0) h[hi++] = hh;
    }
    if (q != 0.0 || hi == 0) h[hi++] = q;
    return hi;
}

// The two tail products of one point: first = tx * p_y - ty * p_x, second = ty * q_x -
// tx * q_y, each as 1, 2 or 4 components (built the cheaper way when a tail is zero).
__device__ __forceinline__ void tail_pair(double tx, double ty, double p_x, double p_y, double q_x,
                                          double q_y, double* first, int& n1, double* second,
                                          int& n2) {
    if (tx == 0.0) {
        if (ty == 0.0) {
            first[0] = 0.0;
            second[0] = 0.0;
            n1 = n2 = 1;
        } else {
            two_prod(-ty, p_x, first[1], first[0]);
            two_prod(ty, q_x, second[1], second[0]);
            n1 = n2 = 2;
        }
    } else if (ty == 0.0) {
        two_prod(tx, p_y, first[1], first[0]);
        two_prod(-tx, q_y, second[1], second[0]);
        n1 = n2 = 2;
    } else {
        double a1, a0, b1, b0;
        two_prod(tx, p_y, a1, a0);
        two_prod(ty, p_x, b1, b0);
        two_two_diff(a1, a0, b1, b0, first);
        two_prod(ty, q_x, a1, a0);
        two_prod(tx, q_y, b1, b0);
        two_two_diff(a1, a0, b1, b0, second);
        n1 = n2 = 4;
    }
}

struct Fin {
    double a[192], b[192];
    double* now;
    double* other;
    int n;
    __device__ void add(int elen, const double* e) {
        n = xsum(n, now, elen, e, other);
        double* t = now;
        now = other;
        other = t;
    }
};

// The adaptive stages of the reference's orient3d (Shewchuk's published algorithm),
// reached only when the rounded determinant is zero.
static __device__ __noinline__ double o3_adapt(const P3& pa, const P3& pb, const P3& pc,
                                               const P3& pd, double permanent) {
    const double adx = pa.x - pd.x, bdx = pb.x - pd.x, cdx = pc.x - pd.x;
    const double ady = pa.y - pd.y, bdy = pb.y - pd.y, cdy = pc.y - pd.y;
    const double adz = pa.z - pd.z, bdz = pb.z - pd.z, cdz = pc.z - pd.z;
    double bc[4], ca[4], ab[4], adet[8], bdet[8], cdet[8], abdet[16];
    double x1, x0, y1, y0;
    Fin F;
    F.now = F.a;
    F.other = F.b;

    two_prod(bdx, cdy, x1, x0);
    two_prod(cdx, bdy, y1, y0);
    two_two_diff(x1, x0, y1, y0, bc);
    const int alen = xscale(4, bc, adz, adet);
    two_prod(cdx, ady, x1, x0);
    two_prod(adx, cdy, y1, y0);
    two_two_diff(x1, x0, y1, y0, ca);
    const int blen = xscale(4, ca, bdz, bdet);
    two_prod(adx, bdy, x1, x0);
    two_prod(bdx, ady, y1, y0);
    two_two_diff(x1, x0, y1, y0, ab);
    const int clen = xscale(4, ab, cdz, cdet);
    const int ablen = xsum(alen, adet, blen, bdet, abdet);
    F.n = xsum(ablen, abdet, clen, cdet, F.now);

    double det = F.now[0];
    for (int i = 1; i < F.n; ++i) det = det + F.now[i];
    double bound = (3.0 + 28.0 * kU) * kU * permanent;
    if (det >= bound || -det >= bound) return det;

    const double adxt = diff_tail(pa.x, pd.x, adx), bdxt = diff_tail(pb.x, pd.x, bdx),
                 cdxt = diff_tail(pc.x, pd.x, cdx), adyt = diff_tail(pa.y, pd.y, ady),
                 bdyt = diff_tail(pb.y, pd.y, bdy), cdyt = diff_tail(pc.y, pd.y, cdy),
                 adzt = diff_tail(pa.z, pd.z, adz), bdzt = diff_tail(pb.z, pd.z, bdz),
                 cdzt = diff_tail(pc.z, pd.z, cdz);
    if (adxt == 0.0 && bdxt == 0.0 && cdxt == 0.0 && adyt == 0.0 && bdyt == 0.0 && cdyt == 0.0 &&
        adzt == 0.0 && bdzt == 0.0 && cdzt == 0.0)
        return det;

    bound = (26.0 + 288.0 * kU) * kU * kU * permanent + (3.0 + 8.0 * kU) * kU * fabs(det);
    const double ta = adz * ((bdx * cdyt + cdy * bdxt) - (bdy * cdxt + cdx * bdyt)) +
                      adzt * (bdx * cdy - bdy * cdx);
    const double tb = bdz * ((cdx * adyt + ady * cdxt) - (cdy * adxt + adx * cdyt)) +
                      bdzt * (cdx * ady - cdy * adx);
    const double tc = cdz * ((adx * bdyt + bdy * adxt) - (ady * bdxt + bdx * adyt)) +
                      cdzt * (adx * bdy - ady * bdx);
    det = det + ((ta + tb) + tc);
    if (det >= bound || -det >= bound) return det;

    double at_b[4], at_c[4], bt_c[4], bt_a[4], ct_a[4], ct_b[4];
    int at_bn, at_cn, bt_cn, bt_an, ct_an, ct_bn;
    tail_pair(adxt, adyt, bdx, bdy, cdx, cdy, at_b, at_bn, at_c, at_cn);
    tail_pair(bdxt, bdyt, cdx, cdy, adx, ady, bt_c, bt_cn, bt_a, bt_an);
    tail_pair(cdxt, cdyt, adx, ady, bdx, bdy, ct_a, ct_an, ct_b, ct_bn);

    double bct[8], cat[8], abt[8], w[16], v[12], u[4];
    const int bctn = xsum(bt_cn, bt_c, ct_bn, ct_b, bct);
    F.add(xscale(bctn, bct, adz, w), w);
    const int catn = xsum(ct_an, ct_a, at_cn, at_c, cat);
    F.add(xscale(catn, cat, bdz, w), w);
    const int abtn = xsum(at_bn, at_b, bt_an, bt_a, abt);
    F.add(xscale(abtn, abt, cdz, w), w);
    if (adzt != 0.0) F.add(xscale(4, bc, adzt, v), v);
    if (bdzt != 0.0) F.add(xscale(4, ca, bdzt, v), v);
    if (cdzt != 0.0) F.add(xscale(4, ab, cdzt, v), v);

    // tail x tail products: point k's x tail with the next point's y tail (scaled by
    // the third point's z difference and tail), and with the previous one's (negated,
    // scaled by the middle point's)
    const double tx[3] = {adxt, bdxt, cdxt};
    const double ty_next[3] = {bdyt, cdyt, adyt}, ty_prev[3] = {cdyt, adyt, bdyt};
    const double zd_third[3] = {cdz, adz, bdz}, zt_third[3] = {cdzt, adzt, bdzt};
    const double zd_mid[3] = {bdz, cdz, adz}, zt_mid[3] = {bdzt, cdzt, adzt};
    for (int k = 0; k < 3; ++k) {
        if (tx[k] == 0.0) continue;
        double p1, p0;
        if (ty_next[k] != 0.0) {
            two_prod(tx[k], ty_next[k], p1, p0);
            two_one_prod(p1, p0, zd_third[k], u);
            F.add(4, u);
            if (zt_third[k] != 0.0) {
                two_one_prod(p1, p0, zt_third[k], u);
                F.add(4, u);
            }
        }
        if (ty_prev[k] != 0.0) {
            two_prod(-tx[k], ty_prev[k], p1, p0);
            two_one_prod(p1, p0, zd_mid[k], u);
            F.add(4, u);
            if (zt_mid[k] != 0.0) {
                two_one_prod(p1, p0, zt_mid[k], u);
                F.add(4, u);
            }
        }
    }
    if (adzt != 0.0) F.add(xscale(bctn, bct, adzt, w), w);
    if (bdzt != 0.0) F.add(xscale(catn, cat, bdzt, w), w);
    if (cdzt != 0.0) F.add(xscale(abtn, abt, cdzt, w), w);
    return F.now[F.n - 1];
}

// robust::orient3d(a, b, c, d): the rounded determinant in the reference's order when
// it is not zero, else the adaptive answer.
__device__ __forceinline__ double o3_value(const P3& a, const P3& b, const P3& c, const P3& d) {
    const double adx = a.x - d.x, ady = a.y - d.y, adz = a.z - d.z;
    const double bdx = b.x - d.x, bdy = b.y - d.y, bdz = b.z - d.z;
    const double cdx = c.x - d.x, cdy = c.y - d.y, cdz = c.z - d.z;
    const double bdxcdy = bdx * cdy, cdxbdy = cdx * bdy;
    const double cdxady = cdx * ady, adxcdy = adx * cdy;
    const double adxbdy = adx * bdy, bdxady = bdx * ady;
    const double det = adz * (bdxcdy - cdxbdy) + bdz * (cdxady - adxcdy) + cdz * (adxbdy - bdxady);
    if (det > 0.0 || det < 0.0) return det;
    const double permanent = (fabs(bdxcdy) + fabs(cdxbdy)) * fabs(adz) +
                             (fabs(cdxady) + fabs(adxcdy)) * fabs(bdz) +
                             (fabs(adxbdy) + fabs(bdxady)) * fabs(cdz);
    const double bound = (7.0 + 56.0 * kU) * kU * permanent;
    if (det > bound || -det > bound) return det;
    return o3_adapt(a, b, c, d, permanent);
}

// ------------------------------------------------------------ tetrahedron records

struct __align__(32) Node4 {
    double x, y, z, w;  // a node and its index (exact as a double)
};

// Everything the containment test reads for one tetrahedron, and its inflated box.
struct __align__(16) TetRec {
    P3 v[4];
    double D;        // orient3d(v0, v1, v2, v3) value; 0 never answers
    double s[4];     // node sizes
};

// What a candidate is screened with before the full test, all in FP32 (the FP64 pipe
// of this part is narrow): the inflated box rounded outward, and the barycentric
// coordinates lambda_i(p) = [i == 3] + g_i . (p - v3) with the error terms that make the
// screen safe. A candidate is dropped only when some lambda_i provably lies below thr =
// -1e-9 - e64, where e64 bounds |w_i - lambda_i| for the reference's rounded w_i
// everywhere in the inflated box: its test would fail.
struct __align__(16) TetFilt {
    float blo[3], bhi[3];  // inflated box, rounded outward
    float v3h[3], v3l[3];  // v3 = hi + lo to 2^-48
    float g[12];           // g_0 .. g_3, rounded to FP32
    float eg;              // bound on |g (exact) - g (FP64)| per component
    float thr;             // NaN: no screen
};

// A query in the screen's terms: p rounded down and up (the box test) and as hi + lo.
struct Q32 {
    float lo[3], hi[3];
    float ph[3], pl[3];
};

__device__ __forceinline__ Q32 make_q32(const P3& p) {
    Q32 q;
    const double c[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        q.lo[a] = __double2float_rd(c[a]);
        q.hi[a] = __double2float_ru(c[a]);
        q.ph[a] = __double2float_rn(c[a]);
        q.pl[a] = __double2float_rn(c[a] - static_cast<double>(q.ph[a]));
    }
    return q;
}

__device__ __forceinline__ bool outside_box(const TetFilt& f, const Q32& q) {
    return q.hi[0] < f.blo[0] || q.lo[0] > f.bhi[0] || q.hi[1] < f.blo[1] || q.lo[1] > f.bhi[1] ||
           q.hi[2] < f.blo[2] || q.lo[2] > f.bhi[2];
}

// True when the screen proves the reference's test fails for this candidate.
__device__ __forceinline__ bool screened_out(const TetFilt& f, const Q32& q) {
    if (!(f.thr <= 0.0f)) return false;
    float x[3], ex[3];
    float S = 0.0f, E = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        // x = (ph - v3h) + (pl - v3l): three roundings, and the two hi/lo splits
        const float d1 = q.ph[a] - f.v3h[a], d2 = q.pl[a] - f.v3l[a];
        x[a] = d1 + d2;
        const float r = __fadd_ru(__fadd_ru(fabsf(d1), fabsf(d2)), fabsf(x[a]));
        ex[a] = __fmaf_ru(r, 6.0e-8f, __fmul_ru(__fadd_ru(fabsf(q.ph[a]), fabsf(f.v3h[a])), 7.2e-15f));
        S = __fadd_ru(S, fabsf(x[a]));
        E = __fadd_ru(E, ex[a]);
    }
    const float egt = __fmul_ru(f.eg, __fadd_ru(S, E));
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float gx = f.g[3 * i], gy = f.g[3 * i + 1], gz = f.g[3 * i + 2];
        const float est = fmaf(gx, x[0], fmaf(gy, x[1], fmaf(gz, x[2], i == 3 ? 1.0f : 0.0f)));
        const float A = __fmaf_ru(fabsf(gx), fabsf(x[0]),
                                  __fmaf_ru(fabsf(gy), fabsf(x[1]), __fmul_ru(fabsf(gz), fabsf(x[2]))));
        const float GE = __fmaf_ru(fabsf(gx), ex[0], __fmaf_ru(fabsf(gy), ex[1], __fmul_ru(fabsf(gz), ex[2])));
        const float gs = __fadd_ru(__fadd_ru(fabsf(gx), fabsf(gy)), fabsf(gz));
        // rounding of g (2^-24) and of the three fused steps (3 2^-24) on A; the error of
        // g in FP64 (eg) on |x| + its error; |g| times the error of x; the constant 1 of
        // lambda_3 in the fused steps; flushed tiny x
        float bound = __fmaf_ru(A, 2.41e-7f, __fmul_ru(__fadd_ru(egt, GE), 1.01f));
        bound = __fmaf_ru(gs, 1.2e-38f, __fadd_ru(bound, i == 3 ? 2e-7f : 0.0f));
        if (__fadd_ru(est, bound) < f.thr) return true;
    }
    return false;
}

struct Grid {
    double lo[3];
    double h;
    int n[3];
};

// A grid's corner and cell size rounded down and up to FP32, and the bound on how far
// a point may lie beyond the faces of the cell a rounded quotient put it in.
struct GridF {
    float lo_rd[3], lo_ru[3];
    float h_rd, h_ru;
    float tol[3];
};

__device__ __forceinline__ int cell_axis(double x, double lo, double h, int n) {
    // monotone in x: (x - lo) / h rounded, then floor; the binning and the queries use it alike
    int i = __double2int_rd((x - lo) / h);
    return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

// The reference's test for one tetrahedron: true with *out = the interpolated size.
__device__ __forceinline__ bool interp(const TetRec& r, const P3& p, double& out) {
    const double w0 = o3_value(p, r.v[1], r.v[2], r.v[3]) / r.D;
    const double w1 = o3_value(r.v[0], p, r.v[2], r.v[3]) / r.D;
    const double w2 = o3_value(r.v[0], r.v[1], p, r.v[3]) / r.D;
    const double w3 = o3_value(r.v[0], r.v[1], r.v[2], p) / r.D;
    if (w0 < kEps || w1 < kEps || w2 < kEps || w3 < kEps) return false;
    out = w0 * r.s[0] + w1 * r.s[1] + w2 * r.s[2] + w3 * r.s[3];
    return true;
}

enum : int { kNever = 0, kBinned = 1, kGlobal = 2 };
constexpr int kMaxCellsPerTet = 4096;

// g(delta) = delta / (3 L) - 1e-9 - c (delta + L)^3 > 0, with slack for its own rounding.
__device__ __forceinline__ bool gap_positive(double delta, double L, double c) {
    const double a = delta / (3.0 * L);
    const double t = delta + L;
    const double b = 1e-9 + c * t * t * t;
    return a * (1.0 - 1e-12) > b * (1.0 + 1e-12);
}

// Per tetrahedron: record, determinant value, margin and cell range (binned), or the
// global list (no margin found), or never (D == 0).
__global__ void __launch_bounds__(kThreads) k_tet_prep(const double* __restrict__ pts,
                                                       const int4* __restrict__ tets, int64_t nt,
                                                       const double* __restrict__ sizes, Grid g,
                                                       double3 dlo, double3 dhi,
                                                       TetRec* __restrict__ rec,
                                                       TetFilt* __restrict__ filt,
                                                       int* __restrict__ far,
                                                       double* __restrict__ farbox,
                                                       int* __restrict__ kind,
                                                       int* __restrict__ ncell,
                                                       int* __restrict__ cellbox) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const int4 q = tets[t];
    const int id[4] = {q.x, q.y, q.z, q.w};
    TetRec r;
    TetFilt fl;
    fl.thr = __int_as_float(0x7fc00000);  // NaN: no screen
    fl.eg = 0.0f;
    double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
    for (int k = 0; k < 4; ++k) {
        r.v[k] = P3{pts[3 * static_cast<int64_t>(id[k])], pts[3 * static_cast<int64_t>(id[k]) + 1],
                    pts[3 * static_cast<int64_t>(id[k]) + 2]};
        r.s[k] = sizes[id[k]];
        const double c[3] = {r.v[k].x, r.v[k].y, r.v[k].z};
        for (int a = 0; a < 3; ++a) {
            lo[a] = fmin(lo[a], c[a]);
            hi[a] = fmax(hi[a], c[a]);
        }
    }
    r.D = o3_value(r.v[0], r.v[1], r.v[2], r.v[3]);
    ncell[t] = 0;
    far[t] = 0;
    {
        const double v3[3] = {r.v[3].x, r.v[3].y, r.v[3].z};
        for (int a = 0; a < 3; ++a) {
            fl.v3h[a] = __double2float_rn(v3[a]);
            fl.v3l[a] = __double2float_rn(v3[a] - static_cast<double>(fl.v3h[a]));
        }
    }
    double blo[3], bhi[3];
    if (r.D == 0.0) {
        kind[t] = kNever;
        for (int a = 0; a < 3; ++a) {
            fl.blo[a] = __int_as_float(0x7f800000);  // never inside
            fl.bhi[a] = __int_as_float(0xff800000);
        }
        rec[t] = r;
        filt[t] = fl;
        return;
    }
    // error model: |D_fl - D| <= 16 u P_D, P_D <= 6 L^3; per weight |w - lambda| <= c (delta + L)^3
    double L = 0.0;
    for (int a = 0; a < 3; ++a) L = fmax(L, __dsub_ru(hi[a], lo[a]));
    const double PD = 6.0 * L * L * L * (1.0 + 1e-12);
    const double Dlb = fabs(r.D) - 16.0 * kU * PD;
    int k_out = kGlobal;
    double m = 0.0;
    if (Dlb > 0.0) {
        const double rho = 16.0 * kU * PD / Dlb;
        if (rho < 0.1) {
            const double K = ((rho + kU) * (1.0 + 4.0 * kU) + 18.0 * kU) * (1.0 + kU) /
                             ((1.0 - rho) * Dlb);
            const double c = 6.0 * (1.0 + 4.0 * kU) * K * (1.0 + 1e-12);
            for (int it = 0; it < 3; ++it) {
                const double t3 = L + m;
                m = 3.0 * L * (1e-9 + c * t3 * t3 * t3) * (1.0 + 1e-6);
            }
            // the farthest point of the domain from the box (max norm)
            double dmax = 0.0;
            dmax = fmax(dmax, fmax(__dsub_ru(lo[0], dlo.x), __dsub_ru(dhi.x, hi[0])));
            dmax = fmax(dmax, fmax(__dsub_ru(lo[1], dlo.y), __dsub_ru(dhi.y, hi[1])));
            dmax = fmax(dmax, fmax(__dsub_ru(lo[2], dlo.z), __dsub_ru(dhi.z, hi[2])));
            if (gap_positive(m, L, c)) {
                k_out = kBinned;
                if (dmax > m && !gap_positive(dmax * (1.0 + 1e-12), L, c)) {
                    // g turns negative again before the domain's far corner: queries
                    // beyond rfar (where g is still positive) must test this tetrahedron too
                    double a0 = m, a1 = dmax;
                    for (int it = 0; it < 80; ++it) {
                        const double mid = 0.5 * (a0 + a1);
                        if (gap_positive(mid, L, c)) a0 = mid;
                        else a1 = mid;
                    }
                    const double rfar = a0 * (1.0 - 1e-9);
                    if (rfar > m && gap_positive(rfar, L, c)) {
                        for (int a = 0; a < 3; ++a) {
                            farbox[6 * t + a] = __dsub_rd(lo[a], rfar);
                            farbox[6 * t + 3 + a] = __dadd_ru(hi[a], rfar);
                        }
                        far[t] = 1;
                    } else {
                        k_out = kGlobal;
                    }
                }
            }
            if (k_out == kBinned) {
                // barycentric gradients: (e1 x e2, e2 x e0, e0 x e1) / D and minus their sum
                const double e0[3] = {r.v[0].x - r.v[3].x, r.v[0].y - r.v[3].y, r.v[0].z - r.v[3].z};
                const double e1[3] = {r.v[1].x - r.v[3].x, r.v[1].y - r.v[3].y, r.v[1].z - r.v[3].z};
                const double e2[3] = {r.v[2].x - r.v[3].x, r.v[2].y - r.v[3].y, r.v[2].z - r.v[3].z};
                const double* pr[3][2] = {{e1, e2}, {e2, e0}, {e0, e1}};
                double gsum[3] = {0.0, 0.0, 0.0};
                for (int i = 0; i < 3; ++i) {
                    const double* u = pr[i][0];
                    const double* v = pr[i][1];
                    const double cr[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2],
                                          u[0] * v[1] - u[1] * v[0]};
                    for (int a = 0; a < 3; ++a) {
                        const double ga = cr[a] / r.D;
                        fl.g[3 * i + a] = __double2float_rn(ga);
                        gsum[a] += ga;
                    }
                }
                for (int a = 0; a < 3; ++a) fl.g[9 + a] = __double2float_rn(-gsum[a]);
                // per component: the cross product (rounded differences, products and
                // difference), the division by the rounded D, and for g_3 the two sums
                const double eg = 3.0 * (rho + 12.0 * kU) * 2.0 * L * L / Dlb * 1.01;
                const double tm = L + m;
                const double e64 = c * tm * tm * tm * 1.01;
                if (eg < 1e30 && e64 < 1e-3) {
                    fl.eg = __double2float_ru(eg);
                    fl.thr = __fsub_rd(__double2float_rd(kEps), __double2float_ru(e64));
                }
            }
        }
    }
    for (int a = 0; a < 3; ++a) {
        blo[a] = __dsub_rd(lo[a], m);
        bhi[a] = __dadd_ru(hi[a], m);
        fl.blo[a] = __double2float_rd(blo[a]);
        fl.bhi[a] = __double2float_ru(bhi[a]);
    }
    if (k_out == kGlobal) {
        // the whole domain: a global tetrahedron has no box check and no screen
        for (int a = 0; a < 3; ++a) {
            fl.blo[a] = __int_as_float(0xff800000);
            fl.bhi[a] = __int_as_float(0x7f800000);
        }
        fl.thr = __int_as_float(0x7fc00000);
    }
    if (k_out == kBinned) {
        int c0[3], c1[3];
        int64_t cnt = 1;
        const double glo[3] = {g.lo[0], g.lo[1], g.lo[2]};
        for (int a = 0; a < 3; ++a) {
            c0[a] = cell_axis(blo[a], glo[a], g.h, g.n[a]);
            c1[a] = cell_axis(bhi[a], glo[a], g.h, g.n[a]);
            cnt *= (c1[a] - c0[a] + 1);
        }
        if (cnt > kMaxCellsPerTet) {
            k_out = kGlobal;
            far[t] = 0;
            for (int a = 0; a < 3; ++a) {
                fl.blo[a] = __int_as_float(0xff800000);
                fl.bhi[a] = __int_as_float(0x7f800000);
            }
            fl.thr = __int_as_float(0x7fc00000);
        } else {
            ncell[t] = static_cast<int>(cnt);
            for (int a = 0; a < 3; ++a) {
                cellbox[6 * t + a] = c0[a];
                cellbox[6 * t + 3 + a] = c1[a];
            }
        }
    }
    kind[t] = k_out;
    rec[t] = r;
    filt[t] = fl;
}

// (cell, tetrahedron) pairs in tetrahedron order, and per-cell counts.
__global__ void __launch_bounds__(kThreads) k_tet_pairs(int64_t nt, const int* __restrict__ ncell,
                                                        const int* __restrict__ cellbox,
                                                        const int64_t* __restrict__ off, Grid g,
                                                        uint32_t* __restrict__ key,
                                                        uint32_t* __restrict__ val,
                                                        int* __restrict__ cellcnt) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= nt || ncell[t] == 0) return;
    int64_t o = off[t];
    const int* b = cellbox + 6 * t;
    for (int x = b[0]; x <= b[3]; ++x)
        for (int y = b[1]; y <= b[4]; ++y)
            for (int z = b[2]; z <= b[5]; ++z) {
                const uint32_t c = static_cast<uint32_t>((static_cast<int64_t>(x) * g.n[1] + y) * g.n[2] + z);
                key[o] = c;
                val[o] = static_cast<uint32_t>(t);
                atomicAdd(&cellcnt[c], 1);
                ++o;
            }
}

__global__ void __launch_bounds__(kThreads) k_flag_of(int64_t n, const int* __restrict__ kind,
                                                      int want, int* __restrict__ flag) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) flag[i] = kind[i] == want ? 1 : 0;
}

__global__ void __launch_bounds__(kThreads) k_compact(int64_t n, const int* __restrict__ flag,
                                                      const int64_t* __restrict__ pos,
                                                      int* __restrict__ out) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n && flag[i]) out[pos[i]] = static_cast<int>(i);
}

// Nodes: cell keys on the node grid (values = node index, for a stable sort).
__global__ void __launch_bounds__(kThreads) k_node_keys(const double* __restrict__ pts, int64_t np,
                                                        Grid g, uint32_t* __restrict__ key,
                                                        uint32_t* __restrict__ val,
                                                        int* __restrict__ cellcnt) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const int x = cell_axis(pts[3 * i], g.lo[0], g.h, g.n[0]);
    const int y = cell_axis(pts[3 * i + 1], g.lo[1], g.h, g.n[1]);
    const int z = cell_axis(pts[3 * i + 2], g.lo[2], g.h, g.n[2]);
    const uint32_t c = static_cast<uint32_t>((static_cast<int64_t>(x) * g.n[1] + y) * g.n[2] + z);
    key[i] = c;
    val[i] = static_cast<uint32_t>(i);
    atomicAdd(&cellcnt[c], 1);
}

// Sorted node coordinates and sizes (nodes of a cell contiguous, ascending index).
__global__ void __launch_bounds__(kThreads) k_node_gather(const double* __restrict__ pts,
                                                          const double* __restrict__ sizes,
                                                          int64_t np, const uint32_t* __restrict__ order,
                                                          Node4* __restrict__ node,
                                                          float4* __restrict__ nodef) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const int64_t v = order[i];
    node[i] = Node4{pts[3 * v], pts[3 * v + 1], pts[3 * v + 2], static_cast<double>(v)};
    nodef[i] = make_float4(__double2float_rn(pts[3 * v]), __double2float_rn(pts[3 * v + 1]),
                           __double2float_rn(pts[3 * v + 2]), 0.0f);
}

// ------------------------------------------------------------ evaluation

struct Field {
    int64_t np, nt, nglobal;
    double scale;
    double3 dlo, dhi;  // fast-path domain
    Grid tg, ng;       // tetrahedron grid over the domain, node grid over the nodes' box
    const TetRec* rec;
    const TetFilt* filt;
    const int* kind;
    const int64_t* tcell_off;  // tg cells + 1
    const uint32_t* tcell_tet;
    const int* global;
    int64_t nfar;
    const int* farlist;        // binned tetrahedra also tested by queries beyond their far box
    const double* farbox;      // per tetrahedron: lo[3], hi[3] of the box inflated by rfar
    const int64_t* ncell_off;  // ng cells + 1
    const Node4* node;       // sorted nodes: x, y, z, original index
    const float4* nodef;     // the same nodes rounded to FP32 (pruning only)
    GridF ngf;               // the node grid in FP32, rounded outward
    const double* pts;         // nodes in their own order (the scan of the slow path)
    const double* sizes;       // padded to np
};

struct EvalCounters {
    unsigned long long inside, nearest, slow, tests, boxed;
};

// Rounded squared distance as the reference computes it (dx = node - query).
__device__ __forceinline__ double dist2(const Node4& n, const P3& p) {
    const double dx = n.x - p.x, dy = n.y - p.y, dz = n.z - p.z;
    return dx * dx + dy * dy + dz * dz;
}

// Nearest node by rings of cells around p's (clamped) cell; stops once every unvisited
// node's rounded squared distance provably exceeds the best found. Cells and nodes are
// pruned in FP32 with outward rounding before any node pays the reference's FP64
// squared distance: skipped only when even their lower bound exceeds the best.
__device__ int64_t nearest_node(const Field& F, const P3& p, const Q32& q) {
    const Grid& g = F.ng;
    const GridF& gf = F.ngf;
    const double pc[3] = {p.x, p.y, p.z};
    int c[3];
    float tolf[3];
    for (int a = 0; a < 3; ++a) {
        c[a] = cell_axis(pc[a], g.lo[a], g.h, g.n[a]);
        // a node's cell comes from a rounded quotient: it may lie this far beyond its faces
        tolf[a] = __fmaf_ru(fabsf(q.ph[a]), 3.6e-15f, gf.tol[a]);
    }
    double best = DBL_MAX;
    float best_f = __int_as_float(0x7f800000);
    int64_t bi = -1;
    const int kmax = max(g.n[0], max(g.n[1], g.n[2]));
    for (int k = 0; k <= kmax; ++k) {
        for (int x = c[0] - k; x <= c[0] + k; ++x) {
            if (x < 0 || x >= g.n[0]) continue;
            const bool xs = (x == c[0] - k || x == c[0] + k);
            for (int y = c[1] - k; y <= c[1] + k; ++y) {
                if (y < 0 || y >= g.n[1]) continue;
                const bool ys = xs || (y == c[1] - k || y == c[1] + k);
                for (int z = c[2] - k; z <= c[2] + k; ++z) {
                    if (z < 0 || z >= g.n[2]) continue;
                    if (!ys && z != c[2] - k && z != c[2] + k) {
                        z = c[2] + k - 1;  // interior of the shell: jump to its far face
                        continue;
                    }
                    const int cx[3] = {x, y, z};
                    float lb = 0.0f;
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const float clo = __fsub_rd(__fmaf_rd(static_cast<float>(cx[a]), gf.h_rd, gf.lo_rd[a]), tolf[a]);
                        const float chi = __fadd_ru(__fmaf_ru(static_cast<float>(cx[a] + 1), gf.h_ru, gf.lo_ru[a]), tolf[a]);
                        const float d = fmaxf(0.0f, fmaxf(__fsub_rd(clo, q.hi[a]), __fsub_rd(q.lo[a], chi)));
                        lb = __fmaf_rd(d, d, lb);
                    }
                    if (__fmul_rd(lb, 0.999999f) > best_f) continue;
                    const int64_t cell = (static_cast<int64_t>(x) * g.n[1] + y) * g.n[2] + z;
                    for (int64_t j = F.ncell_off[cell]; j < F.ncell_off[cell + 1]; ++j) {
                        const float4 nf = F.nodef[j];
                        const float nfa[3] = {nf.x, nf.y, nf.z};
                        float lbn = 0.0f;
#pragma unroll
                        for (int a = 0; a < 3; ++a) {
                            const float dd = fabsf(nfa[a] - q.ph[a]);
                            const float e = __fmul_ru(__fadd_ru(fabsf(nfa[a]), fabsf(q.ph[a])), 1.2e-7f);
                            const float d = fmaxf(0.0f, __fsub_rd(__fmul_rd(dd, 0.99999988f), e));
                            lbn = __fmaf_rd(d, d, lbn);
                        }
                        if (__fmul_rd(lbn, 0.999999f) > best_f) continue;
                        const Node4 nd = F.node[j];
                        const double d = dist2(nd, p);
                        const int64_t id = static_cast<int64_t>(nd.w);
                        if (d < best || (d == best && id < bi)) {
                            best = d;
                            bi = id;
                            best_f = __double2float_ru(best);
                        }
                    }
                }
            }
        }
        // distance from p to the cells not yet visited (sides on the grid's edge bound
        // nothing); a node's cell comes from a rounded quotient, so it may lie up to tol
        // beyond its cell's face
        double R = DBL_MAX;
        bool all = true;
        for (int a = 0; a < 3; ++a) {
            const double tol = 16.0 * kU * (fabs(g.lo[a]) + (g.n[a] + 1.0) * g.h + fabs(pc[a]));
            if (c[a] - k > 0) {
                all = false;
                const double face = __dadd_ru(g.lo[a], __dmul_ru(static_cast<double>(c[a] - k), g.h));
                R = fmin(R, __dsub_rd(__dsub_rd(pc[a], face), tol));
            }
            if (c[a] + k + 1 < g.n[a]) {
                all = false;
                const double face = __dadd_rd(g.lo[a], __dmul_rd(static_cast<double>(c[a] + k + 1), g.h));
                R = fmin(R, __dsub_rd(__dsub_rd(face, pc[a]), tol));
            }
        }
        if (all) break;
        if (R > 0.0 && bi >= 0) {
            const double lb = __dmul_rd(__dmul_rd(R, R), 1.0 - 1e-14);
            if (best < lb) break;
        }
    }
    return bi < 0 ? 0 : bi;
}

__device__ __forceinline__ void warp_count(unsigned v, unsigned long long* dst) {
    const unsigned t = __reduce_add_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0 && t) atomicAdd(dst, static_cast<unsigned long long>(t));
}

// Sort keys of the queries: the cell of the tetrahedron grid (the evaluation then runs
// in cell order: neighbouring threads share candidates and take the same branch), or
// the cell count for the queries the reference's scan answers (sorted last).
__global__ void __launch_bounds__(kThreads) k_query_keys(Field F, const double* __restrict__ q,
                                                         int64_t n, uint32_t* __restrict__ key,
                                                         uint32_t* __restrict__ val,
                                                         int* __restrict__ nslow) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const P3 p{q[3 * i], q[3 * i + 1], q[3 * i + 2]};
    const bool fin = isfinite(p.x) && isfinite(p.y) && isfinite(p.z);
    const Grid& g = F.tg;
    uint32_t k;
    if (!fin || p.x < F.dlo.x || p.x > F.dhi.x || p.y < F.dlo.y || p.y > F.dhi.y || p.z < F.dlo.z ||
        p.z > F.dhi.z) {
        k = static_cast<uint32_t>(static_cast<int64_t>(g.n[0]) * g.n[1] * g.n[2]);
        atomicAdd(nslow, 1);
    } else {
        k = static_cast<uint32_t>((static_cast<int64_t>(cell_axis(p.x, g.lo[0], g.h, g.n[0])) * g.n[1] +
                                   cell_axis(p.y, g.lo[1], g.h, g.n[1])) * g.n[2] +
                                  cell_axis(p.z, g.lo[2], g.h, g.n[2]));
    }
    key[i] = k;
    val[i] = static_cast<uint32_t>(i);
}

__global__ void __launch_bounds__(kThreads) k_sizing_eval(Field F, const double* __restrict__ q,
                                                          const uint32_t* __restrict__ skey,
                                                          const uint32_t* __restrict__ order,
                                                          int64_t n, double* __restrict__ out,
                                                          int* __restrict__ which,
                                                          EvalCounters* __restrict__ ctr) {
    const int64_t pos = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    unsigned inside = 0, nearest = 0, tests = 0, boxed = 0;
    const int64_t ncells = static_cast<int64_t>(F.tg.n[0]) * F.tg.n[1] * F.tg.n[2];
    if (pos < n && static_cast<int64_t>(skey[pos]) < ncells) {
        const int64_t i = order[pos];
        const P3 p{q[3 * i], q[3 * i + 1], q[3 * i + 2]};
        {
            const int64_t cell = skey[pos];
            int64_t ia = F.tcell_off[cell];
            const int64_t ea = F.tcell_off[cell + 1];
            int64_t ib = 0, ic = 0;
            const int64_t eb = F.nglobal, ec = F.nfar;
            // next far-list entry this query must test (it lies beyond the far box)
            auto next_far = [&]() -> int64_t {
                for (; ic < ec; ++ic) {
                    const int64_t t = F.farlist[ic];
                    const double* fb = F.farbox + 6 * t;
                    if (p.x < fb[0] || p.x > fb[3] || p.y < fb[1] || p.y > fb[4] || p.z < fb[2] ||
                        p.z > fb[5])
                        return t;
                }
                return INT64_MAX;
            };
            int64_t tc = next_far();
            const Q32 q32 = make_q32(p);
            // candidates of the cell, the global list and the far list, merged ascending:
            // the first that passes is the reference's answer. Each lane screens ahead to
            // its next surviving candidate; the full tests then run with the warp
            // reconverged (the six tetrahedra of one cell of a structured mesh share a
            // box, so testing in the screening loop would run them one lane group at a time)
            for (;;) {
                int64_t t = -1;
                while (ia < ea || ib < eb || tc != INT64_MAX) {
                    const int64_t ta = ia < ea ? static_cast<int64_t>(F.tcell_tet[ia]) : INT64_MAX;
                    const int64_t tb = ib < eb ? static_cast<int64_t>(F.global[ib]) : INT64_MAX;
                    int64_t t0;
                    bool far_hit = false;
                    if (ta <= tb && ta <= tc) {
                        t0 = ta;
                        ++ia;
                    } else if (tb <= tc) {
                        t0 = tb;
                        ++ib;
                    } else {
                        t0 = tc;
                        ++ic;
                        tc = next_far();
                        far_hit = true;  // beyond the far box: no box or screen applies
                    }
                    ++boxed;
                    if (!far_hit) {
                        const TetFilt& fc = F.filt[t0];
                        if (outside_box(fc, q32) || screened_out(fc, q32)) continue;
                    }
                    t = t0;
                    break;
                }
                if (t < 0) break;
                ++tests;
                double sz;
                if (interp(F.rec[t], p, sz)) {
                    out[i] = sz * F.scale;
                    if (which) which[i] = static_cast<int>(t);
                    inside = 1;
                    break;
                }
            }
            if (!inside) {
                const int64_t bi = F.np > 0 ? nearest_node(F, p, q32) : 0;
                out[i] = (F.np > 0 ? F.sizes[bi] : 0.0) * F.scale;
                if (which) which[i] = -1;
                nearest = 1;
            }
        }
    }
    warp_count(inside, &ctr->inside);
    warp_count(nearest, &ctr->nearest);
    warp_count(tests, &ctr->tests);
    warp_count(boxed, &ctr->boxed);
}

// The reference's own scan for queries outside the domain or not finite: one warp per
// query, 32 tetrahedra at a time in order (the first passing one answers), then the
// nearest node by a warp-wide (distance, index) minimum with the reference's rules.
__global__ void __launch_bounds__(kThreads) k_sizing_slow(Field F, const double* __restrict__ q,
                                                          const uint32_t* __restrict__ order,
                                                          int64_t n, const int* __restrict__ nslow,
                                                          double* __restrict__ out,
                                                          int* __restrict__ which,
                                                          EvalCounters* __restrict__ ctr) {
    const int lane = threadIdx.x & 31;
    const int64_t w = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    const int ns = *nslow;
    for (int64_t s = w; s < ns; s += nw) {
        const int64_t i = order[n - ns + s];
        const P3 p{q[3 * i], q[3 * i + 1], q[3 * i + 2]};
        int64_t found = -1;
        double val = 0.0;
        for (int64_t base = 0; base < F.nt && found < 0; base += 32) {
            const int64_t t = base + lane;
            bool pass = false;
            double v = 0.0;
            if (t < F.nt && F.kind[t] != kNever) pass = interp(F.rec[t], p, v);
            const unsigned m = __ballot_sync(0xffffffffu, pass);
            if (m) {
                const int src = __ffs(m) - 1;
                val = __shfl_sync(0xffffffffu, v, src);
                found = base + src;
            }
        }
        if (found >= 0) {
            if (lane == 0) {
                out[i] = val * F.scale;
                if (which) which[i] = static_cast<int>(found);
                atomicAdd(&ctr->inside, 1ull);
            }
            continue;
        }
        // nearest: smallest d < DBL_MAX (NaN never), first index; none -> node 0
        double best = DBL_MAX;
        int64_t bi = INT64_MAX;
        for (int64_t j = lane; j < F.np; j += 32) {
            const Node4 nd = Node4{F.pts[3 * j], F.pts[3 * j + 1], F.pts[3 * j + 2], 0.0};
            const double d = dist2(nd, p);
            if (d < best) {
                best = d;
                bi = j;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int64_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob < best || (ob == best && oi < bi)) {
                best = ob;
                bi = oi;
            }
        }
        if (lane == 0) {
            const int64_t k = bi == INT64_MAX ? 0 : bi;
            out[i] = (F.np > 0 ? F.sizes[k] : 0.0) * F.scale;
            if (which) which[i] = -1;
            atomicAdd(&ctr->nearest, 1ull);
        }
    }
    if (threadIdx.x == 0 && blockIdx.x == 0) atomicAdd(&ctr->slow, static_cast<unsigned long long>(ns));
}

// robust::orient3d_batch: the orient3d value of every candidate tetrahedron.
__global__ void __launch_bounds__(kThreads) k_o3_batch(const double* __restrict__ pts,
                                                       const int4* __restrict__ tets, int64_t n,
                                                       double* __restrict__ out) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int4 q = tets[t];
    auto P = [&](int i) {
        const int64_t k = 3 * static_cast<int64_t>(i);
        return P3{pts[k], pts[k + 1], pts[k + 2]};
    };
    out[t] = o3_value(P(q.x), P(q.y), P(q.z), P(q.w));
}

unsigned blocks(int64_t n) { return static_cast<unsigned>((n + kThreads - 1) / kThreads); }

Grid make_grid(const double lo[3], const double hi[3], double target_cells, int64_t max_cells) {
    Grid g{};
    double ext[3], V = 1.0, emax = 0.0;
    for (int a = 0; a < 3; ++a) {
        ext[a] = hi[a] - lo[a];
        emax = std::max(emax, ext[a]);
    }
    if (!(emax > 0.0)) emax = 1.0;
    for (int a = 0; a < 3; ++a) V *= std::max(ext[a], emax * 1e-3);
    double h = std::cbrt(V / std::max(1.0, target_cells));
    h = std::max(h, emax / 4096.0);
    for (;;) {
        int64_t total = 1;
        for (int a = 0; a < 3; ++a) {
            g.n[a] = std::max(1, static_cast<int>(std::ceil(ext[a] / h)));
            total *= g.n[a];
        }
        if (total <= max_cells) break;
        h *= 1.25;
    }
    for (int a = 0; a < 3; ++a) g.lo[a] = lo[a];
    g.h = h;
    return g;
}

float down(double x) {
    float f = static_cast<float>(x);
    return static_cast<double>(f) > x ? std::nextafter(f, -INFINITY) : f;
}
float up(double x) {
    float f = static_cast<float>(x);
    return static_cast<double>(f) < x ? std::nextafter(f, INFINITY) : f;
}

GridF grid_f(const Grid& g) {
    GridF f{};
    for (int a = 0; a < 3; ++a) {
        f.lo_rd[a] = down(g.lo[a]);
        f.lo_ru[a] = up(g.lo[a]);
        f.tol[a] = up(16.0 * kU * (std::fabs(g.lo[a]) + (g.n[a] + 1.0) * g.h) * 1.01);
    }
    f.h_rd = down(g.h);
    f.h_ru = up(g.h);
    return f;
}

}  // namespace

struct SizingField {
    Field f{};
    std::vector<void*> owned;
    EvalCounters* ctr = nullptr;
    uint32_t* skey = nullptr;   // per evaluation: sort keys (cells), query order, sort space
    uint32_t* order = nullptr;
    char* sort_tmp = nullptr;
    int* nslow = nullptr;
    int64_t slow_cap = 0;
    double* dq = nullptr;
    double* dout = nullptr;
    int* dwhich = nullptr;
    int64_t io_cap = 0;
    SizingStats last{};
    float last_ms[3] = {0.f, 0.f, 0.f};
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    std::mutex mu;

    template <typename T>
    T* alloc(size_t n) {
        void* p = nullptr;
        CMG_CUDA(device_alloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
        owned.push_back(p);
        return static_cast<T*>(p);
    }
    ~SizingField() {
        for (void* p : owned) cudaFree(p);
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
    }
};

SizingField* sizing_create(const double* pts, int64_t np, const int* tets, int64_t nt,
                           const double* sizes, int64_t ns, double scale, cudaStream_t st) {
    if (np < 0 || nt < 0 || ns < 0) throw std::invalid_argument("sizing: negative count");
    if (np >= (int64_t(1) << 31) || nt >= (int64_t(1) << 31))
        throw std::invalid_argument("sizing: too many nodes or tetrahedra");
    for (int64_t i = 0; i < 3 * np; ++i)
        if (!std::isfinite(pts[i])) throw std::invalid_argument("sizing: non-finite background point");
    for (int64_t k = 0; k < 4 * nt; ++k)
        if (tets[k] < 0 || tets[k] >= np)
            throw std::invalid_argument("sizing: tetrahedron vertex index out of range");
    std::unique_ptr<SizingField> S(new SizingField);
    Field& F = S->f;
    F.np = np;
    F.nt = nt;
    F.scale = scale;
    // node box, domain = box grown by half its largest extent
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    if (np > 0) {
        for (int a = 0; a < 3; ++a) lo[a] = hi[a] = pts[a];
        for (int64_t i = 1; i < np; ++i)
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], pts[3 * i + a]);
                hi[a] = std::max(hi[a], pts[3 * i + a]);
            }
    }
    double ext = 0.0;
    for (int a = 0; a < 3; ++a) ext = std::max(ext, hi[a] - lo[a]);
    const double grow = ext > 0.0 ? 0.5 * ext : 1.0;
    double dlo[3], dhi[3];
    for (int a = 0; a < 3; ++a) {
        dlo[a] = lo[a] - grow;
        dhi[a] = hi[a] + grow;
    }
    F.dlo = make_double3(dlo[0], dlo[1], dlo[2]);
    F.dhi = make_double3(dhi[0], dhi[1], dhi[2]);
    F.tg = make_grid(dlo, dhi, std::max<double>(1.0, static_cast<double>(nt)) * 1.0, int64_t(1) << 24);
    F.ng = make_grid(lo, hi, std::max<double>(1.0, 0.5 * static_cast<double>(np)), int64_t(1) << 22);

    // device copies; sizes padded with 0 / truncated to the node count
    std::vector<double> hs(static_cast<size_t>(np), 0.0);
    for (int64_t i = 0; i < std::min(np, ns); ++i) hs[i] = sizes[i];
    double* dp = S->alloc<double>(3 * np);
    int4* dt = S->alloc<int4>(nt);
    double* dsz = S->alloc<double>(np);
    if (np) CMG_CUDA(cudaMemcpyAsync(dp, pts, sizeof(double) * 3 * np, cudaMemcpyHostToDevice, st));
    if (nt) CMG_CUDA(cudaMemcpyAsync(dt, tets, sizeof(int4) * nt, cudaMemcpyHostToDevice, st));
    if (np) CMG_CUDA(cudaMemcpyAsync(dsz, hs.data(), sizeof(double) * np, cudaMemcpyHostToDevice, st));
    F.sizes = dsz;
    F.pts = dp;

    TetRec* rec = S->alloc<TetRec>(nt);
    TetFilt* filt = S->alloc<TetFilt>(nt);
    int* farflag = S->alloc<int>(nt);
    double* farbox = S->alloc<double>(6 * nt);
    int* kind = S->alloc<int>(nt);
    int* ncell = S->alloc<int>(nt);
    int* cellbox = S->alloc<int>(6 * nt);
    const int64_t tcells = int64_t(F.tg.n[0]) * F.tg.n[1] * F.tg.n[2];
    int* tcnt = S->alloc<int>(tcells);
    int64_t* toff = S->alloc<int64_t>(tcells + 1);
    CMG_CUDA(cudaMemsetAsync(tcnt, 0, sizeof(int) * tcells, st));
    int64_t npairs = 0, nglobal = 0;
    std::vector<void*> tmp;
    auto talloc = [&](size_t bytes) {
        void* p = nullptr;
        CMG_CUDA(device_alloc(&p, std::max<size_t>(bytes, 16)));
        tmp.push_back(p);
        return p;
    };
    struct Free {
        std::vector<void*>& v;
        ~Free() {
            for (void* p : v) cudaFree(p);
        }
    } free_tmp{tmp};
    uint32_t* tkey = nullptr;
    if (nt > 0) {
        k_tet_prep<<<blocks(nt), kThreads, 0, st>>>(dp, dt, nt, dsz, F.tg, F.dlo, F.dhi, rec, filt,
                                                    farflag, farbox, kind, ncell, cellbox);
        CMG_LAUNCH();
        int64_t* poff = static_cast<int64_t*>(talloc(sizeof(int64_t) * (nt + 1)));
        int64_t* stmp = static_cast<int64_t*>(talloc(sizeof(int64_t) * scan_tmp_elems(std::max(nt, tcells))));
        exclusive_scan(ncell, poff, nt, stmp, st);
        CMG_CUDA(cudaMemcpyAsync(&npairs, poff + nt, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        CMG_CUDA(cudaStreamSynchronize(st));
        if (npairs >= (int64_t(1) << 31)) throw std::runtime_error("sizing: too many cell entries");
        tkey = static_cast<uint32_t*>(talloc(sizeof(uint32_t) * npairs));
        uint32_t* tval = S->alloc<uint32_t>(npairs);
        k_tet_pairs<<<blocks(nt), kThreads, 0, st>>>(nt, ncell, cellbox, poff, F.tg, tkey, tval, tcnt);
        CMG_LAUNCH();
        int bits = 1;
        while ((int64_t(1) << bits) < tcells) ++bits;
        void* stmp2 = talloc(radix_sort_tmp_bytes(npairs));
        radix_sort_pairs(tkey, tval, npairs, bits, stmp2, st);
        exclusive_scan(tcnt, toff, tcells, stmp, st);
        F.tcell_tet = tval;
        // global list, ascending
        int* flag = static_cast<int*>(talloc(sizeof(int) * nt));
        int64_t* gpos = static_cast<int64_t*>(talloc(sizeof(int64_t) * (nt + 1)));
        k_flag_of<<<blocks(nt), kThreads, 0, st>>>(nt, kind, kGlobal, flag);
        CMG_LAUNCH();
        exclusive_scan(flag, gpos, nt, stmp, st);
        CMG_CUDA(cudaMemcpyAsync(&nglobal, gpos + nt, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        CMG_CUDA(cudaStreamSynchronize(st));
        int* glist = S->alloc<int>(nglobal);
        k_compact<<<blocks(nt), kThreads, 0, st>>>(nt, flag, gpos, glist);
        CMG_LAUNCH();
        F.global = glist;
        // far list, ascending
        int64_t nfar = 0;
        int64_t* fpos = static_cast<int64_t*>(talloc(sizeof(int64_t) * (nt + 1)));
        exclusive_scan(farflag, fpos, nt, stmp, st);
        CMG_CUDA(cudaMemcpyAsync(&nfar, fpos + nt, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        CMG_CUDA(cudaStreamSynchronize(st));
        int* flist = S->alloc<int>(nfar);
        k_compact<<<blocks(nt), kThreads, 0, st>>>(nt, farflag, fpos, flist);
        CMG_LAUNCH();
        F.farlist = flist;
        F.nfar = nfar;
        F.farbox = farbox;
    } else {
        int64_t* stmp = static_cast<int64_t*>(talloc(sizeof(int64_t) * scan_tmp_elems(tcells)));
        exclusive_scan(tcnt, toff, tcells, stmp, st);
        F.tcell_tet = S->alloc<uint32_t>(1);
        F.global = S->alloc<int>(1);
        F.farlist = S->alloc<int>(1);
        F.farbox = farbox;
        F.nfar = 0;
    }
    F.nglobal = nglobal;
    F.rec = rec;
    F.filt = filt;
    F.kind = kind;
    F.tcell_off = toff;

    // nodes by cell of the node grid
    const int64_t ncells = int64_t(F.ng.n[0]) * F.ng.n[1] * F.ng.n[2];
    int* ncnt = static_cast<int*>(talloc(sizeof(int) * ncells));
    int64_t* noff = S->alloc<int64_t>(ncells + 1);
    Node4* node = S->alloc<Node4>(np);
    float4* nodef = S->alloc<float4>(np);
    CMG_CUDA(cudaMemsetAsync(ncnt, 0, sizeof(int) * ncells, st));
    int64_t* stmp = static_cast<int64_t*>(talloc(sizeof(int64_t) * scan_tmp_elems(ncells)));
    if (np > 0) {
        uint32_t* nkey = static_cast<uint32_t*>(talloc(sizeof(uint32_t) * np));
        uint32_t* nval = static_cast<uint32_t*>(talloc(sizeof(uint32_t) * np));
        k_node_keys<<<blocks(np), kThreads, 0, st>>>(dp, np, F.ng, nkey, nval, ncnt);
        CMG_LAUNCH();
        int bits = 1;
        while ((int64_t(1) << bits) < ncells) ++bits;
        void* stmp2 = talloc(radix_sort_tmp_bytes(np));
        radix_sort_pairs(nkey, nval, np, bits, stmp2, st);
        k_node_gather<<<blocks(np), kThreads, 0, st>>>(dp, dsz, np, nval, node, nodef);
        CMG_LAUNCH();
    }
    exclusive_scan(ncnt, noff, ncells, stmp, st);
    F.ncell_off = noff;
    F.node = node;
    F.nodef = nodef;
    F.ngf = grid_f(F.ng);
    S->ctr = S->alloc<EvalCounters>(1);
    CMG_CUDA(cudaStreamSynchronize(st));  // the temporaries are freed on return
    S->last.binned_pairs = npairs;
    S->last.global_tets = nglobal;
    S->last.far_tets = F.nfar;
    return S.release();
}

void sizing_destroy(SizingField* f) { delete f; }

void orient3d_batch(const double* pts, int64_t np, const int* tets, int64_t n, double* out,
                    cudaStream_t st) {
    static std::mutex mu;
    static Arena arena;
    std::lock_guard<std::mutex> lk(mu);
    double *dp, *dv;
    int4* dt;
    auto plan = [&]() {
        arena.reset();
        dp = arena.take<double>(3 * np);
        dt = arena.take<int4>(n);
        dv = arena.take<double>(n);
    };
    arena.clear_need();
    plan();
    if (arena.overflowed()) {
        arena.reserve(arena.need());
        plan();
    }
    CMG_CUDA(cudaMemcpyAsync(dp, pts, sizeof(double) * 3 * np, cudaMemcpyHostToDevice, st));
    CMG_CUDA(cudaMemcpyAsync(dt, tets, sizeof(int4) * n, cudaMemcpyHostToDevice, st));
    k_o3_batch<<<blocks(n), kThreads, 0, st>>>(dp, dt, n, dv);
    CMG_LAUNCH();
    CMG_CUDA(cudaMemcpyAsync(out, dv, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    CMG_CUDA(cudaStreamSynchronize(st));
}

void sizing_eval_device(SizingField* S, const double* q, int64_t n, double* out, int* which,
                        cudaStream_t st) {
    std::lock_guard<std::mutex> lk(S->mu);
    if (n <= 0) return;
    if (n >= (int64_t(1) << 31)) throw std::invalid_argument("sizing: too many queries in one call");
    if (n > S->slow_cap) {
        const int64_t cap = std::max<int64_t>(n, 2 * S->slow_cap);
        S->skey = S->alloc<uint32_t>(cap);
        S->order = S->alloc<uint32_t>(cap);
        S->sort_tmp = S->alloc<char>(radix_sort_tmp_bytes(cap));
        S->slow_cap = cap;
    }
    if (!S->nslow) S->nslow = S->alloc<int>(1);
    CMG_CUDA(cudaMemsetAsync(S->nslow, 0, sizeof(int), st));
    CMG_CUDA(cudaMemsetAsync(S->ctr, 0, sizeof(EvalCounters), st));
    k_query_keys<<<blocks(n), kThreads, 0, st>>>(S->f, q, n, S->skey, S->order, S->nslow);
    CMG_LAUNCH();
    const int64_t tcells = int64_t(S->f.tg.n[0]) * S->f.tg.n[1] * S->f.tg.n[2];
    int bits = 1;
    while ((int64_t(1) << bits) <= tcells) ++bits;
    radix_sort_pairs(S->skey, S->order, n, bits, S->sort_tmp, st);
    k_sizing_eval<<<blocks(n), kThreads, 0, st>>>(S->f, q, S->skey, S->order, n, out, which, S->ctr);
    CMG_LAUNCH();
    // the slow queries are the tail of the sorted order
    k_sizing_slow<<<152 * 4, kThreads, 0, st>>>(S->f, q, S->order, n, S->nslow, out, which, S->ctr);
    CMG_LAUNCH();
}

void sizing_eval_host(SizingField* S, const double* q, int64_t n, double* out, int* which,
                      cudaStream_t st) {
    if (n <= 0) return;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (n > S->io_cap) {
            const int64_t cap = std::max<int64_t>(n, 2 * S->io_cap);
            S->dq = S->alloc<double>(3 * cap);
            S->dout = S->alloc<double>(cap);
            S->dwhich = S->alloc<int>(cap);
            S->io_cap = cap;
        }
        if (!S->ev[0])
            for (cudaEvent_t& e : S->ev) CMG_CUDA(cudaEventCreate(&e));
        CMG_CUDA(cudaEventRecord(S->ev[0], st));
        CMG_CUDA(cudaMemcpyAsync(S->dq, q, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
        CMG_CUDA(cudaEventRecord(S->ev[1], st));
    }
    sizing_eval_device(S, S->dq, n, S->dout, which ? S->dwhich : nullptr, st);
    std::lock_guard<std::mutex> lk(S->mu);
    CMG_CUDA(cudaEventRecord(S->ev[2], st));
    CMG_CUDA(cudaMemcpyAsync(out, S->dout, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    if (which) CMG_CUDA(cudaMemcpyAsync(which, S->dwhich, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
    CMG_CUDA(cudaEventRecord(S->ev[3], st));
    CMG_CUDA(cudaStreamSynchronize(st));
    for (int k = 0; k < 3; ++k) CMG_CUDA(cudaEventElapsedTime(&S->last_ms[k], S->ev[k], S->ev[k + 1]));
}

SizingStats sizing_stats(SizingField* S, cudaStream_t st) {
    std::lock_guard<std::mutex> lk(S->mu);
    EvalCounters c{};
    CMG_CUDA(cudaMemcpyAsync(&c, S->ctr, sizeof(c), cudaMemcpyDeviceToHost, st));
    CMG_CUDA(cudaStreamSynchronize(st));
    SizingStats r = S->last;
    r.inside = static_cast<int64_t>(c.inside);
    r.nearest = static_cast<int64_t>(c.nearest);
    r.slow = static_cast<int64_t>(c.slow);
    r.tests = static_cast<int64_t>(c.tests);
    r.candidates = static_cast<int64_t>(c.boxed);
    r.upload_ms = S->last_ms[0];
    r.eval_ms = S->last_ms[1];
    r.download_ms = S->last_ms[2];
    return r;
}

}  // namespace cmg::gpu
