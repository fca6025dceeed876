// cmg_exact.cuh — exact signs of orient3d and insphere on the device.
//
// Expansion arithmetic after J. R. Shewchuk, "Adaptive Precision Floating-Point
// Arithmetic and Fast Robust Geometric Predicates" (CMU-CS-96-140): a number is a
// sum of non-overlapping doubles sorted by magnitude; Two-Sum and Two-Product are
// error-free (Two-Product here uses the fused multiply-add residual a*b - fl(a*b),
// which is exact), sums merge by magnitude, and the sign of an expansion is the
// sign of its largest component. Inputs must stay clear of overflow and underflow,
// as for the reference's predicates.
//
// These routines run only in the compacted second passes (columns or queries the
// FP64 filter could not decide), one thread per case, so their local arrays never
// load the main kernels.
#pragma once

#include "cmg_device.cuh"

namespace cmg::gpu::exact {

__device__ __forceinline__ void two_sum(double a, double b, double& x, double& y) {
    x = __dadd_rn(a, b);
    double bv = __dsub_rn(x, a);
    double av = __dsub_rn(x, bv);
    y = __dadd_rn(__dsub_rn(a, av), __dsub_rn(b, bv));
}
__device__ __forceinline__ void fast_two_sum(double a, double b, double& x, double& y) {
    x = __dadd_rn(a, b);
    y = __dsub_rn(b, __dsub_rn(x, a));
}
__device__ __forceinline__ void two_prod(double a, double b, double& x, double& y) {
    x = __dmul_rn(a, b);
    y = __fma_rn(a, b, -x);
}
__device__ __forceinline__ void two_diff(double a, double b, double& x, double& y) {
    two_sum(a, -b, x, y);
}

// ---- exactness certificates
// An FP64 evaluation whose every operation was exact gives the exact determinant.
// Each step checks its own rounding: a subtraction or sum through its Two-Sum tail,
// a product through its FMA residual (a nonzero product below 2^-960, or one that
// underflowed to zero, is not trusted: its residual may not be representable).
// Overflow produces a non-finite tail and fails the check.
__device__ __forceinline__ double xsub(double a, double b, bool& ok) {
    double x, y;
    two_diff(a, b, x, y);
    ok = ok && y == 0.0;
    return x;
}
__device__ __forceinline__ double xadd(double a, double b, bool& ok) {
    double x, y;
    two_sum(a, b, x, y);
    ok = ok && y == 0.0;
    return x;
}
__device__ __forceinline__ double xmul(double a, double b, bool& ok) {
    const double p = __dmul_rn(a, b);
    const bool tiny = p != 0.0 ? fabs(p) < 0x1p-960 : (a != 0.0 && b != 0.0);
    ok = ok && !tiny && __fma_rn(a, b, -p) == 0.0;
    return p;
}

// orient3d(a, b, c, d) evaluated with exactness tracking; true when *det is exact.
static __device__ __noinline__ bool orient3d_certified(const d3& a, const d3& b, const d3& c,
                                                       const d3& d, double* det) {
    bool ok = true;
    const double adx = xsub(a.x, d.x, ok), ady = xsub(a.y, d.y, ok), adz = xsub(a.z, d.z, ok);
    const double bdx = xsub(b.x, d.x, ok), bdy = xsub(b.y, d.y, ok), bdz = xsub(b.z, d.z, ok);
    const double cdx = xsub(c.x, d.x, ok), cdy = xsub(c.y, d.y, ok), cdz = xsub(c.z, d.z, ok);
    const double m1 = xsub(xmul(bdx, cdy, ok), xmul(cdx, bdy, ok), ok);
    const double m2 = xsub(xmul(cdx, ady, ok), xmul(adx, cdy, ok), ok);
    const double m3 = xsub(xmul(adx, bdy, ok), xmul(bdx, ady, ok), ok);
    *det = xadd(xadd(xmul(adz, m1, ok), xmul(bdz, m2, ok), ok), xmul(cdz, m3, ok), ok);
    return ok;
}

// insphere(a, b, c, d, e) (the lifted 4x4 form, e as origin) with exactness
// tracking; true when *det is exact.
static __device__ __noinline__ bool insphere_certified(const d3& a, const d3& b, const d3& c,
                                                       const d3& d, const d3& e, double* det) {
    bool ok = true;
    const double aex = xsub(a.x, e.x, ok), aey = xsub(a.y, e.y, ok), aez = xsub(a.z, e.z, ok);
    const double bex = xsub(b.x, e.x, ok), bey = xsub(b.y, e.y, ok), bez = xsub(b.z, e.z, ok);
    const double cex = xsub(c.x, e.x, ok), cey = xsub(c.y, e.y, ok), cez = xsub(c.z, e.z, ok);
    const double dex = xsub(d.x, e.x, ok), dey = xsub(d.y, e.y, ok), dez = xsub(d.z, e.z, ok);
    if (!ok) return false;
    const double ab = xsub(xmul(aex, bey, ok), xmul(bex, aey, ok), ok);
    const double bc = xsub(xmul(bex, cey, ok), xmul(cex, bey, ok), ok);
    const double cd = xsub(xmul(cex, dey, ok), xmul(dex, cey, ok), ok);
    const double da = xsub(xmul(dex, aey, ok), xmul(aex, dey, ok), ok);
    const double ac = xsub(xmul(aex, cey, ok), xmul(cex, aey, ok), ok);
    const double bd = xsub(xmul(bex, dey, ok), xmul(dex, bey, ok), ok);
    const double abc = xadd(xsub(xmul(aez, bc, ok), xmul(bez, ac, ok), ok), xmul(cez, ab, ok), ok);
    const double bcd = xadd(xsub(xmul(bez, cd, ok), xmul(cez, bd, ok), ok), xmul(dez, bc, ok), ok);
    const double cda = xadd(xadd(xmul(cez, da, ok), xmul(dez, ac, ok), ok), xmul(aez, cd, ok), ok);
    const double dab = xadd(xadd(xmul(dez, ab, ok), xmul(aez, bd, ok), ok), xmul(bez, da, ok), ok);
    const double al = xadd(xadd(xmul(aex, aex, ok), xmul(aey, aey, ok), ok), xmul(aez, aez, ok), ok);
    const double bl = xadd(xadd(xmul(bex, bex, ok), xmul(bey, bey, ok), ok), xmul(bez, bez, ok), ok);
    const double cl = xadd(xadd(xmul(cex, cex, ok), xmul(cey, cey, ok), ok), xmul(cez, cez, ok), ok);
    const double dl = xadd(xadd(xmul(dex, dex, ok), xmul(dey, dey, ok), ok), xmul(dez, dez, ok), ok);
    *det = xadd(xsub(xmul(dl, abc, ok), xmul(cl, dab, ok), ok),
                xsub(xmul(bl, cda, ok), xmul(al, bcd, ok), ok), ok);
    return ok;
}

// ---- integer certificates
// When every coordinate of a query is an integer multiple of one power of two 2^L
// and |v| / 2^L < 2^B, the scaled coordinates are exact integers (int64) and the
// determinant of their differences, evaluated in 128-bit integers, is exact; scaling
// by 2^-L > 0 keeps its sign. B is chosen per predicate so that no intermediate can
// overflow. Decomposition is on the integer pipe (the FP64 pipe is narrow here).
__device__ __forceinline__ bool scale_to_ints(const double* v, int n, int B, long long* out,
                                              int* scale_exp = nullptr) {
    int lmin = 0x7fffffff, emax = -0x7fffffff;
    for (int i = 0; i < n; ++i) {
        const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v[i]));
        if ((b << 1) == 0ull) continue;  // +-0
        const int ef = static_cast<int>((b >> 52) & 0x7ffull);
        if (ef == 0 || ef == 0x7ff) return false;  // subnormal, infinite or NaN
        const unsigned long long m = (b & 0xfffffffffffffull) | (1ull << 52);
        const int e = ef - 1023;
        const int lb = e - 52 + (__ffsll(static_cast<long long>(m)) - 1);
        lmin = min(lmin, lb);
        emax = max(emax, e);
    }
    if (lmin == 0x7fffffff) {  // all zero
        for (int i = 0; i < n; ++i) out[i] = 0;
        if (scale_exp) *scale_exp = 0;
        return true;
    }
    if (emax - lmin + 1 > B) return false;
    if (scale_exp) *scale_exp = lmin;
    for (int i = 0; i < n; ++i) {
        const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v[i]));
        if ((b << 1) == 0ull) {
            out[i] = 0;
            continue;
        }
        const unsigned long long m = (b & 0xfffffffffffffull) | (1ull << 52);
        const int tz = __ffsll(static_cast<long long>(m)) - 1;
        const int lb = static_cast<int>((b >> 52) & 0x7ffull) - 1023 - 52 + tz;
        const long long x = static_cast<long long>((m >> tz) << (lb - lmin));
        out[i] = (b >> 63) ? -x : x;
    }
    return true;
}

// orient3d on integers: differences < 2^41, 2x2 minors < 2^83, terms < 2^124,
// the sum of three < 2^126.
__device__ __forceinline__ bool orient3d_int(const d3& a, const d3& b, const d3& c, const d3& d,
                                             int* sign) {
    const double v[12] = {a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z, d.x, d.y, d.z};
    long long X[12];
    if (!scale_to_ints(v, 12, 40, X)) return false;
    const long long adx = X[0] - X[9], ady = X[1] - X[10], adz = X[2] - X[11];
    const long long bdx = X[3] - X[9], bdy = X[4] - X[10], bdz = X[5] - X[11];
    const long long cdx = X[6] - X[9], cdy = X[7] - X[10], cdz = X[8] - X[11];
    const __int128 m1 = static_cast<__int128>(bdx) * cdy - static_cast<__int128>(cdx) * bdy;
    const __int128 m2 = static_cast<__int128>(cdx) * ady - static_cast<__int128>(adx) * cdy;
    const __int128 m3 = static_cast<__int128>(adx) * bdy - static_cast<__int128>(bdx) * ady;
    const __int128 det = adz * m1 + bdz * m2 + cdz * m3;
    *sign = det > 0 ? 1 : (det < 0 ? -1 : 0);
    return true;
}

// The sign of orient3d on integer coordinates, and whether the reference's FP64
// evaluation (any operation order) is exact there: with every difference at most 2^16
// in the common scale 2^L, products stay below 2^32, minors below 2^33, terms below
// 2^50 and the determinant below 2^53 (6 D^3), and with -320 <= L, and every
// coordinate below 2^300, nothing underflows or overflows; the FP64 rounded
// determinant then equals the exact one.
__device__ __forceinline__ bool orient3d_int_exact64(const d3& a, const d3& b, const d3& c,
                                                     const d3& d, int* sign, bool* fp64_exact) {
    const double v[12] = {a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z, d.x, d.y, d.z};
    long long X[12];
    int L = 0;
    if (!scale_to_ints(v, 12, 40, X, &L)) return false;
    const long long adx = X[0] - X[9], ady = X[1] - X[10], adz = X[2] - X[11];
    const long long bdx = X[3] - X[9], bdy = X[4] - X[10], bdz = X[5] - X[11];
    const long long cdx = X[6] - X[9], cdy = X[7] - X[10], cdz = X[8] - X[11];
    const __int128 m1 = static_cast<__int128>(bdx) * cdy - static_cast<__int128>(cdx) * bdy;
    const __int128 m2 = static_cast<__int128>(cdx) * ady - static_cast<__int128>(adx) * cdy;
    const __int128 m3 = static_cast<__int128>(adx) * bdy - static_cast<__int128>(bdx) * ady;
    const __int128 det = adz * m1 + bdz * m2 + cdz * m3;
    *sign = det > 0 ? 1 : (det < 0 ? -1 : 0);
    long long D = 0;
    const long long dd[9] = {adx, ady, adz, bdx, bdy, bdz, cdx, cdy, cdz};
    for (int k = 0; k < 9; ++k) D = max(D, dd[k] < 0 ? -dd[k] : dd[k]);
    long long M = 0;
    for (int k = 0; k < 12; ++k) M = max(M, X[k] < 0 ? -X[k] : X[k]);
    *fp64_exact = D <= (1ll << 16) && L >= -320 && (M == 0 || L + 41 <= 300);
    return true;
}

// insphere (lifted 4x4, e as origin) on integers: differences < 2^23, 2x2 minors
// < 2^47, 3x3 minors < 2^72, lifts < 2^48, terms < 2^120, the sum of four < 2^122.
__device__ __forceinline__ bool insphere_int(const d3& a, const d3& b, const d3& c, const d3& d,
                                             const d3& e, int* sign) {
    const double v[15] = {a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z,
                          d.x, d.y, d.z, e.x, e.y, e.z};
    long long X[15];
    if (!scale_to_ints(v, 15, 22, X)) return false;
    const long long aex = X[0] - X[12], aey = X[1] - X[13], aez = X[2] - X[14];
    const long long bex = X[3] - X[12], bey = X[4] - X[13], bez = X[5] - X[14];
    const long long cex = X[6] - X[12], cey = X[7] - X[13], cez = X[8] - X[14];
    const long long dex = X[9] - X[12], dey = X[10] - X[13], dez = X[11] - X[14];
    const long long ab = aex * bey - bex * aey, bc = bex * cey - cex * bey;
    const long long cd = cex * dey - dex * cey, da = dex * aey - aex * dey;
    const long long ac = aex * cey - cex * aey, bd = bex * dey - dex * bey;
    const __int128 abc = static_cast<__int128>(aez) * bc - static_cast<__int128>(bez) * ac +
                         static_cast<__int128>(cez) * ab;
    const __int128 bcd = static_cast<__int128>(bez) * cd - static_cast<__int128>(cez) * bd +
                         static_cast<__int128>(dez) * bc;
    const __int128 cda = static_cast<__int128>(cez) * da + static_cast<__int128>(dez) * ac +
                         static_cast<__int128>(aez) * cd;
    const __int128 dab = static_cast<__int128>(dez) * ab + static_cast<__int128>(aez) * bd +
                         static_cast<__int128>(bez) * da;
    const long long al = aex * aex + aey * aey + aez * aez;
    const long long bl = bex * bex + bey * bey + bez * bez;
    const long long cl = cex * cex + cey * cey + cez * cez;
    const long long dl = dex * dex + dey * dey + dez * dez;
    const __int128 det = (dl * abc - cl * dab) + (bl * cda - al * bcd);
    *sign = det > 0 ? 1 : (det < 0 ? -1 : 0);
    return true;
}

// The same for insphere: differences at most 2^9 keep every intermediate of the
// lifted evaluation below 2^53 (72 D^5), with -190 <= L and coordinates below 2^180.
__device__ __forceinline__ bool insphere_int_exact64(const d3& a, const d3& b, const d3& c,
                                                     const d3& d, const d3& e, int* sign,
                                                     bool* fp64_exact) {
    const double v[15] = {a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z,
                          d.x, d.y, d.z, e.x, e.y, e.z};
    long long X[15];
    int L = 0;
    if (!scale_to_ints(v, 15, 22, X, &L)) return false;
    long long D = 0;
    for (int k = 0; k < 12; ++k) {
        const long long q = X[k] - X[12 + k % 3];
        D = max(D, q < 0 ? -q : q);
    }
    long long M = 0;
    for (int k = 0; k < 15; ++k) M = max(M, X[k] < 0 ? -X[k] : X[k]);
    *fp64_exact = D <= (1ll << 9) && L >= -190 && (M == 0 || L + 23 <= 180);
    return insphere_int(a, b, c, d, e, sign);
}

// h = e + f: merge by magnitude, then a Two-Sum sweep, zero-eliminated.
// h holds elen + flen doubles and may not alias e or f.
static __device__ __noinline__ int sum(int elen, const double* e, int flen, const double* f,
                                double* h) {
    int i = 0, j = 0, hn = 0;
    double q;
    bool have = false;
    while (i < elen || j < flen) {
        double g;
        if (j >= flen || (i < elen && fabs(e[i]) <= fabs(f[j]))) g = e[i++];
        else g = f[j++];
        if (!have) {
            q = g;
            have = true;
            continue;
        }
        double qn, hh;
        two_sum(q, g, qn, hh);
        q = qn;
        if (hh != 0.0) h[hn++] = hh;
    }
    if (!have) q = 0.0;
    if (q != 0.0 || hn == 0) h[hn++] = q;
    return hn;
}

// h = b * e, zero-eliminated; h holds 2 * elen doubles.
static __device__ __noinline__ int scale(int elen, const double* e, double b, double* h) {
    double q, hh;
    int hn = 0;
    two_prod(e[0], b, q, hh);
    if (hh != 0.0) h[hn++] = hh;
    for (int i = 1; i < elen; ++i) {
        double p1, p0, s;
        two_prod(e[i], b, p1, p0);
        two_sum(q, p0, s, hh);
        if (hh != 0.0) h[hn++] = hh;
        fast_two_sum(p1, s, q, hh);
        if (hh != 0.0) h[hn++] = hh;
    }
    if (q != 0.0 || hn == 0) h[hn++] = q;
    return hn;
}

// Renormalise in place (Shewchuk's Compress): same value, fewer components.
static __device__ __noinline__ int compress(int m, double* e) {
    if (m <= 1) return m;
    double q = e[m - 1];
    int bottom = m - 1;
    for (int i = m - 2; i >= 0; --i) {
        double qn, lo;
        fast_two_sum(q, e[i], qn, lo);
        if (lo != 0.0) {
            e[bottom--] = qn;
            q = lo;
        } else {
            q = qn;
        }
    }
    e[bottom] = q;
    int top = 0;
    for (int i = bottom + 1; i < m; ++i) {
        double qn, lo;
        fast_two_sum(e[i], q, qn, lo);
        q = qn;
        if (lo != 0.0) e[top++] = lo;
    }
    e[top++] = q;
    return top;
}

__device__ __forceinline__ int sign_of(int n, const double* e) {
    double t = e[n - 1];
    return t > 0.0 ? 1 : (t < 0.0 ? -1 : 0);
}

// m(u, v) = ux*vy - vx*uy, exactly (<= 4 components).
__device__ __forceinline__ int minor2(double ux, double uy, double vx, double vy, double* out) {
    double p[2], q[2];
    two_prod(ux, vy, p[1], p[0]);
    two_prod(vx, uy, q[1], q[0]);
    q[0] = -q[0];
    q[1] = -q[1];
    return sum(2, p, 2, q, out);
}

// |pqr| (rows of x, y, z) = pz*m(q,r) - qz*m(p,r) + rz*m(p,q), exactly (<= 24).
static __device__ __noinline__ int det3(const d3& p, const d3& q, const d3& r, double* out) {
    double mqr[4], mpr[4], mpq[4], s1[8], s2[8], s3[8], t[16];
    int n1 = minor2(q.x, q.y, r.x, r.y, mqr);
    int n2 = minor2(p.x, p.y, r.x, r.y, mpr);
    int n3 = minor2(p.x, p.y, q.x, q.y, mpq);
    int l1 = scale(n1, mqr, p.z, s1);
    int l2 = scale(n2, mpr, -q.z, s2);
    int l3 = scale(n3, mpq, r.z, s3);
    int lt = sum(l1, s1, l2, s2, t);
    return sum(lt, t, l3, s3, out);
}

// Exact orient3d(a,b,c,d) with homogeneous coordinates (no rounding in the
// differences): |abc| - |abd| + |acd| - |bcd| (<= 96 components).
static __device__ __noinline__ int orient3d_homogeneous(const d3& a, const d3& b, const d3& c,
                                                 const d3& d, double* out) {
    double t1[24], t2[24], t3[24], t4[24], u[48], v[48];
    int n1 = det3(a, b, c, t1);
    int n2 = det3(a, b, d, t2);
    int n3 = det3(a, c, d, t3);
    int n4 = det3(b, c, d, t4);
    for (int i = 0; i < n2; ++i) t2[i] = -t2[i];
    for (int i = 0; i < n4; ++i) t4[i] = -t4[i];
    int nu = sum(n1, t1, n2, t2, u);
    int nv = sum(n3, t3, n4, t4, v);
    return sum(nu, u, nv, v, out);
}

// Exact sign of orient3d(a, b, c, d).
static __device__ __noinline__ int orient3d_sign(const d3& a, const d3& b, const d3& c, const d3& d) {
    {
        int sg;
        if (orient3d_int(a, b, c, d, &sg)) return sg;
        double det;
        if (orient3d_certified(a, b, c, d, &det)) return det > 0.0 ? 1 : (det < 0.0 ? -1 : 0);
    }
    double adx, ady, adz, bdx, bdy, bdz, cdx, cdy, cdz;
    double t0, t1, t2, t3, t4, t5, t6, t7, t8;
    two_diff(a.x, d.x, adx, t0);
    two_diff(a.y, d.y, ady, t1);
    two_diff(a.z, d.z, adz, t2);
    two_diff(b.x, d.x, bdx, t3);
    two_diff(b.y, d.y, bdy, t4);
    two_diff(b.z, d.z, bdz, t5);
    two_diff(c.x, d.x, cdx, t6);
    two_diff(c.y, d.y, cdy, t7);
    two_diff(c.z, d.z, cdz, t8);
    if (t0 == 0.0 && t1 == 0.0 && t2 == 0.0 && t3 == 0.0 && t4 == 0.0 && t5 == 0.0 &&
        t6 == 0.0 && t7 == 0.0 && t8 == 0.0) {
        // the differences are exact: a 3x3 determinant suffices
        double e[24];
        int n = det3({adx, ady, adz}, {bdx, bdy, bdz}, {cdx, cdy, cdz}, e);
        return sign_of(n, e);
    }
    double e[96];
    int n = orient3d_homogeneous(a, b, c, d, e);
    return sign_of(n, e);
}

// acc += s * w * x (w a short expansion, x up to 96 components); acc holds cap
// doubles, work holds cap + 192. Returns the new length or -1 on overflow.
static __device__ __noinline__ int accumulate(int nacc, double* acc, int nw, const double* w, double s,
                                       int nx, const double* x, double* work, int cap) {
    double prod[192];
    for (int c = 0; c < nw; ++c) {
        int np = scale(nx, x, s * w[c], prod);
        if (nacc + np > cap + 192) return -1;
        int nn = sum(nacc, acc, np, prod, work);
        nn = compress(nn, work);
        if (nn > cap) return -1;
        for (int i = 0; i < nn; ++i) acc[i] = work[i];
        nacc = nn;
    }
    return nacc;
}

// Exact lift x^2 + y^2 + z^2 (<= 6 components).
__device__ __forceinline__ int lift(const d3& p, double* out) {
    double sx[2], sy[2], sz[2], t[4];
    two_prod(p.x, p.x, sx[1], sx[0]);
    two_prod(p.y, p.y, sy[1], sy[0]);
    two_prod(p.z, p.z, sz[1], sz[0]);
    int n = sum(2, sx, 2, sy, t);
    return sum(n, t, 2, sz, out);
}

constexpr int kInsphereCap = 256;

// Exact sign of insphere(a, b, c, d, e); sets *overflow when the accumulator
// capacity is exceeded (the sign is then 0 and must not be trusted).
static __device__ __noinline__ int insphere_sign(const d3& a, const d3& b, const d3& c, const d3& d,
                                          const d3& e, int* overflow) {
    {
        int sg;
        if (insphere_int(a, b, c, d, e, &sg)) return sg;
        double det;
        if (insphere_certified(a, b, c, d, e, &det)) return det > 0.0 ? 1 : (det < 0.0 ? -1 : 0);
    }
    double acc[kInsphereCap], work[kInsphereCap + 192];
    int nacc = 1;
    acc[0] = 0.0;
    double tails[12];
    double aex, aey, aez, bex, bey, bez, cex, cey, cez, dex, dey, dez;
    two_diff(a.x, e.x, aex, tails[0]);
    two_diff(a.y, e.y, aey, tails[1]);
    two_diff(a.z, e.z, aez, tails[2]);
    two_diff(b.x, e.x, bex, tails[3]);
    two_diff(b.y, e.y, bey, tails[4]);
    two_diff(b.z, e.z, bez, tails[5]);
    two_diff(c.x, e.x, cex, tails[6]);
    two_diff(c.y, e.y, cey, tails[7]);
    two_diff(c.z, e.z, cez, tails[8]);
    two_diff(d.x, e.x, dex, tails[9]);
    two_diff(d.y, e.y, dey, tails[10]);
    two_diff(d.z, e.z, dez, tails[11]);
    bool exact_diff = true;
    for (int i = 0; i < 12; ++i) exact_diff = exact_diff && tails[i] == 0.0;
    if (exact_diff) {
        // translated form: det4 = -la|bcd| + lb|acd| - lc|abd| + ld|abc|
        const d3 P[4] = {{aex, aey, aez}, {bex, bey, bez}, {cex, cey, cez}, {dex, dey, dez}};
        for (int i = 0; i < 4; ++i) {
            const d3* q[3];
            int k = 0;
            for (int j = 0; j < 4; ++j)
                if (j != i) q[k++] = &P[j];
            double m[24], w[6];
            int nm = det3(*q[0], *q[1], *q[2], m);
            int nw = lift(P[i], w);
            double s = (i % 2 == 0) ? -1.0 : 1.0;
            nacc = accumulate(nacc, acc, nw, w, s, nm, m, work, kInsphereCap);
            if (nacc < 0) {
                *overflow = 1;
                return 0;
            }
        }
        return sign_of(nacc, acc);
    }
    // homogeneous form: det5 = sum_i (-1)^(i+1) w_i O(others), i over a..e
    const d3 P[5] = {a, b, c, d, e};
    for (int i = 0; i < 5; ++i) {
        const d3* q[4];
        int k = 0;
        for (int j = 0; j < 5; ++j)
            if (j != i) q[k++] = &P[j];
        double o[96], w[6];
        int no = orient3d_homogeneous(*q[0], *q[1], *q[2], *q[3], o);
        int nw = lift(P[i], w);
        double s = (i % 2 == 0) ? -1.0 : 1.0;
        nacc = accumulate(nacc, acc, nw, w, s, no, o, work, kInsphereCap);
        if (nacc < 0) {
            *overflow = 1;
            return 0;
        }
    }
    return sign_of(nacc, acc);
}

}  // namespace cmg::gpu::exact
