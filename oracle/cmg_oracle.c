/* cmg_oracle.c — CPU restatement of the reference voxelization path.
 *
 * TEST INFRASTRUCTURE ONLY (the parity checker; see cmg_oracle.h). Compile with
 * -ffp-contract=off and without -ffast-math: every floating-point expression here
 * must round exactly as the reference's x86-64 (SSE2, no FMA) build rounds it.
 */
#define _POSIX_C_SOURCE 199309L /* clock_gettime */
#include "cmg_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifdef _OPENMP
#include <omp.h>
#define ORC_PRAGMA(x) _Pragma(#x)
#define ORC_PAR_FOR(n) ORC_PRAGMA(omp parallel for schedule(dynamic, 64) num_threads(n))
#else
#define ORC_PAR_FOR(n)
#endif

/* ========================================================================== */
/* Expansion arithmetic (Shewchuk CMU-CS-96-140, restated).                   */
/* ========================================================================== */

/* epsilon = 2^-53 and splitter = 2^27 + 1 are what the reference's exactinit
 * computes on an IEEE binary64 machine (src/predicates/predicates.cpp:591-610). */
static const double kEps = 1.1102230246251565e-16;        /* 2^-53 */
static const double kSplitter = 134217729.0;               /* 2^27 + 1 */

static void two_sum(double a, double b, double* x, double* y) {
    double s = a + b;
    double bv = s - a;
    double av = s - bv;
    double br = b - bv;
    double ar = a - av;
    *x = s;
    *y = ar + br;
}

static void fast_two_sum(double a, double b, double* x, double* y) {
    double s = a + b;
    double bv = s - a;
    *x = s;
    *y = b - bv;
}

static void split(double a, double* hi, double* lo) {
    double c = kSplitter * a;
    double abig = c - a;
    *hi = c - abig;
    *lo = a - *hi;
}

static void two_product(double a, double b, double* x, double* y) {
    double p = a * b;
    double ahi, alo, bhi, blo;
    split(a, &ahi, &alo);
    split(b, &bhi, &blo);
    double err1 = p - ahi * bhi;
    double err2 = err1 - alo * bhi;
    double err3 = err2 - ahi * blo;
    *x = p;
    *y = alo * blo - err3;
}

/* h = e + b, zero-eliminated; returns the length of h. h may not alias e. */
static int grow_expansion(int elen, const double* e, double b, double* h) {
    double q = b;
    int hn = 0;
    for (int i = 0; i < elen; ++i) {
        double qn, hh;
        two_sum(q, e[i], &qn, &hh);
        q = qn;
        if (hh != 0.0) h[hn++] = hh;
    }
    if (q != 0.0 || hn == 0) h[hn++] = q;
    return hn;
}

/* h = e + f by repeated growth (Shewchuk's Expansion-Sum), zero-eliminated.
 * tmp must hold elen+flen doubles; h likewise. */
static int expansion_sum(int elen, const double* e, int flen, const double* f,
                         double* h, double* tmp) {
    int n = elen;
    memcpy(h, e, sizeof(double) * (size_t)elen);
    for (int j = 0; j < flen; ++j) {
        int m = grow_expansion(n, h, f[j], tmp);
        memcpy(h, tmp, sizeof(double) * (size_t)m);
        n = m;
    }
    return n;
}

/* h = b * e (Scale-Expansion), zero-eliminated. h holds 2*elen doubles. */
static int scale_expansion(int elen, const double* e, double b, double* h) {
    double q, hh;
    int hn = 0;
    two_product(e[0], b, &q, &hh);
    if (hh != 0.0) h[hn++] = hh;
    for (int i = 1; i < elen; ++i) {
        double p1, p0, sum;
        two_product(e[i], b, &p1, &p0);
        two_sum(q, p0, &sum, &hh);
        if (hh != 0.0) h[hn++] = hh;
        fast_two_sum(p1, sum, &q, &hh);
        if (hh != 0.0) h[hn++] = hh;
    }
    if (q != 0.0 || hn == 0) h[hn++] = q;
    return hn;
}

static int expansion_sign(int n, const double* e) {
    double top = e[n - 1];
    return top > 0 ? 1 : (top < 0 ? -1 : 0);
}

static void negate(int n, double* e) {
    for (int i = 0; i < n; ++i) e[i] = -e[i];
}

/* Exact 2x2 xy minor m(u,v) = ux*vy - vx*uy; up to 4 components. */
static int minor2(const double* u, const double* v, double* out) {
    double p[2], q[2], tmp[4];
    two_product(u[0], v[1], &p[1], &p[0]);
    two_product(v[0], u[1], &q[1], &q[0]);
    q[0] = -q[0];
    q[1] = -q[1];
    return expansion_sum(2, p, 2, q, out, tmp);
}

/* Exact 3x3 determinant of rows p,q,r (x,y,z), expanded along z:
 *   |pqr| = pz*m(q,r) - qz*m(p,r) + rz*m(p,q); up to 24 components. */
static int det3(const double* p, const double* q, const double* r, double* out) {
    double mqr[4], mpr[4], mpq[4], s1[8], s2[8], s3[8], t[24], tmp[24];
    int n1 = minor2(q, r, mqr), n2 = minor2(p, r, mpr), n3 = minor2(p, q, mpq);
    int l1 = scale_expansion(n1, mqr, p[2], s1);
    int l2 = scale_expansion(n2, mpr, -q[2], s2);
    int l3 = scale_expansion(n3, mpq, r[2], s3);
    int lt = expansion_sum(l1, s1, l2, s2, t, tmp);
    return expansion_sum(lt, t, l3, s3, out, tmp);
}

/* Exact orient3d(a,b,c,d) = det[[a,1],[b,1],[c,1],[d,1]]
 *                         = |abc| - |abd| + |acd| - |bcd|; up to 96 components. */
static int orient3d_expansion(const double* a, const double* b, const double* c,
                              const double* d, double* out) {
    double t1[24], t2[24], t3[24], t4[24], u[48], v[48], tmp[96];
    int n1 = det3(a, b, c, t1);
    int n2 = det3(a, b, d, t2);
    int n3 = det3(a, c, d, t3);
    int n4 = det3(b, c, d, t4);
    negate(n2, t2);
    negate(n4, t4);
    int nu = expansion_sum(n1, t1, n2, t2, u, tmp);
    int nv = expansion_sum(n3, t3, n4, t4, v, tmp);
    return expansion_sum(nu, u, nv, v, out, tmp);
}

int orc_orient3d_exact_sign(const double* pa, const double* pb, const double* pc,
                            const double* pd) {
    double e[96];
    int n = orient3d_expansion(pa, pb, pc, pd, e);
    return expansion_sign(n, e);
}

/* Exact insphere(a,b,c,d,e) = det of the 5x5 rows [x, y, z, x^2+y^2+z^2, 1]
 * (equal to the reference's translated 4x4 lifted determinant). Expanded along
 * the lift column:
 *   det5 = -wa*O(b,c,d,e) + wb*O(a,c,d,e) - wc*O(a,b,d,e) + wd*O(a,b,c,e)
 *          - we*O(a,b,c,d)
 * with O the exact orient3d expansion and w the exact lift (6 components). */
int orc_insphere_exact_sign(const double* pa, const double* pb, const double* pc,
                            const double* pd, const double* pe) {
    const double* P[5] = {pa, pb, pc, pd, pe};
    const size_t cap = 8192;
    double* acc = (double*)malloc(sizeof(double) * cap);
    double* nxt = (double*)malloc(sizeof(double) * cap);
    double* tmp = (double*)malloc(sizeof(double) * cap);
    int nacc = 1;
    acc[0] = 0.0;
    for (int i = 0; i < 5; ++i) {
        const double* q[4];
        int k = 0;
        for (int j = 0; j < 5; ++j)
            if (j != i) q[k++] = P[j];
        double o[96];
        int no = orient3d_expansion(q[0], q[1], q[2], q[3], o);
        /* lift of P[i]: three exact squares summed */
        double sq[6], lift[6], t6[6];
        two_product(P[i][0], P[i][0], &sq[1], &sq[0]);
        two_product(P[i][1], P[i][1], &sq[3], &sq[2]);
        two_product(P[i][2], P[i][2], &sq[5], &sq[4]);
        int nl = expansion_sum(2, sq, 2, sq + 2, lift, t6);
        double l4[4];
        memcpy(l4, lift, sizeof(double) * (size_t)nl);
        nl = expansion_sum(nl, l4, 2, sq + 4, lift, t6);
        double sgn = (i % 2 == 0) ? -1.0 : 1.0;
        for (int c = 0; c < nl; ++c) {
            double prod[192];
            int np = scale_expansion(no, o, sgn * lift[c], prod);
            int nn = expansion_sum(nacc, acc, np, prod, nxt, tmp);
            double* sw = acc;
            acc = nxt;
            nxt = sw;
            nacc = nn;
        }
    }
    int s = expansion_sign(nacc, acc);
    free(acc);
    free(nxt);
    free(tmp);
    return s;
}

/* ========================================================================== */
/* Rounded determinants in the reference's operation order.                   */
/* ========================================================================== */

static double o3d_fast_perm(const double* pa, const double* pb, const double* pc,
                            const double* pd, double* permanent) {
    double adx = pa[0] - pd[0], ady = pa[1] - pd[1], adz = pa[2] - pd[2];
    double bdx = pb[0] - pd[0], bdy = pb[1] - pd[1], bdz = pb[2] - pd[2];
    double cdx = pc[0] - pd[0], cdy = pc[1] - pd[1], cdz = pc[2] - pd[2];
    double bdxcdy = bdx * cdy, cdxbdy = cdx * bdy;
    double cdxady = cdx * ady, adxcdy = adx * cdy;
    double adxbdy = adx * bdy, bdxady = bdx * ady;
    double det = adz * (bdxcdy - cdxbdy) + bdz * (cdxady - adxcdy) +
                 cdz * (adxbdy - bdxady);
    if (permanent)
        *permanent = (fabs(bdxcdy) + fabs(cdxbdy)) * fabs(adz) +
                     (fabs(cdxady) + fabs(adxcdy)) * fabs(bdz) +
                     (fabs(adxbdy) + fabs(bdxady)) * fabs(cdz);
    return det;
}

double orc_orient3d_fast(const double* pa, const double* pb, const double* pc,
                         const double* pd) {
    return o3d_fast_perm(pa, pb, pc, pd, NULL);
}

static double isp_fast_perm(const double* pa, const double* pb, const double* pc,
                            const double* pd, const double* pe, double* permanent) {
    double aex = pa[0] - pe[0], bex = pb[0] - pe[0], cex = pc[0] - pe[0],
           dex = pd[0] - pe[0];
    double aey = pa[1] - pe[1], bey = pb[1] - pe[1], cey = pc[1] - pe[1],
           dey = pd[1] - pe[1];
    double aez = pa[2] - pe[2], bez = pb[2] - pe[2], cez = pc[2] - pe[2],
           dez = pd[2] - pe[2];
    double aexbey = aex * bey, bexaey = bex * aey;
    double ab = aexbey - bexaey;
    double bexcey = bex * cey, cexbey = cex * bey;
    double bc = bexcey - cexbey;
    double cexdey = cex * dey, dexcey = dex * cey;
    double cd = cexdey - dexcey;
    double dexaey = dex * aey, aexdey = aex * dey;
    double da = dexaey - aexdey;
    double aexcey = aex * cey, cexaey = cex * aey;
    double ac = aexcey - cexaey;
    double bexdey = bex * dey, dexbey = dex * bey;
    double bd = bexdey - dexbey;
    double abc = aez * bc - bez * ac + cez * ab;
    double bcd = bez * cd - cez * bd + dez * bc;
    double cda = cez * da + dez * ac + aez * cd;
    double dab = dez * ab + aez * bd + bez * da;
    double alift = aex * aex + aey * aey + aez * aez;
    double blift = bex * bex + bey * bey + bez * bez;
    double clift = cex * cex + cey * cey + cez * cez;
    double dlift = dex * dex + dey * dey + dez * dez;
    double det = (dlift * abc - clift * dab) + (blift * cda - alift * bcd);
    if (permanent) {
        double aezp = fabs(aez), bezp = fabs(bez), cezp = fabs(cez), dezp = fabs(dez);
        double aexbeyp = fabs(aexbey), bexaeyp = fabs(bexaey);
        double bexceyp = fabs(bexcey), cexbeyp = fabs(cexbey);
        double cexdeyp = fabs(cexdey), dexceyp = fabs(dexcey);
        double dexaeyp = fabs(dexaey), aexdeyp = fabs(aexdey);
        double aexceyp = fabs(aexcey), cexaeyp = fabs(cexaey);
        double bexdeyp = fabs(bexdey), dexbeyp = fabs(dexbey);
        *permanent = ((cexdeyp + dexceyp) * bezp + (dexbeyp + bexdeyp) * cezp +
                      (bexceyp + cexbeyp) * dezp) * alift +
                     ((dexaeyp + aexdeyp) * cezp + (aexceyp + cexaeyp) * dezp +
                      (cexdeyp + dexceyp) * aezp) * blift +
                     ((aexbeyp + bexaeyp) * dezp + (bexdeyp + dexbeyp) * aezp +
                      (dexaeyp + aexdeyp) * bezp) * clift +
                     ((bexceyp + cexbeyp) * aezp + (cexaeyp + aexceyp) * bezp +
                      (aexbeyp + bexaeyp) * cezp) * dlift;
    }
    return det;
}

double orc_insphere_fast(const double* pa, const double* pb, const double* pc,
                         const double* pd, const double* pe) {
    return isp_fast_perm(pa, pb, pc, pd, pe, NULL);
}

static int sgn(double v) { return v > 0 ? 1 : (v < 0 ? -1 : 0); }

/* Error-bound constants (predicates.cpp:617, :623). */
#define O3D_ERRBOUND_A ((7.0 + 56.0 * kEps) * kEps)
#define ISP_ERRBOUND_A ((16.0 + 224.0 * kEps) * kEps)

int orc_orient3d_sign(const double* pa, const double* pb, const double* pc,
                      const double* pd, int mode) {
    double perm;
    double det = o3d_fast_perm(pa, pb, pc, pd, &perm);
    if (mode == ORC_COMPAT) {
        /* as initialised: static filter 0 -> rounded det returned when nonzero */
        if (det != 0.0) return sgn(det);
    } else {
        double eb = O3D_ERRBOUND_A * perm;
        if (det > eb || -det > eb) return sgn(det);
    }
    return orc_orient3d_exact_sign(pa, pb, pc, pd);
}

int orc_insphere_sign(const double* pa, const double* pb, const double* pc,
                      const double* pd, const double* pe, int mode) {
    double perm;
    double det = isp_fast_perm(pa, pb, pc, pd, pe, &perm);
    if (mode == ORC_COMPAT) {
        if (det != 0.0) return sgn(det);
    } else {
        double eb = ISP_ERRBOUND_A * perm;
        if (det > eb || -det > eb) return sgn(det);
    }
    return orc_insphere_exact_sign(pa, pb, pc, pd, pe);
}

void orc_orient3d_stream(const double* const* s, int64_t n, int mode, int8_t* out,
                         int nthreads) {
    (void)nthreads;
    ORC_PAR_FOR(nthreads)
    for (int64_t i = 0; i < n; ++i) {
        double a[3] = {s[0][i], s[1][i], s[2][i]};
        double b[3] = {s[3][i], s[4][i], s[5][i]};
        double c[3] = {s[6][i], s[7][i], s[8][i]};
        double d[3] = {s[9][i], s[10][i], s[11][i]};
        out[i] = (int8_t)orc_orient3d_sign(a, b, c, d, mode);
    }
}

void orc_insphere_stream(const double* const* s, int64_t n, int mode, int8_t* out,
                         int nthreads) {
    (void)nthreads;
    ORC_PAR_FOR(nthreads)
    for (int64_t i = 0; i < n; ++i) {
        double a[3] = {s[0][i], s[1][i], s[2][i]};
        double b[3] = {s[3][i], s[4][i], s[5][i]};
        double c[3] = {s[6][i], s[7][i], s[8][i]};
        double d[3] = {s[9][i], s[10][i], s[11][i]};
        double e[3] = {s[12][i], s[13][i], s[14][i]};
        out[i] = (int8_t)orc_insphere_sign(a, b, c, d, e, mode);
    }
}

/* ========================================================================== */
/* Grid (voxelize.cpp:52-74) and fan triangulation (voxelize.cpp:29-38).      */
/* ========================================================================== */

int orc_make_grid(const double* pts, int64_t npts, int resolution, int pad,
                  orc_grid* g) {
    double lo[3] = {pts[0], pts[1], pts[2]}, hi[3] = {pts[0], pts[1], pts[2]};
    for (int64_t i = 0; i < npts; ++i)
        for (int a = 0; a < 3; ++a) {
            double v = pts[3 * i + a];
            if (v < lo[a]) lo[a] = v;
            if (v > hi[a]) hi[a] = v;
        }
    double ext = 0;
    for (int a = 0; a < 3; ++a) {
        double e = hi[a] - lo[a];
        if (e > ext) ext = e; /* std::max(ext, e) keeps ext on ties */
    }
    memset(g, 0, sizeof(*g));
    g->spacing = ext / resolution;
    if (!(g->spacing > 0)) return -1;
    int* dims[3] = {&g->nx, &g->ny, &g->nz};
    for (int a = 0; a < 3; ++a) {
        double e = hi[a] - lo[a];
        int core = (int)ceil(e / g->spacing);
        if (core < 1) core = 1;
        double covered = core * g->spacing;
        g->corner[a] = lo[a] - (covered - e) / 2.0 - pad * g->spacing;
        *dims[a] = core + 2 * pad;
    }
    return 0;
}

int64_t orc_fan_triangles(const int* idx, const int64_t* off, int64_t nfacets,
                          int* tris) {
    int64_t nt = 0;
    for (int64_t f = 0; f < nfacets; ++f) {
        int64_t b = off[f], e = off[f + 1];
        for (int64_t i = b + 2; i < e; ++i) {
            if (tris) {
                tris[3 * nt] = idx[b];
                tris[3 * nt + 1] = idx[i - 1];
                tris[3 * nt + 2] = idx[i];
            }
            ++nt;
        }
    }
    return nt;
}

/* ========================================================================== */
/* Occupancy by vertical ray parity (voxelize.cpp:78-196).                    */
/* ========================================================================== */

static int cell_clamped(double x, double corner, double spacing, int n) {
    int i = (int)floor((x - corner) / spacing);
    return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

/* z of the vertical line (x,y) on the plane of abc (voxelize.cpp:107-114). */
static double plane_z(const double* a, const double* b, const double* c, double x,
                      double y) {
    double ux = b[0] - a[0], uy = b[1] - a[1], uz = b[2] - a[2];
    double vx = c[0] - a[0], vy = c[1] - a[1], vz = c[2] - a[2];
    double nx = uy * vz - uz * vy;
    double ny = uz * vx - ux * vz;
    double nz = ux * vy - uy * vx;
    return a[2] - (nx * (x - a[0]) + ny * (y - a[1])) / nz;
}

typedef struct col_ctx {
    const double* pts;
    const int* tris;
    int mode;
    int64_t exact_calls, orient_calls;
} col_ctx;

static int o3d_counted(col_ctx* c, const double* pa, const double* pb,
                       const double* pc, const double* pd) {
    double perm;
    double det = o3d_fast_perm(pa, pb, pc, pd, &perm);
    c->orient_calls++;
    if (c->mode == ORC_COMPAT) {
        if (det != 0.0) return sgn(det);
    } else {
        double eb = O3D_ERRBOUND_A * perm;
        if (det > eb || -det > eb) return sgn(det);
    }
    c->exact_calls++;
    return orc_orient3d_exact_sign(pa, pb, pc, pd);
}

/* column_crossings (voxelize.cpp:121-143): returns 0 on a graze. */
static int column_crossings(col_ctx* c, double x, double y, double zmin, double zmax,
                            const int* bucket, int64_t nb, double* heights,
                            int* nh) {
    *nh = 0;
    const double P[3] = {x, y, zmin}, Q[3] = {x, y, zmax};
    for (int64_t k = 0; k < nb; ++k) {
        int ti = bucket[k];
        const double* a = c->pts + 3 * (int64_t)c->tris[3 * (int64_t)ti];
        const double* b = c->pts + 3 * (int64_t)c->tris[3 * (int64_t)ti + 1];
        const double* cc = c->pts + 3 * (int64_t)c->tris[3 * (int64_t)ti + 2];
        int sa = o3d_counted(c, P, a, b, cc);
        int sb = o3d_counted(c, Q, a, b, cc);
        if (sa == 0 || sb == 0) return 0;
        if (sa == sb) continue;
        int s1 = o3d_counted(c, P, Q, a, b);
        int s2 = o3d_counted(c, P, Q, b, cc);
        int s3 = o3d_counted(c, P, Q, cc, a);
        if (s1 == 0 || s2 == 0 || s3 == 0) return 0;
        if (s1 != s2 || s2 != s3) continue;
        heights[(*nh)++] = plane_z(a, b, cc, x, y);
    }
    return 1;
}

static const double kNudge[6][2] = {
    {1.0e-6, 3.0e-7},  {-7.0e-7, 5.0e-7}, {4.0e-7, -9.0e-7},
    {-2.0e-6, -1.0e-6}, {8.0e-7, 6.0e-7}, {-5.0e-7, -4.0e-6},
};

static int cmp_double(const void* a, const void* b) {
    double x = *(const double*)a, y = *(const double*)b;
    return (x > y) - (x < y);
}

void orc_occupancy(const double* pts, const int* tris, int64_t ntris,
                   const orc_grid* g, int mode, uint8_t* occ, orc_occ_stats* st,
                   int nthreads) {
    (void)nthreads;
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    const int64_t ncol = (int64_t)nx * ny;
    memset(occ, 0, (size_t)(ncol * nz));
    /* xy buckets as CSR in ascending triangle order (build_xy_buckets) */
    int* box = (int*)malloc(sizeof(int) * 4 * (size_t)(ntris ? ntris : 1));
    int64_t* cnt = (int64_t*)calloc((size_t)ncol + 1, sizeof(int64_t));
    for (int64_t t = 0; t < ntris; ++t) {
        int i0 = nx, i1 = 0, j0 = ny, j1 = 0;
        for (int v = 0; v < 3; ++v) {
            const double* p = pts + 3 * (int64_t)tris[3 * t + v];
            int i = cell_clamped(p[0], g->corner[0], g->spacing, nx);
            int j = cell_clamped(p[1], g->corner[1], g->spacing, ny);
            if (i < i0) i0 = i;
            if (i > i1) i1 = i;
            if (j < j0) j0 = j;
            if (j > j1) j1 = j;
        }
        box[4 * t] = i0; box[4 * t + 1] = i1; box[4 * t + 2] = j0; box[4 * t + 3] = j1;
        for (int j = j0; j <= j1; ++j)
            for (int i = i0; i <= i1; ++i) cnt[(int64_t)j * nx + i + 1]++;
    }
    for (int64_t c = 0; c < ncol; ++c) cnt[c + 1] += cnt[c];
    int* lists = (int*)malloc(sizeof(int) * (size_t)(cnt[ncol] ? cnt[ncol] : 1));
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)ncol);
    memcpy(fill, cnt, sizeof(int64_t) * (size_t)ncol);
    for (int64_t t = 0; t < ntris; ++t)
        for (int j = box[4 * t + 2]; j <= box[4 * t + 3]; ++j)
            for (int i = box[4 * t]; i <= box[4 * t + 1]; ++i)
                lists[fill[(int64_t)j * nx + i]++] = (int)t;
    free(fill);

    const double h = g->spacing;
    const double zmin = g->corner[2] - h;
    const double zmax = g->corner[2] + (nz + 1) * h;
    int64_t nudged = 0, exhausted = 0, exact_calls = 0, orient_calls = 0, crossings = 0;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads) reduction(+ : nudged, exhausted, exact_calls, orient_calls, crossings)
#endif
    {
        int64_t maxb = 0;
        for (int64_t c = 0; c < ncol; ++c)
            if (cnt[c + 1] - cnt[c] > maxb) maxb = cnt[c + 1] - cnt[c];
        double* heights = (double*)malloc(sizeof(double) * (size_t)(maxb + 1));
        col_ctx ctx = {pts, tris, mode, 0, 0};
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (int64_t col = 0; col < ncol; ++col) {
            int i = (int)(col % nx), j = (int)(col / nx);
            double cx = g->corner[0] + (i + 0.5) * h;
            double cy = g->corner[1] + (j + 0.5) * h;
            const int* bucket = lists + cnt[col];
            int64_t nb = cnt[col + 1] - cnt[col];
            int nh = 0;
            int ok = column_crossings(&ctx, cx, cy, zmin, zmax, bucket, nb, heights, &nh);
            if (!ok) {
                nudged++;
                for (int d = 0; d < 6 && !ok; ++d)
                    ok = column_crossings(&ctx, cx + kNudge[d][0] * h,
                                          cy + kNudge[d][1] * h, zmin, zmax, bucket, nb,
                                          heights, &nh);
                if (!ok) exhausted++;
            }
            crossings += nh;
            qsort(heights, (size_t)nh, sizeof(double), cmp_double);
            for (int k = 0; k < nz; ++k) {
                double zc = g->corner[2] + (k + 0.5) * h;
                /* elements strictly greater than zc (upper_bound) */
                int lo = 0, hi2 = nh;
                while (lo < hi2) {
                    int mid = (lo + hi2) / 2;
                    if (zc < heights[mid]) hi2 = mid; else lo = mid + 1;
                }
                int above = nh - lo;
                if (above & 1) occ[((int64_t)k * ny + j) * nx + i] = 1;
            }
        }
        exact_calls += ctx.exact_calls;
        orient_calls += ctx.orient_calls;
        free(heights);
    }
    if (st) {
        st->columns = ncol;
        st->nudged_columns = nudged;
        st->exhausted_columns = exhausted;
        st->exact_calls = exact_calls;
        st->orient_calls = orient_calls;
        st->crossings = crossings;
    }
    free(lists);
    free(cnt);
    free(box);
}

/* ========================================================================== */
/* Distance (voxelize.cpp:197-358).                                           */
/* ========================================================================== */

static double dot3(const double* a, const double* b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

static double d2q(const double* p, const double* q) {
    double dx = p[0] - q[0], dy = p[1] - q[1], dz = p[2] - q[2];
    return dx * dx + dy * dy + dz * dz;
}

double orc_point_tri_dist2(const double* p, const double* a, const double* b,
                           const double* c, int* region) {
    double ab[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    double ac[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    double ap[3] = {p[0] - a[0], p[1] - a[1], p[2] - a[2]};
    double d1 = dot3(ab, ap), d2 = dot3(ac, ap);
    int r;
    double out;
    if (d1 <= 0 && d2 <= 0) { r = 0; out = d2q(p, a); goto done; }
    {
        double bp[3] = {p[0] - b[0], p[1] - b[1], p[2] - b[2]};
        double d3 = dot3(ab, bp), d4 = dot3(ac, bp);
        if (d3 >= 0 && d4 <= d3) { r = 1; out = d2q(p, b); goto done; }
        double vc = d1 * d4 - d3 * d2;
        if (vc <= 0 && d1 >= 0 && d3 <= 0) {
            double v = d1 / (d1 - d3);
            double q[3] = {a[0] + v * ab[0], a[1] + v * ab[1], a[2] + v * ab[2]};
            r = 2; out = d2q(p, q); goto done;
        }
        double cp[3] = {p[0] - c[0], p[1] - c[1], p[2] - c[2]};
        double d5 = dot3(ab, cp), d6 = dot3(ac, cp);
        if (d6 >= 0 && d5 <= d6) { r = 3; out = d2q(p, c); goto done; }
        double vb = d5 * d2 - d1 * d6;
        if (vb <= 0 && d2 >= 0 && d6 <= 0) {
            double w = d2 / (d2 - d6);
            double q[3] = {a[0] + w * ac[0], a[1] + w * ac[1], a[2] + w * ac[2]};
            r = 4; out = d2q(p, q); goto done;
        }
        double va = d3 * d6 - d5 * d4;
        if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0) {
            double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
            double q[3] = {b[0] + w * (c[0] - b[0]), b[1] + w * (c[1] - b[1]),
                           b[2] + w * (c[2] - b[2])};
            r = 5; out = d2q(p, q); goto done;
        }
        double denom = 1.0 / (va + vb + vc);
        double v = vb * denom, w = vc * denom;
        double q[3] = {a[0] + ab[0] * v + ac[0] * w, a[1] + ab[1] * v + ac[1] * w,
                       a[2] + ab[2] * v + ac[2] * w};
        r = 6; out = d2q(p, q);
    }
done:
    if (region) *region = r;
    return out;
}

static void voxel_center(const orc_grid* g, int64_t idx, double* p, int* ijk) {
    int64_t nxy = (int64_t)g->nx * g->ny;
    int k = (int)(idx / nxy);
    int64_t rem = idx % nxy;
    int j = (int)(rem / g->nx), i = (int)(rem % g->nx);
    p[0] = g->corner[0] + (i + 0.5) * g->spacing;
    p[1] = g->corner[1] + (j + 0.5) * g->spacing;
    p[2] = g->corner[2] + (k + 0.5) * g->spacing;
    if (ijk) { ijk[0] = i; ijk[1] = j; ijk[2] = k; }
}

/* 3-D buckets as CSR in ascending triangle order (build_xyz_buckets). */
typedef struct xyz_buckets {
    int64_t* off;
    int* list;
} xyz_buckets;

static void build_xyz(const double* pts, const int* tris, int64_t ntris,
                      const orc_grid* g, xyz_buckets* B) {
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    const int64_t ncell = (int64_t)nx * ny * nz;
    int* box = (int*)malloc(sizeof(int) * 6 * (size_t)(ntris ? ntris : 1));
    B->off = (int64_t*)calloc((size_t)ncell + 1, sizeof(int64_t));
    for (int64_t t = 0; t < ntris; ++t) {
        int lo[3] = {nx, ny, nz}, hi[3] = {0, 0, 0}, n[3] = {nx, ny, nz};
        for (int v = 0; v < 3; ++v) {
            const double* p = pts + 3 * (int64_t)tris[3 * t + v];
            for (int a = 0; a < 3; ++a) {
                int c = cell_clamped(p[a], g->corner[a], g->spacing, n[a]);
                if (c < lo[a]) lo[a] = c;
                if (c > hi[a]) hi[a] = c;
            }
        }
        for (int a = 0; a < 3; ++a) { box[6 * t + a] = lo[a]; box[6 * t + 3 + a] = hi[a]; }
        for (int k = lo[2]; k <= hi[2]; ++k)
            for (int j = lo[1]; j <= hi[1]; ++j)
                for (int i = lo[0]; i <= hi[0]; ++i)
                    B->off[((int64_t)k * ny + j) * nx + i + 1]++;
    }
    for (int64_t c = 0; c < ncell; ++c) B->off[c + 1] += B->off[c];
    B->list = (int*)malloc(sizeof(int) * (size_t)(B->off[ncell] ? B->off[ncell] : 1));
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)ncell);
    memcpy(fill, B->off, sizeof(int64_t) * (size_t)ncell);
    for (int64_t t = 0; t < ntris; ++t)
        for (int k = box[6 * t + 2]; k <= box[6 * t + 5]; ++k)
            for (int j = box[6 * t + 1]; j <= box[6 * t + 4]; ++j)
                for (int i = box[6 * t]; i <= box[6 * t + 3]; ++i)
                    B->list[fill[((int64_t)k * ny + j) * nx + i]++] = (int)t;
    free(fill);
    free(box);
}

typedef struct ring_ctx {
    const orc_grid* g;
    const xyz_buckets* B;
    const double* tp; /* 9 doubles per triangle */
    int* seen;
    int stamp;
    double best;
    const double* p;
    int any;
} ring_ctx;

static void visit_cell(ring_ctx* c, int i, int j, int k) {
    const orc_grid* g = c->g;
    if (i < 0 || i >= g->nx || j < 0 || j >= g->ny || k < 0 || k >= g->nz) return;
    c->any = 1;
    int64_t cell = ((int64_t)k * g->ny + j) * g->nx + i;
    for (int64_t e = c->B->off[cell]; e < c->B->off[cell + 1]; ++e) {
        int t = c->B->list[e];
        if (c->seen[t] == c->stamp) continue;
        c->seen[t] = c->stamp;
        const double* q = c->tp + 9 * (int64_t)t;
        double d = orc_point_tri_dist2(c->p, q, q + 3, q + 6, NULL);
        if (d < c->best) c->best = d;
    }
}

/* Chebyshev shell of radius r (for_shell, voxelize.cpp:282-293). */
static void visit_shell(ring_ctx* c, int ci, int cj, int ck, int r) {
    if (r == 0) { visit_cell(c, ci, cj, ck); return; }
    for (int s = -r; s <= r; s += 2 * r)
        for (int dj = -r; dj <= r; ++dj)
            for (int di = -r; di <= r; ++di) visit_cell(c, ci + di, cj + dj, ck + s);
    for (int s = -r; s <= r; s += 2 * r)
        for (int dk = -r + 1; dk <= r - 1; ++dk)
            for (int di = -r; di <= r; ++di) visit_cell(c, ci + di, cj + s, ck + dk);
    for (int s = -r; s <= r; s += 2 * r)
        for (int dk = -r + 1; dk <= r - 1; ++dk)
            for (int dj = -r + 1; dj <= r - 1; ++dj) visit_cell(c, ci + s, cj + dj, ck + dk);
}

/* nearest_tri_dist2 (voxelize.cpp:299-326). */
static double ring_nearest(ring_ctx* c, const int* ijk) {
    const orc_grid* g = c->g;
    c->best = DBL_MAX;
    const int max_r = g->nx + g->ny + g->nz;
    for (int r = 0; r <= max_r; ++r) {
        double ring_min = (r - 1) * g->spacing;
        if (r > 0 && c->best != DBL_MAX && ring_min * ring_min >= c->best) break;
        c->any = 0;
        visit_shell(c, ijk[0], ijk[1], ijk[2], r);
        if (!c->any && c->best != DBL_MAX) break;
    }
    return c->best;
}

static double* tri_points(const double* pts, const int* tris, int64_t ntris) {
    double* tp = (double*)malloc(sizeof(double) * 9 * (size_t)(ntris ? ntris : 1));
    for (int64_t t = 0; t < ntris; ++t)
        for (int v = 0; v < 3; ++v)
            for (int a = 0; a < 3; ++a)
                tp[9 * t + 3 * v + a] = pts[3 * (int64_t)tris[3 * t + v] + a];
    return tp;
}

static double now_seconds(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* times (nullable): [0] the bucket build, [1] the queries, in seconds. */
static void ring_run(const double* pts, const int* tris, int64_t ntris,
                     const orc_grid* g, const int64_t* vox, int64_t nq, double* d2out,
                     const uint8_t* occ, double* sdf64, float* sdf32, int nthreads,
                     double* times) {
    (void)nthreads;
    double t0 = now_seconds();
    xyz_buckets B;
    build_xyz(pts, tris, ntris, g, &B);
    double* tp = tri_points(pts, tris, ntris);
    double t1 = now_seconds();
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
        int* seen = (int*)malloc(sizeof(int) * (size_t)(ntris ? ntris : 1));
        for (int64_t t = 0; t < ntris; ++t) seen[t] = -1;
        ring_ctx c = {g, &B, tp, seen, 0, DBL_MAX, NULL, 0};
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
        for (int64_t q = 0; q < nq; ++q) {
            int64_t idx = vox ? vox[q] : q;
            double p[3];
            int ijk[3];
            voxel_center(g, idx, p, ijk);
            c.p = p;
            c.stamp++;
            double best = ring_nearest(&c, ijk);
            if (d2out) d2out[q] = best;
            if (sdf64 || sdf32) {
                double d = sqrt(best);
                double s = occ[idx] ? -d : d;
                if (sdf64) sdf64[idx] = s;
                if (sdf32) sdf32[idx] = (float)s;
            }
        }
        free(seen);
    }
    if (times) {
        times[0] = t1 - t0;
        times[1] = now_seconds() - t1;
    }
    free(tp);
    free(B.off);
    free(B.list);
}

void orc_sdf_ring(const double* pts, const int* tris, int64_t ntris,
                  const orc_grid* g, const uint8_t* occ, double* sdf64, float* sdf32,
                  int nthreads) {
    int64_t n = (int64_t)g->nx * g->ny * g->nz;
    ring_run(pts, tris, ntris, g, NULL, n, NULL, occ, sdf64, sdf32, nthreads, NULL);
}

void orc_sdf_ring_sample(const double* pts, const int* tris, int64_t ntris,
                         const orc_grid* g, const int64_t* vox, int64_t nq,
                         double* d2, int nthreads, double* times) {
    ring_run(pts, tris, ntris, g, vox, nq, d2, NULL, NULL, NULL, nthreads, times);
}

void orc_dist2_points(const double* pts, const int* tris, int64_t ntris,
                      const double* q, int64_t nq, double* d2, int* tri, int nthreads) {
    (void)nthreads;
    double* tp = tri_points(pts, tris, ntris);
    ORC_PAR_FOR(nthreads)
    for (int64_t s = 0; s < nq; ++s) {
        double best = DBL_MAX;
        int bt = -1;
        for (int64_t t = 0; t < ntris; ++t) {
            const double* v = tp + 9 * t;
            double d = orc_point_tri_dist2(q + 3 * s, v, v + 3, v + 6, NULL);
            if (d < best) { best = d; bt = (int)t; }
        }
        d2[s] = best;
        if (tri) tri[s] = bt;
    }
    free(tp);
}

void orc_sdf_brute(const double* pts, const int* tris, int64_t ntris,
                   const orc_grid* g, const int64_t* vox, int64_t nq, double* d2,
                   int* tri, int* region, int nthreads) {
    (void)nthreads;
    double* tp = tri_points(pts, tris, ntris);
    ORC_PAR_FOR(nthreads)
    for (int64_t s = 0; s < nq; ++s) {
        double p[3];
        voxel_center(g, vox ? vox[s] : s, p, NULL);
        double best = DBL_MAX;
        int bt = -1, br = -1;
        for (int64_t t = 0; t < ntris; ++t) {
            const double* v = tp + 9 * t;
            int r;
            double d = orc_point_tri_dist2(p, v, v + 3, v + 6, &r);
            if (d < best) { best = d; bt = (int)t; br = r; }
        }
        d2[s] = best;
        if (tri) tri[s] = bt;
        if (region) region[s] = br;
    }
    free(tp);
}

/* ========================================================================== */
/* Analytic gradient (envelope theorem on the Ericson closest point).         */
/* ========================================================================== */

/* Closest point barycentrics (la, lb, lc) for the region the Ericson walk picks. */
static void closest_bary(const double* p, const double* a, const double* b,
                         const double* c, double* lam) {
    int r;
    orc_point_tri_dist2(p, a, b, c, &r);
    double ab[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    double ac[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    double ap[3] = {p[0] - a[0], p[1] - a[1], p[2] - a[2]};
    double bp[3] = {p[0] - b[0], p[1] - b[1], p[2] - b[2]};
    double cp[3] = {p[0] - c[0], p[1] - c[1], p[2] - c[2]};
    double d1 = dot3(ab, ap), d2 = dot3(ac, ap);
    double d3 = dot3(ab, bp), d4 = dot3(ac, bp);
    double d5 = dot3(ab, cp), d6 = dot3(ac, cp);
    lam[0] = lam[1] = lam[2] = 0;
    switch (r) {
    case 0: lam[0] = 1; break;
    case 1: lam[1] = 1; break;
    case 2: { double v = d1 / (d1 - d3); lam[0] = 1 - v; lam[1] = v; break; }
    case 3: lam[2] = 1; break;
    case 4: { double w = d2 / (d2 - d6); lam[0] = 1 - w; lam[2] = w; break; }
    case 5: { double w = (d4 - d3) / ((d4 - d3) + (d5 - d6)); lam[1] = 1 - w; lam[2] = w; break; }
    default: {
        double vc = d1 * d4 - d3 * d2, vb = d5 * d2 - d1 * d6, va = d3 * d6 - d5 * d4;
        double den = 1.0 / (va + vb + vc);
        double v = vb * den, w = vc * den;
        lam[0] = 1 - v - w; lam[1] = v; lam[2] = w;
    }
    }
}

void orc_sdf_grad(const double* pts, int64_t npts, const int* tris,
                  const orc_grid* g, const uint8_t* occ, const int* tri,
                  const double* w, const double* t, double* grad) {
    memset(grad, 0, sizeof(double) * 3 * (size_t)npts);
    int64_t n = (int64_t)g->nx * g->ny * g->nz;
    for (int64_t v = 0; v < n; ++v) {
        int ti = tri[v];
        if (ti < 0) continue;
        double p[3];
        voxel_center(g, v, p, NULL);
        const int* T = tris + 3 * (int64_t)ti;
        const double* A = pts + 3 * (int64_t)T[0];
        const double* B = pts + 3 * (int64_t)T[1];
        const double* C = pts + 3 * (int64_t)T[2];
        double lam[3];
        closest_bary(p, A, B, C, lam);
        double q[3];
        for (int a = 0; a < 3; ++a) q[a] = lam[0] * A[a] + lam[1] * B[a] + lam[2] * C[a];
        double d = sqrt(orc_point_tri_dist2(p, A, B, C, NULL));
        if (!(d > 0)) continue;
        double s = occ[v] ? -1.0 : 1.0;
        double dLdd = 2.0 * w[v] * (s * d - t[v]) * s;
        for (int k = 0; k < 3; ++k)
            for (int a = 0; a < 3; ++a)
                grad[3 * (int64_t)T[k] + a] += dLdd * (-lam[k] * (p[a] - q[a]) / d);
    }
}

/* ------------------------------------------------------------------ self-intersections
 * Restatement of src/detect/self_intersection.cpp: every pair of fan triangles i < j
 * that share no vertex index is tested with the Guigue-Devillers orientation test
 * (O. Devillers, P. Guigue, "Faster Triangle-Triangle Intersection Tests", INRIA
 * RR-4488, 2002), every decision a sign of the reference's robust::orient3d (the
 * rounded determinant unless it is exactly zero, then the exact sign); coplanar pairs
 * count as not crossing (:20-103, :110-188). */
static int o3s(const double* a, const double* b, const double* c, const double* d) {
    return orc_orient3d_sign(a, b, c, d, ORC_COMPAT);
}

/* The two intersection intervals on the line of the planes overlap. */
static int gd_interval(const double* p1, const double* q1, const double* r1, const double* p2,
                       const double* q2, const double* r2) {
    if (o3s(q2, p2, p1, q1) > 0) return 0;
    if (o3s(r2, p2, r1, p1) > 0) return 0;
    return 1;
}

/* Triangle 2's vertex signs (s_p, s_q, s_r) with respect to triangle 1's plane; both
 * triangles already rotated so that p1 is alone on its side of plane 2. */
static int gd_core(const double* p1, const double* q1, const double* r1, const double* p2,
                   const double* q2, const double* r2, int sp, int sq, int sr) {
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
    return 0; /* coplanar */
}

int orc_tri_tri_cross(const double* p1, const double* q1, const double* r1, const double* p2,
                      const double* q2, const double* r2) {
    const int a = o3s(p1, p2, q2, r2), b = o3s(q1, p2, q2, r2), c = o3s(r1, p2, q2, r2);
    if (a * b > 0 && a * c > 0) return 0;
    const int d = o3s(p2, q1, r1, p1), e = o3s(q2, q1, r1, p1), f = o3s(r2, q1, r1, p1);
    if (d * e > 0 && d * f > 0) return 0;
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
    return 0; /* coplanar */
}

int64_t orc_self_intersections(const double* pts, int64_t npts, const int* tris, int64_t ntris,
                               int64_t* out_pairs, int64_t cap) {
    int64_t n = 0;
    for (int64_t i = 0; i < ntris; ++i) {
        const int* A = tris + 3 * i;
        if (A[0] < 0 || A[0] >= npts || A[1] < 0 || A[1] >= npts || A[2] < 0 || A[2] >= npts) continue;
        for (int64_t j = i + 1; j < ntris; ++j) {
            const int* B = tris + 3 * j;
            int shared = 0;
            for (int x = 0; x < 3; ++x)
                for (int y = 0; y < 3; ++y) shared |= A[x] == B[y];
            if (shared) continue;
            if (B[0] < 0 || B[0] >= npts || B[1] < 0 || B[1] >= npts || B[2] < 0 || B[2] >= npts) continue;
            if (orc_tri_tri_cross(pts + 3 * A[0], pts + 3 * A[1], pts + 3 * A[2], pts + 3 * B[0],
                                  pts + 3 * B[1], pts + 3 * B[2])) {
                if (n < cap) {
                    out_pairs[2 * n] = i;
                    out_pairs[2 * n + 1] = j;
                }
                ++n;
            }
        }
    }
    return n;
}
