/* sizing_oracle.c — CPU restatement of the reference's background sizing field
 * (src/sizing/background.cpp) and of the orient3d VALUE it interpolates with
 * (src/predicates/robust.cpp:36-42 over src/predicates/predicates.cpp), test
 * infrastructure only.
 *
 * orient3d value. The reference initialises the predicates with a zero static filter
 * (robust.cpp:28-34, predicates.cpp:626-645), so robust::orient3d returns the rounded
 * determinant (predicates.cpp:2194-2245, this operation order) whenever it is not
 * zero; a zero goes to the adaptive routine (:1778-2178), whose answer is, in order:
 * the estimate of the exact determinant of the rounded coordinate differences when it
 * clears errbound B; that estimate when every difference was exact; the estimate plus
 * the first-order tail correction when it clears errbound C; else the largest
 * component of the exact expansion. Which of these values comes back depends on the
 * exact sequence of expansion operations, so the sequence (Shewchuk's published
 * algorithm: Two-Sum, Two-Diff, Dekker's Two-Product with splitter 2^27 + 1,
 * zero-eliminating expansion sum and scale, the tail products) is followed here in
 * code of its own.
 *
 * Sizing (background.cpp:29-74): for a query p, the first tetrahedron (in order) whose
 * determinant value D is not zero and whose four weights orient3d(...)/D (p in place
 * of vertex i) are all >= -1e-9 gives (w0 s0 + w1 s1 + w2 s2 + w3 s3) * scale; else the
 * size of the nearest node (first index among equal squared distances, from
 * DBL_MAX), times scale; node sizes padded with 0 or truncated to the node count.
 *
 * Used only by tests/, the fixture generator and bench.py's CPU legs, as the checker
 * and the timed CPU baseline; never by the product path. */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "cmg_oracle.h"

#define EPS_D 1.1102230246251565e-16 /* 2^-53 */
#define SPLITTER 134217729.0          /* 2^27 + 1 */

static const double kErrB = (3.0 + 28.0 * EPS_D) * EPS_D;
static const double kErrC = (26.0 + 288.0 * EPS_D) * EPS_D * EPS_D;
static const double kResult = (3.0 + 8.0 * EPS_D) * EPS_D;
static const double kErrA = (7.0 + 56.0 * EPS_D) * EPS_D;

static void s_two_sum(double a, double b, double* x, double* y) {
    double s = a + b, bv = s - a, av = s - bv;
    *x = s;
    *y = (a - av) + (b - bv);
}
static void s_fast_two_sum(double a, double b, double* x, double* y) {
    double s = a + b;
    *x = s;
    *y = b - (s - a);
}
static double s_diff_tail(double a, double b, double x) {
    double bv = a - x, av = x + bv;
    return (a - av) + (bv - b);
}
static void s_two_diff(double a, double b, double* x, double* y) {
    double d = a - b;
    *x = d;
    *y = s_diff_tail(a, b, d);
}
static void s_split(double a, double* hi, double* lo) {
    double c = SPLITTER * a, big = c - a;
    *hi = c - big;
    *lo = a - *hi;
}
static void s_prod_presplit(double a, double b, double bhi, double blo, double* x, double* y) {
    double p = a * b, ahi, alo;
    s_split(a, &ahi, &alo);
    double e1 = p - ahi * bhi, e2 = e1 - alo * bhi, e3 = e2 - ahi * blo;
    *x = p;
    *y = alo * blo - e3;
}
static void s_two_prod(double a, double b, double* x, double* y) {
    double bhi, blo;
    s_split(b, &bhi, &blo);
    s_prod_presplit(a, b, bhi, blo, x, y);
}
/* (a1, a0) - b -> x[2..0] */
static void s_two_one_diff(double a1, double a0, double b, double* x2, double* x1, double* x0) {
    double i;
    s_two_diff(a0, b, &i, x0);
    s_two_sum(a1, i, x2, x1);
}
/* (a1, a0) - (b1, b0) -> x[0..3], x[3] the largest */
static void s_two_two_diff(double a1, double a0, double b1, double b0, double* x) {
    double j, z;
    s_two_one_diff(a1, a0, b0, &j, &z, &x[0]);
    s_two_one_diff(j, z, b1, &x[3], &x[2], &x[1]);
}
/* (a1, a0) * b -> x[0..3] */
static void s_two_one_prod(double a1, double a0, double b, double* x) {
    double bhi, blo, i, j, z, k;
    s_split(b, &bhi, &blo);
    s_prod_presplit(a0, b, bhi, blo, &i, &x[0]);
    s_prod_presplit(a1, b, bhi, blo, &j, &z);
    s_two_sum(i, z, &k, &x[1]);
    s_fast_two_sum(j, k, &x[3], &x[2]);
}
/* the smaller-magnitude head first: f is taken when (f > e) != (f > -e) */
static int s_take_e(double e, double f) { return (f > e) == (f > -e); }

static int s_sum(int elen, const double* e, int flen, const double* f, double* h) {
    int ei = 0, fi = 0, hi = 0;
    double en = e[0], fn = f[0], q, qn, hh;
    if (s_take_e(en, fn)) {
        q = en;
        en = ++ei < elen ? e[ei] : 0.0;
    } else {
        q = fn;
        fn = ++fi < flen ? f[fi] : 0.0;
    }
    if (ei < elen && fi < flen) {
        if (s_take_e(en, fn)) {
            s_fast_two_sum(en, q, &qn, &hh);
            en = ++ei < elen ? e[ei] : 0.0;
        } else {
            s_fast_two_sum(fn, q, &qn, &hh);
            fn = ++fi < flen ? f[fi] : 0.0;
        }
        q = qn;
        if (hh != 0.0) h[hi++] = hh;
        while (ei < elen && fi < flen) {
            if (s_take_e(en, fn)) {
                s_two_sum(q, en, &qn, &hh);
                en = ++ei < elen ? e[ei] : 0.0;
            } else {
                s_two_sum(q, fn, &qn, &hh);
                fn = ++fi < flen ? f[fi] : 0.0;
            }
            q = qn;
            if (hh != 0.0) h[hi++] = hh;
        }
    }
    while (ei < elen) {
        s_two_sum(q, en, &qn, &hh);
        en = ++ei < elen ? e[ei] : 0.0;
        q = qn;
        if (hh != 0.0) h[hi++] = hh;
    }
    while (fi < flen) {
        s_two_sum(q, fn, &qn, &hh);
        fn = ++fi < flen ? f[fi] : 0.0;
        q = qn;
        if (hh != 0.0) h[hi++] = hh;
    }
    if (q != 0.0 || hi == 0) h[hi++] = q;
    return hi;
}

static int s_scale(int elen, const double* e, double b, double* h) {
    double bhi, blo, q, hh, p1, p0, sum;
    int hi = 0;
    s_split(b, &bhi, &blo);
    s_prod_presplit(e[0], b, bhi, blo, &q, &hh);
    if (hh != 0.0) h[hi++] = hh;
    for (int i = 1; i < elen; ++i) {
        s_prod_presplit(e[i], b, bhi, blo, &p1, &p0);
        s_two_sum(q, p0, &sum, &hh);
        if (hh != 0.0) h[hi++] = hh;
        s_fast_two_sum(p1, sum, &q, &hh);
        if (hh != 0.0) h[hi++] = hh;
    }
    if (q != 0.0 || hi == 0) h[hi++] = q;
    return hi;
}

static double s_estimate(int n, const double* e) {
    double q = e[0];
    for (int i = 1; i < n; ++i) q += e[i];
    return q;
}

/* The two tail products of one point in the exact stage: (tx, ty) its x / y
 * difference tails, p and q the rounded differences of the next two points in the
 * roles the reference gives them; each product as 1, 2 or 4 components, built the
 * cheaper way when a tail is zero. */
static int s_tail_pair(double tx, double ty, double p_x, double p_y, double q_x, double q_y,
                       double* first, int* n1, double* second, int* n2) {
    /* first  = tx * p_y - ty * p_x
     * second = ty * q_x - tx * q_y */
    if (tx == 0.0) {
        if (ty == 0.0) {
            first[0] = 0.0;
            *n1 = 1;
            second[0] = 0.0;
            *n2 = 1;
        } else {
            s_two_prod(-ty, p_x, &first[1], &first[0]);
            *n1 = 2;
            s_two_prod(ty, q_x, &second[1], &second[0]);
            *n2 = 2;
        }
    } else {
        if (ty == 0.0) {
            s_two_prod(tx, p_y, &first[1], &first[0]);
            *n1 = 2;
            s_two_prod(-tx, q_y, &second[1], &second[0]);
            *n2 = 2;
        } else {
            double a1, a0, b1, b0;
            s_two_prod(tx, p_y, &a1, &a0);
            s_two_prod(ty, p_x, &b1, &b0);
            s_two_two_diff(a1, a0, b1, b0, first);
            *n1 = 4;
            s_two_prod(ty, q_x, &a1, &a0);
            s_two_prod(tx, q_y, &b1, &b0);
            s_two_two_diff(a1, a0, b1, b0, second);
            *n2 = 4;
        }
    }
    return 0;
}

/* fin <- fin + e (ping-pong buffers) */
static int s_acc(int n, double** fin, double** other, int elen, const double* e) {
    int m = s_sum(n, *fin, elen, e, *other);
    double* t = *fin;
    *fin = *other;
    *other = t;
    return m;
}

static double orient3d_adapt(const double* pa, const double* pb, const double* pc, const double* pd,
                             double permanent) {
    const double adx = pa[0] - pd[0], bdx = pb[0] - pd[0], cdx = pc[0] - pd[0];
    const double ady = pa[1] - pd[1], bdy = pb[1] - pd[1], cdy = pc[1] - pd[1];
    const double adz = pa[2] - pd[2], bdz = pb[2] - pd[2], cdz = pc[2] - pd[2];
    double bc[4], ca[4], ab[4], adet[8], bdet[8], cdet[8], abdet[16];
    double fin1[192], fin2[192];
    double x1, x0, y1, y0;

    s_two_prod(bdx, cdy, &x1, &x0);
    s_two_prod(cdx, bdy, &y1, &y0);
    s_two_two_diff(x1, x0, y1, y0, bc);
    int alen = s_scale(4, bc, adz, adet);
    s_two_prod(cdx, ady, &x1, &x0);
    s_two_prod(adx, cdy, &y1, &y0);
    s_two_two_diff(x1, x0, y1, y0, ca);
    int blen = s_scale(4, ca, bdz, bdet);
    s_two_prod(adx, bdy, &x1, &x0);
    s_two_prod(bdx, ady, &y1, &y0);
    s_two_two_diff(x1, x0, y1, y0, ab);
    int clen = s_scale(4, ab, cdz, cdet);
    int ablen = s_sum(alen, adet, blen, bdet, abdet);
    int n = s_sum(ablen, abdet, clen, cdet, fin1);

    double det = s_estimate(n, fin1);
    double bound = kErrB * permanent;
    if (det >= bound || -det >= bound) return det;

    const double adxt = s_diff_tail(pa[0], pd[0], adx), bdxt = s_diff_tail(pb[0], pd[0], bdx),
                 cdxt = s_diff_tail(pc[0], pd[0], cdx), adyt = s_diff_tail(pa[1], pd[1], ady),
                 bdyt = s_diff_tail(pb[1], pd[1], bdy), cdyt = s_diff_tail(pc[1], pd[1], cdy),
                 adzt = s_diff_tail(pa[2], pd[2], adz), bdzt = s_diff_tail(pb[2], pd[2], bdz),
                 cdzt = s_diff_tail(pc[2], pd[2], cdz);
    if (adxt == 0.0 && bdxt == 0.0 && cdxt == 0.0 && adyt == 0.0 && bdyt == 0.0 && cdyt == 0.0 &&
        adzt == 0.0 && bdzt == 0.0 && cdzt == 0.0)
        return det;

    bound = kErrC * permanent + kResult * fabs(det);
    det += (adz * ((bdx * cdyt + cdy * bdxt) - (bdy * cdxt + cdx * bdyt)) +
            adzt * (bdx * cdy - bdy * cdx)) +
           (bdz * ((cdx * adyt + ady * cdxt) - (cdy * adxt + adx * cdyt)) +
            bdzt * (cdx * ady - cdy * adx)) +
           (cdz * ((adx * bdyt + bdy * adxt) - (ady * bdxt + bdx * adyt)) +
            cdzt * (adx * bdy - ady * bdx));
    if (det >= bound || -det >= bound) return det;

    double *fin = fin1, *other = fin2;
    double at_b[4], at_c[4], bt_c[4], bt_a[4], ct_a[4], ct_b[4];
    int at_bn, at_cn, bt_cn, bt_an, ct_an, ct_bn;
    /* a's tails against b (at_b = adxt*bdy - adyt*bdx) and c (at_c = adyt*cdx - adxt*cdy) */
    s_tail_pair(adxt, adyt, bdx, bdy, cdx, cdy, at_b, &at_bn, at_c, &at_cn);
    s_tail_pair(bdxt, bdyt, cdx, cdy, adx, ady, bt_c, &bt_cn, bt_a, &bt_an);
    s_tail_pair(cdxt, cdyt, adx, ady, bdx, bdy, ct_a, &ct_an, ct_b, &ct_bn);

    double bct[8], cat[8], abt[8], w[16], v[12], u[4];
    int bctn = s_sum(bt_cn, bt_c, ct_bn, ct_b, bct);
    int wn = s_scale(bctn, bct, adz, w);
    n = s_acc(n, &fin, &other, wn, w);
    int catn = s_sum(ct_an, ct_a, at_cn, at_c, cat);
    wn = s_scale(catn, cat, bdz, w);
    n = s_acc(n, &fin, &other, wn, w);
    int abtn = s_sum(at_bn, at_b, bt_an, bt_a, abt);
    wn = s_scale(abtn, abt, cdz, w);
    n = s_acc(n, &fin, &other, wn, w);

    if (adzt != 0.0) n = s_acc(n, &fin, &other, s_scale(4, bc, adzt, v), v);
    if (bdzt != 0.0) n = s_acc(n, &fin, &other, s_scale(4, ca, bdzt, v), v);
    if (cdzt != 0.0) n = s_acc(n, &fin, &other, s_scale(4, ab, cdzt, v), v);

    /* tail x tail products, each scaled by the third point's z difference and its tail */
    const double tx[3] = {adxt, bdxt, cdxt};
    const double ty_next[3] = {bdyt, cdyt, adyt}; /* b after a, c after b, a after c */
    const double ty_prev[3] = {cdyt, adyt, bdyt};
    const double zd_third[3] = {cdz, adz, bdz}, zt_third[3] = {cdzt, adzt, bdzt};
    const double zd_mid[3] = {bdz, cdz, adz}, zt_mid[3] = {bdzt, cdzt, adzt};
    for (int k = 0; k < 3; ++k) {
        if (tx[k] == 0.0) continue;
        if (ty_next[k] != 0.0) {
            double p1, p0;
            s_two_prod(tx[k], ty_next[k], &p1, &p0);
            s_two_one_prod(p1, p0, zd_third[k], u);
            n = s_acc(n, &fin, &other, 4, u);
            if (zt_third[k] != 0.0) {
                s_two_one_prod(p1, p0, zt_third[k], u);
                n = s_acc(n, &fin, &other, 4, u);
            }
        }
        if (ty_prev[k] != 0.0) {
            double p1, p0;
            s_two_prod(-tx[k], ty_prev[k], &p1, &p0);
            s_two_one_prod(p1, p0, zd_mid[k], u);
            n = s_acc(n, &fin, &other, 4, u);
            if (zt_mid[k] != 0.0) {
                s_two_one_prod(p1, p0, zt_mid[k], u);
                n = s_acc(n, &fin, &other, 4, u);
            }
        }
    }

    if (adzt != 0.0) n = s_acc(n, &fin, &other, s_scale(bctn, bct, adzt, w), w);
    if (bdzt != 0.0) n = s_acc(n, &fin, &other, s_scale(catn, cat, bdzt, w), w);
    if (cdzt != 0.0) n = s_acc(n, &fin, &other, s_scale(abtn, abt, cdzt, w), w);
    return fin[n - 1];
}

double orc_orient3d_value(const double* pa, const double* pb, const double* pc, const double* pd) {
    const double adx = pa[0] - pd[0], ady = pa[1] - pd[1], adz = pa[2] - pd[2];
    const double bdx = pb[0] - pd[0], bdy = pb[1] - pd[1], bdz = pb[2] - pd[2];
    const double cdx = pc[0] - pd[0], cdy = pc[1] - pd[1], cdz = pc[2] - pd[2];
    const double bdxcdy = bdx * cdy, cdxbdy = cdx * bdy;
    const double cdxady = cdx * ady, adxcdy = adx * cdy;
    const double adxbdy = adx * bdy, bdxady = bdx * ady;
    const double det = adz * (bdxcdy - cdxbdy) + bdz * (cdxady - adxcdy) + cdz * (adxbdy - bdxady);
    if (det > 0.0 || det < 0.0) return det; /* the zero static filter */
    const double permanent = (fabs(bdxcdy) + fabs(cdxbdy)) * fabs(adz) +
                             (fabs(cdxady) + fabs(adxcdy)) * fabs(bdz) +
                             (fabs(adxbdy) + fabs(bdxady)) * fabs(cdz);
    const double bound = kErrA * permanent;
    if (det > bound || -det > bound) return det;
    return orient3d_adapt(pa, pb, pc, pd, permanent);
}

void orc_orient3d_values(const double* const* s, int64_t n, double* out) {
    for (int64_t i = 0; i < n; ++i) {
        const double a[3] = {s[0][i], s[1][i], s[2][i]}, b[3] = {s[3][i], s[4][i], s[5][i]};
        const double c[3] = {s[6][i], s[7][i], s[8][i]}, d[3] = {s[9][i], s[10][i], s[11][i]};
        out[i] = orc_orient3d_value(a, b, c, d);
    }
}

/* ---------------------------------------------------------------- sizing */

static int interp_in_tet(const double* P, const int* t, const double* S, const double* p,
                         double* out) {
    const double *v0 = P + 3 * (int64_t)t[0], *v1 = P + 3 * (int64_t)t[1],
                 *v2 = P + 3 * (int64_t)t[2], *v3 = P + 3 * (int64_t)t[3];
    const double D = orc_orient3d_value(v0, v1, v2, v3);
    if (D == 0.0) return 0;
    const double w0 = orc_orient3d_value(p, v1, v2, v3) / D;
    const double w1 = orc_orient3d_value(v0, p, v2, v3) / D;
    const double w2 = orc_orient3d_value(v0, v1, p, v3) / D;
    const double w3 = orc_orient3d_value(v0, v1, v2, p) / D;
    const double eps = -1e-9;
    if (w0 < eps || w1 < eps || w2 < eps || w3 < eps) return 0;
    *out = w0 * S[t[0]] + w1 * S[t[1]] + w2 * S[t[2]] + w3 * S[t[3]];
    return 1;
}

/* One query: the tetrahedron index that answered (or -1 for the nearest node), the
 * size in *out. */
static int64_t sizing_one(const double* P, int64_t np, const int* T, int64_t nt, const double* S,
                          double scale, const double* p, double* out) {
    double s;
    for (int64_t t = 0; t < nt; ++t)
        if (interp_in_tet(P, T + 4 * t, S, p, &s)) {
            *out = s * scale;
            return t;
        }
    double best = DBL_MAX;
    int64_t bi = 0;
    for (int64_t i = 0; i < np; ++i) {
        const double dx = P[3 * i] - p[0], dy = P[3 * i + 1] - p[1], dz = P[3 * i + 2] - p[2];
        const double d = dx * dx + dy * dy + dz * dz;
        if (d < best) {
            best = d;
            bi = i;
        }
    }
    *out = (np == 0 ? 0.0 : S[bi]) * scale;
    return -1;
}

/* sizes: node sizes already padded / truncated to np entries. which (may be NULL):
 * per query, the answering tetrahedron or -1. */
void orc_sizing_eval(const double* P, int64_t np, const int* T, int64_t nt, const double* S,
                     double scale, const double* Q, int64_t nq, double* out, int64_t* which,
                     int nthreads) {
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads > 0 ? nthreads : 1)
    for (int64_t q = 0; q < nq; ++q) {
        const int64_t w = sizing_one(P, np, T, nt, S, scale, Q + 3 * q, out + q);
        if (which) which[q] = w;
    }
}
