/*
 * ves_oracle.c -- CPU restatement of the reference batched eigensolver path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker for the CUDA product and the
 * CPU baseline ("port") timed beside it.  The product never links or calls
 * this file.
 *
 * Every routine restates one reference routine of kipfstuhl/vectorized-eigensolver
 * step for step (cited per function), on the same structure-of-arrays layout,
 * with one matrix per OpenMP iteration exactly as the reference's CPU build
 * (`#pragma omp parallel for schedule(static, 8)` over blocks, Toolbox.hpp:1990).
 * Indices below are 1-based, as in the reference and LAPACK, through the
 * M_(i,j) / V_(i) accessors; `s` is the interleave stride (thread_cnt).
 *
 * Deliberate differences from the shipped reference (all documented in the
 * parity tests):
 *   - vo_eigensolver clears H(i,j), i >= j+2, between zunghr and zlahqr: the
 *     shipped eigensolver() feeds the reflector storage into the QR sweep and
 *     returns wrong eigenvalues (defect B1; LAPACK zlahqr clears it itself).
 *   - ztrevc does not rescale a column of T by its max-norm (Toolbox.hpp:1278-1295,
 *     defect B2).  That scaling never feeds back into the eigenvectors, so V is
 *     identical; T is left intact instead of partly rescaled.
 *   - zgemv's Hermitian branch reads imag(y) where the reference reads real(y)
 *     (Toolbox.hpp:1125, defect B3).  The solver path calls it with beta = 0,
 *     where both agree.
 * Everything else -- including the reference's reflector sign in zgehrd
 * (Toolbox.hpp:1368), its deflation test reading imag(H(K+1,K)) (:840), the
 * absent search for a second small subdiagonal and the 31-iteration cap per
 * eigenvalue (:808) -- is restated as shipped.
 */
#include "ves_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------- */
/* Complex scalar helpers on split (re, im) doubles: the semantics of          */
/* ComplexDouble.hpp:283-488 (Smith division, plain-sqrt modulus).            */
/* ------------------------------------------------------------------------- */

typedef struct { double r, i; } cplx;

static inline cplx cmk(double r, double i) { cplx z; z.r = r; z.i = i; return z; }
static inline double cabs1_(cplx z) { return fabs(z.r) + fabs(z.i); }
static inline double cabs_(cplx z) { return sqrt(z.r * z.r + z.i * z.i); }
static inline cplx cmul_(cplx a, cplx b) { return cmk(a.r * b.r - a.i * b.i, a.i * b.r + a.r * b.i); }
/* a * conj(b) */
static inline cplx cmulc_(cplx a, cplx b) { return cmk(a.r * b.r + a.i * b.i, a.i * b.r - a.r * b.i); }
static inline cplx cadd_(cplx a, cplx b) { return cmk(a.r + b.r, a.i + b.i); }
static inline cplx csub_(cplx a, cplx b) { return cmk(a.r - b.r, a.i - b.i); }
static inline cplx cscal_(cplx a, double d) { return cmk(a.r * d, a.i * d); }
static inline cplx cdivr_(cplx a, double d) { return cmk(a.r / d, a.i / d); }

/* 1/z by Smith's method (ComplexDouble.hpp:283-318). */
static inline cplx cinv_(cplx z)
{
    if (fabs(z.r) <= fabs(z.i)) {
        double ratio = z.r / z.i;
        double den = z.i * (1.0 + ratio * ratio);
        return cmk(ratio / den, -1.0 / den);
    } else {
        double ratio = z.i / z.r;
        double den = z.r * (1.0 + ratio * ratio);
        return cmk(1.0 / den, -ratio / den);
    }
}

/* a/b by Smith's method (ComplexDouble.hpp:320-353). */
static inline cplx cdiv_(cplx a, cplx b)
{
    if (fabs(b.r) <= fabs(b.i)) {
        double ratio = b.r / b.i;
        double den = b.i * (1.0 + ratio * ratio);
        return cmk((a.r * ratio + a.i) / den, (a.i * ratio - a.r) / den);
    } else {
        double ratio = b.i / b.r;
        double den = b.r * (1.0 + ratio * ratio);
        return cmk((a.r + a.i * ratio) / den, (a.i - a.r * ratio) / den);
    }
}

/* Principal square root (ComplexDouble.hpp:451-488). */
static inline cplx csqrt_(cplx z)
{
    double zr = sqrt(0.5 * (cabs_(z) + fabs(z.r)));
    double zi = (zr == 0.0) ? 0.0 : fabs(z.i) / (2.0 * zr);
    cplx w = (z.r < 0.0) ? cmk(zi, zr) : cmk(zr, zi);
    if (z.i < 0.0) w.i = -w.i;
    return w;
}

/* ------------------------------------------------------------------------- */
/* Strided accessors.  A matrix view is (re, im, n, s): element (i,j), 1-based,  */
/* at ((i-1) + (j-1)*n)*s.  A vector view: element i at (i-1)*s.               */
/* ------------------------------------------------------------------------- */

typedef struct { double *r, *i; int n; size_t s; } mview;
typedef struct { double *r, *i; size_t s; } vview;

static inline size_t mix(const mview *m, int i, int j) { return ((size_t)(i - 1) + (size_t)(j - 1) * m->n) * m->s; }
static inline cplx mget(const mview *m, int i, int j) { size_t k = mix(m, i, j); return cmk(m->r[k], m->i[k]); }
static inline void mset(const mview *m, int i, int j, cplx z) { size_t k = mix(m, i, j); m->r[k] = z.r; m->i[k] = z.i; }
static inline cplx vget(const vview *v, int i) { size_t k = (size_t)(i - 1) * v->s; return cmk(v->r[k], v->i[k]); }
static inline void vset(const vview *v, int i, cplx z) { size_t k = (size_t)(i - 1) * v->s; v->r[k] = z.r; v->i[k] = z.i; }

static int g_threads = 0;
void vo_set_threads(int nthreads) { g_threads = nthreads; }
int vo_get_threads(void)
{
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

/* Views of matrix (b, t) of a batch. */
static inline mview batch_mat(double *r, double *i, int dim, int tc, int b, int t)
{
    size_t off = (size_t)b * tc * dim * dim + t;
    mview m; m.r = r + off; m.i = i + off; m.n = dim; m.s = (size_t)tc; return m;
}
static inline vview batch_vec(double *r, double *i, int dim, int tc, int b, int t)
{
    size_t off = (size_t)b * tc * dim + t;
    vview v; v.r = r + off; v.i = i + off; v.s = (size_t)tc; return v;
}

/* ------------------------------------------------------------------------- */
/* zgehrd: unblocked Householder Hessenberg reduction (Toolbox.hpp:1315-1490). */
/* `w` is a length-dim work vector.                                           */
/* ------------------------------------------------------------------------- */
static void zgehrd_one(const mview *A, const vview *tau, cplx *w)
{
    const int n = A->n;
    for (int i = 1; i <= n - 1; ++i) {
        const int m = n - i; /* reflector length, v(1) = 1 at A(i+1,i) */
        cplx alpha = mget(A, i + 1, i);
        double xnorm2 = 0.0;
        for (int k = i + 2; k <= n; ++k) {
            cplx x = mget(A, k, i);
            xnorm2 += x.r * x.r + x.i * x.i;
        }
        /* reflector sign as shipped: beta carries the sign of Re(alpha) (:1368) */
        double beta = copysign(sqrt(alpha.r * alpha.r + alpha.i * alpha.i + xnorm2), alpha.r);
        double rbeta = 1.0 / beta;
        cplx t = cmk((beta - alpha.r) * rbeta, -alpha.i * rbeta);
        cplx scale = cinv_(cmk(alpha.r - beta, alpha.i));
        for (int k = i + 2; k <= n; ++k) mset(A, k, i, cmul_(mget(A, k, i), scale));
        vset(tau, i, t);
        mset(A, i + 1, i, cmk(1.0, 0.0));

        /* A(1:n, i+1:n) := A(1:n, i+1:n) (I - tau v v^H)   (:1405-1441) */
        for (int k = 0; k < n; ++k) w[k] = cmk(0.0, 0.0);
        for (int j = 1; j <= m; ++j) {
            cplx vj = mget(A, i + j, i);
            for (int k = 1; k <= n; ++k) w[k - 1] = cadd_(w[k - 1], cmul_(mget(A, k, i + j), vj));
        }
        for (int j = 1; j <= m; ++j) {
            cplx c = cmulc_(cmk(-t.r, -t.i), mget(A, i + j, i));
            for (int k = 1; k <= n; ++k) mset(A, k, i + j, cadd_(cmul_(w[k - 1], c), mget(A, k, i + j)));
        }

        /* A(i+1:n, i+1:n) := (I - conj(tau) v v^H) A(i+1:n, i+1:n)   (:1448-1481) */
        for (int j = 1; j <= m; ++j) {
            cplx acc = cmk(0.0, 0.0);
            for (int k = 1; k <= m; ++k) acc = cadd_(acc, cmulc_(mget(A, i + k, i), mget(A, i + k, i + j)));
            w[j - 1] = acc;
        }
        for (int j = 1; j <= m; ++j) {
            cplx c = cmulc_(cmk(-t.r, t.i), w[j - 1]);
            for (int k = 1; k <= m; ++k)
                mset(A, i + k, i + j, cadd_(cmul_(mget(A, i + k, i), c), mget(A, i + k, i + j)));
        }
        mset(A, i + 1, i, cmk(beta, 0.0));
    }
}

/* ------------------------------------------------------------------------- */
/* zunghr: Q from the reflectors, shift + zung2r (Toolbox.hpp:1492-1659).      */
/* ------------------------------------------------------------------------- */
static void zunghr_one(const mview *A, const vview *tau, cplx *w)
{
    const int n = A->n;
    for (int j = n; j >= 2; --j) {
        for (int i = 1; i <= j - 1; ++i) mset(A, i, j, cmk(0.0, 0.0));
        for (int i = j + 1; i <= n; ++i) mset(A, i, j, mget(A, i, j - 1));
    }
    for (int i = 1; i <= n; ++i) mset(A, i, 1, cmk(0.0, 0.0));
    mset(A, 1, 1, cmk(1.0, 0.0));

    /* zung2r on the trailing (n-1) x (n-1) block, B(i,j) = A(i+1, j+1) */
    const int nh = n - 1;
    for (int i = nh; i >= 1; --i) {
        const cplx t = vget(tau, i);
        mset(A, i + 1, i + 1, cmk(1.0, 0.0));
        const int lastv = nh - i + 1, lastc = nh - i;
        for (int j = 1; j <= lastc; ++j) {
            cplx acc = cmk(0.0, 0.0);
            for (int k = 1; k <= lastv; ++k) acc = cadd_(acc, cmulc_(mget(A, i + k, i + 1), mget(A, i + k, i + 1 + j)));
            w[j - 1] = acc;
        }
        for (int j = 1; j <= lastc; ++j) {
            cplx c = cmulc_(cmk(-t.r, -t.i), w[j - 1]);
            for (int k = 1; k <= lastv; ++k)
                mset(A, i + k, i + 1 + j, cadd_(cmul_(mget(A, i + k, i + 1), c), mget(A, i + k, i + 1 + j)));
        }
        for (int k = i + 1; k <= nh; ++k) mset(A, k + 1, i + 1, cmul_(mget(A, k + 1, i + 1), cmk(-t.r, -t.i)));
        mset(A, i + 1, i + 1, cmk(1.0 - t.r, -t.i));
        for (int k = 1; k <= i - 1; ++k) mset(A, k + 1, i + 1, cmk(0.0, 0.0));
    }
}

/* ------------------------------------------------------------------------- */
/* One single-shift QR sweep with Schur vectors (Toolbox.hpp:138-369).         */
/* ------------------------------------------------------------------------- */
static void qr_sweep_one(const mview *H, const mview *Z, int I, int M, int I1, int I2, cplx v0, cplx v1)
{
    const int n = H->n;
    const double safmin = DBL_MIN / (DBL_EPSILON * 0.5);
    for (int K = M; K <= I - 1; ++K) {
        if (K > M) {
            v0 = mget(H, K, K - 1);
            v1 = mget(H, K + 1, K - 1);
        }
        /* 2-element zlarfg (:186-241) */
        cplx t1;
        if (v1.r == 0.0 && v1.i == 0.0 && v0.i == 0.0) {
            t1 = cmk(0.0, 0.0);
        } else {
            double norm = sqrt(v0.r * v0.r + v0.i * v0.i + v1.r * v1.r + v1.i * v1.i);
            int knt = 0;
            if (norm < safmin) {
                double rs = 1.0 / safmin;
                do {
                    ++knt;
                    v1 = cscal_(v1, rs);
                    v0 = cscal_(v0, rs);
                    norm *= rs;
                } while (norm < safmin);
                norm = sqrt(v0.r * v0.r + v0.i * v0.i + v1.r * v1.r + v1.i * v1.i);
            }
            double beta = copysign(norm, v0.r);
            cplx z = cmk(v0.r + beta, v0.i);
            t1 = cdivr_(z, beta);
            v1 = cmul_(v1, cinv_(z));
            for (int q = 0; q < knt; ++q) beta *= safmin;
            v0 = cmk(-beta, 0.0);
        }
        if (K > M) {
            mset(H, K, K - 1, v0);
            mset(H, K + 1, K - 1, cmk(0.0, 0.0));
        }
        const double t2 = t1.r * v1.r - t1.i * v1.i;
        /* rows K, K+1, columns K..I2 */
        for (int j = K; j <= I2; ++j) {
            cplx h1 = mget(H, K, j), h2 = mget(H, K + 1, j);
            cplx z = cadd_(cmulc_(h1, t1), cscal_(h2, t2));
            mset(H, K, j, csub_(h1, z));
            mset(H, K + 1, j, csub_(h2, cmul_(z, v1)));
        }
        /* columns K, K+1, rows I1..min(K+2, I) */
        const int jend = (K + 2) < I ? (K + 2) : I;
        for (int j = I1; j <= jend; ++j) {
            cplx h1 = mget(H, j, K), h2 = mget(H, j, K + 1);
            cplx z = cadd_(cmul_(h1, t1), cscal_(h2, t2));
            mset(H, j, K, csub_(h1, z));
            mset(H, j, K + 1, csub_(h2, cmulc_(z, v1)));
        }
        /* Schur vectors, all rows */
        for (int j = 1; j <= n; ++j) {
            cplx z1 = mget(Z, j, K), z2 = mget(Z, j, K + 1);
            cplx z = cadd_(cmul_(z1, t1), cscal_(z2, t2));
            mset(Z, j, K, csub_(z1, z));
            mset(Z, j, K + 1, csub_(z2, cmulc_(z, v1)));
        }
    }
    /* make H(I, I-1) real (:337-367, scale_rc :14-29) */
    cplx h = mget(H, I, I - 1);
    if (h.i != 0.0) {
        double d = cabs_(h);
        cplx z = cdivr_(h, d);
        z.i = -z.i;
        mset(H, I, I - 1, cmk(d, 0.0));
        for (int j = I + 1; j <= I2; ++j) mset(H, I, j, cmul_(mget(H, I, j), z));
        for (int j = I1; j <= I - 1; ++j) mset(H, j, I, cmulc_(mget(H, j, I), z));
        for (int j = 1; j <= n; ++j) mset(Z, j, I, cmulc_(mget(Z, j, I), z));
    }
}

/* ------------------------------------------------------------------------- */
/* zlahqr with wantT = wantZ = true (Toolbox.hpp:690-1031).  Returns sweeps.   */
/* ------------------------------------------------------------------------- */
static int zlahqr_one(const mview *H, const mview *Z, const vview *E)
{
    const int n = H->n;
    const double ulp = DBL_EPSILON;
    const double smlnum = DBL_MIN * ((double)n / ulp);
    int sweeps = 0;

    /* make the subdiagonal real (:735-793) */
    for (int i = 2; i <= n; ++i) {
        cplx h = mget(H, i, i - 1);
        if (h.i != 0.0) {
            cplx sc = cdivr_(h, cabs1_(h));
            double d = cabs_(sc);
            sc = cdivr_(cmk(sc.r, -sc.i), d);
            mset(H, i, i - 1, cmk(cabs_(h), 0.0));
            for (int j = i; j <= n; ++j) mset(H, i, j, cmul_(mget(H, i, j), sc));
            int rend = (i + 1) < n ? (i + 1) : n;
            for (int j = 1; j <= rend; ++j) mset(H, j, i, cmulc_(mget(H, j, i), sc));
            for (int j = 1; j <= n; ++j) mset(Z, j, i, cmulc_(mget(Z, j, i), sc));
        }
    }

    const int I1 = 1, I2 = n;
    for (int I = n; I >= 1; --I) {
        int L = 1;
        for (int its = 0; its <= 30; ++its) {
            int K;
            /* look for a single small subdiagonal (:810-867) */
            for (K = I; K >= L + 1; --K) {
                cplx hk = mget(H, K, K - 1);
                if (cabs1_(hk) <= smlnum) break;
                cplx hkm = mget(H, K - 1, K - 1), hkk = mget(H, K, K);
                double tst = cabs1_(hkm) + cabs1_(hkk);
                if (tst == 0.0) {
                    if (K - 2 >= 1) tst += fabs(mget(H, K - 1, K - 2).r);
                    if (K + 1 <= n) tst += fabs(mget(H, K + 1, K).i); /* as shipped (:840) */
                }
                if (fabs(hk.r) <= ulp * tst) {
                    double d2 = cabs1_(hk), d3 = cabs1_(mget(H, K - 1, K));
                    double ab = fmax(d2, d3), ba = fmin(d2, d3);
                    d2 = cabs1_(hkk);
                    d3 = cabs1_(csub_(hkm, hkk));
                    double aa = fmax(d2, d3), bb = fmin(d2, d3);
                    double s = aa + ab;
                    if (ba * (ab / s) <= fmax(smlnum, ulp * (bb * (aa / s)))) break;
                }
            }
            L = K;
            if (L > 1) mset(H, L, L - 1, cmk(0.0, 0.0));
            if (L >= I) break;

            /* shift (:896-990) */
            cplx t;
            if (its == 10) {
                t = cadd_(cmk(0.75 * fabs(mget(H, L + 1, L).r), 0.0), mget(H, L, L));
            } else if (its == 20) {
                t = cadd_(cmk(0.75 * fabs(mget(H, I, I - 1).r), 0.0), mget(H, I, I));
            } else {
                t = mget(H, I, I);
                cplx u = cmul_(csqrt_(mget(H, I - 1, I)), csqrt_(mget(H, I, I - 1)));
                double s = cabs1_(u);
                if (s != 0.0) {
                    cplx x = cscal_(csub_(mget(H, I - 1, I - 1), t), 0.5);
                    double sx = cabs1_(x);
                    s = fmax(s, sx);
                    cplx xs = cdivr_(x, s), us = cdivr_(u, s);
                    cplx y = cscal_(csqrt_(cadd_(cmul_(xs, xs), cmul_(us, us))), s);
                    if (sx > 0.0) {
                        double zr = x.r / sx, zi = x.i / sx;
                        if (zr * y.r + zi * y.i < 0.0) y = cmk(-y.r, -y.i);
                    }
                    t = csub_(t, cmul_(cdiv_(u, cadd_(x, y)), u));
                }
            }
            /* first column of the shifted matrix; M = L (:993-1015) */
            cplx h11s = csub_(mget(H, L, L), t);
            double h21 = mget(H, L + 1, L).r;
            double s = cabs1_(h11s) + fabs(h21);
            cplx v0 = cdivr_(h11s, s);
            cplx v1 = cmk(h21 / s, 0.0);
            ++sweeps;
            qr_sweep_one(H, Z, I, L, I1, I2, v0, v1);
        }
    }
    for (int I = n; I >= 1; --I) vset(E, I, mget(H, I, I));
    return sweeps;
}

/* ------------------------------------------------------------------------- */
/* Upper-triangular solve, right-hand side in x (Toolbox.hpp:31-136).          */
/* ------------------------------------------------------------------------- */
static void backsubs_one(int m, const mview *T, const vview *x)
{
    for (int j = m; j >= 1; --j) {
        cplx xj = cdiv_(vget(x, j), mget(T, j, j));
        vset(x, j, xj);
        for (int i = j - 1; i >= 1; --i) vset(x, i, csub_(vget(x, i), cmul_(mget(T, i, j), xj)));
    }
}

/* ------------------------------------------------------------------------- */
/* ztrevc, right eigenvectors back-transformed (Toolbox.hpp:1133-1313).        */
/* diag, rhs: length-dim work.                                                */
/* ------------------------------------------------------------------------- */
static void ztrevc_one(const mview *T, const mview *R, cplx *diag, cplx *rhs)
{
    const int n = T->n;
    const double ulp = DBL_EPSILON;
    const double smlnum = DBL_MIN * ((double)n / ulp);
    for (int i = 1; i <= n; ++i) diag[i - 1] = mget(T, i, i);
    vview xv; /* rhs as a unit-stride vector view */
    double *xr = (double *)rhs, *xi = xr + 1;
    xv.r = xr; xv.i = xi; xv.s = 2;
    for (int ki = n; ki >= 1; --ki) {
        cplx tkk = mget(T, ki, ki);
        double smin = fmax(ulp * cabs1_(tkk), smlnum);
        for (int k = 1; k <= ki - 1; ++k) vset(&xv, k, cmk(-mget(T, k, ki).r, -mget(T, k, ki).i));
        for (int k = 1; k <= ki - 1; ++k) {
            cplx d = csub_(mget(T, k, k), tkk);
            if (cabs1_(d) < smin) d = cmk(smin, 0.0);
            mset(T, k, k, d);
        }
        if (ki > 1) {
            backsubs_one(ki - 1, T, &xv);
            /* R(:,ki) := R(:,1:ki-1) x + R(:,ki) */
            for (int j = 1; j <= ki - 1; ++j) {
                cplx xj = vget(&xv, j);
                for (int i = 1; i <= n; ++i) mset(R, i, ki, cadd_(mget(R, i, ki), cmul_(mget(R, i, j), xj)));
            }
        }
        for (int k = 1; k <= ki - 1; ++k) mset(T, k, k, diag[k - 1]);
    }
}

/* ------------------------------------------------------------------------- */
/* Batch drivers.                                                              */
/* ------------------------------------------------------------------------- */
#define VO_MAXDIM 4096

void vo_zgehrd(int dim, int block_cnt, int thread_cnt, double *rA, double *iA, double *rtau, double *itau)
{
    if (dim <= 0 || block_cnt <= 0 || thread_cnt <= 0 || dim > VO_MAXDIM) return;
#pragma omp parallel for schedule(static, 8) num_threads(vo_get_threads())
    for (int b = 0; b < block_cnt; ++b) {
        cplx *w = (cplx *)malloc(sizeof(cplx) * (size_t)dim);
        for (int t = 0; t < thread_cnt; ++t) {
            mview A = batch_mat(rA, iA, dim, thread_cnt, b, t);
            vview tau = batch_vec(rtau, itau, dim, thread_cnt, b, t);
            zgehrd_one(&A, &tau, w);
        }
        free(w);
    }
}

void vo_zunghr(int dim, int block_cnt, int thread_cnt, double *rQ, double *iQ, const double *rtau, const double *itau)
{
    if (dim <= 0 || block_cnt <= 0 || thread_cnt <= 0 || dim > VO_MAXDIM) return;
#pragma omp parallel for schedule(static, 8) num_threads(vo_get_threads())
    for (int b = 0; b < block_cnt; ++b) {
        cplx *w = (cplx *)malloc(sizeof(cplx) * (size_t)dim);
        for (int t = 0; t < thread_cnt; ++t) {
            mview Q = batch_mat(rQ, iQ, dim, thread_cnt, b, t);
            vview tau = batch_vec((double *)rtau, (double *)itau, dim, thread_cnt, b, t);
            zunghr_one(&Q, &tau, w);
        }
        free(w);
    }
}

void vo_clear_below_subdiag(int dim, int block_cnt, int thread_cnt, double *rH, double *iH)
{
    if (dim <= 0 || block_cnt <= 0 || thread_cnt <= 0) return;
#pragma omp parallel for schedule(static, 8) num_threads(vo_get_threads())
    for (int b = 0; b < block_cnt; ++b)
        for (int t = 0; t < thread_cnt; ++t) {
            mview H = batch_mat(rH, iH, dim, thread_cnt, b, t);
            for (int j = 1; j <= dim; ++j)
                for (int i = j + 2; i <= dim; ++i) mset(&H, i, j, cmk(0.0, 0.0));
        }
}

void vo_zlahqr(int dim, int block_cnt, int thread_cnt, double *rE, double *iE,
               double *rH, double *iH, double *rZ, double *iZ, int *sweeps)
{
    if (dim <= 0 || block_cnt <= 0 || thread_cnt <= 0) return;
#pragma omp parallel for schedule(static, 8) num_threads(vo_get_threads())
    for (int b = 0; b < block_cnt; ++b)
        for (int t = 0; t < thread_cnt; ++t) {
            mview H = batch_mat(rH, iH, dim, thread_cnt, b, t);
            mview Z = batch_mat(rZ, iZ, dim, thread_cnt, b, t);
            vview E = batch_vec(rE, iE, dim, thread_cnt, b, t);
            int sw = zlahqr_one(&H, &Z, &E);
            if (sweeps) sweeps[(size_t)b * thread_cnt + t] = sw;
        }
}

void vo_ztrevc(int dim, int block_cnt, int thread_cnt, double *rT, double *iT, double *rZ, double *iZ)
{
    if (dim <= 0 || block_cnt <= 0 || thread_cnt <= 0 || dim > VO_MAXDIM) return;
#pragma omp parallel for schedule(static, 8) num_threads(vo_get_threads())
    for (int b = 0; b < block_cnt; ++b) {
        cplx *work = (cplx *)malloc(sizeof(cplx) * 2 * (size_t)dim);
        for (int t = 0; t < thread_cnt; ++t) {
            mview T = batch_mat(rT, iT, dim, thread_cnt, b, t);
            mview R = batch_mat(rZ, iZ, dim, thread_cnt, b, t);
            ztrevc_one(&T, &R, work, work + dim);
        }
        free(work);
    }
}

void vo_zgemv(int hermitian, int dim, int block_cnt, int thread_cnt,
              const double *rA, const double *iA, const double *rx, const double *ix,
              double rbeta, double ibeta, double *ry, double *iy)
{
    if (dim <= 0 || block_cnt <= 0 || thread_cnt <= 0) return;
    const cplx beta = cmk(rbeta, ibeta);
#pragma omp parallel for num_threads(vo_get_threads())
    for (int b = 0; b < block_cnt; ++b)
        for (int t = 0; t < thread_cnt; ++t) {
            mview A = batch_mat((double *)rA, (double *)iA, dim, thread_cnt, b, t);
            vview x = batch_vec((double *)rx, (double *)ix, dim, thread_cnt, b, t);
            vview y = batch_vec(ry, iy, dim, thread_cnt, b, t);
            for (int i = 1; i <= dim; ++i) vset(&y, i, cmul_(vget(&y, i), beta));
            if (!hermitian) {
                for (int j = 1; j <= dim; ++j) {
                    cplx xj = vget(&x, j);
                    for (int i = 1; i <= dim; ++i) vset(&y, i, cadd_(vget(&y, i), cmul_(mget(&A, i, j), xj)));
                }
            } else {
                for (int j = 1; j <= dim; ++j) {
                    cplx acc = cmk(0.0, 0.0);
                    for (int i = 1; i <= dim; ++i) acc = cadd_(acc, cmulc_(vget(&x, i), mget(&A, i, j)));
                    vset(&y, j, cadd_(vget(&y, j), acc));
                }
            }
        }
}

void vo_backsubstitution(int dim, int block_cnt, int thread_cnt,
                         const double *rT, const double *iT, double *rx, double *ix)
{
    if (dim <= 0 || block_cnt <= 0 || thread_cnt <= 0) return;
#pragma omp parallel for num_threads(vo_get_threads())
    for (int b = 0; b < block_cnt; ++b)
        for (int t = 0; t < thread_cnt; ++t) {
            mview T = batch_mat((double *)rT, (double *)iT, dim, thread_cnt, b, t);
            vview x = batch_vec(rx, ix, dim, thread_cnt, b, t);
            backsubs_one(dim, &T, &x);
        }
}

void vo_eigensolver(int dim, int block_cnt, int thread_cnt,
                    double *rA, double *iA, double *rE, double *iE,
                    double *rV, double *iV, int *sweeps)
{
    /* Staged over the whole batch exactly as utils.cpp:578-620: zgehrd, copy
     * A -> V, zunghr, [clear below the subdiagonal], zlahqr, ztrevc. */
    if (dim <= 0 || block_cnt <= 0 || thread_cnt <= 0 || dim > VO_MAXDIM) return;
    size_t nv = (size_t)dim * block_cnt * thread_cnt;
    size_t nm = nv * (size_t)dim;
    double *rtau = (double *)malloc(sizeof(double) * nv);
    double *itau = (double *)malloc(sizeof(double) * nv);
    vo_zgehrd(dim, block_cnt, thread_cnt, rA, iA, rtau, itau);
    memcpy(rV, rA, nm * sizeof(double));
    memcpy(iV, iA, nm * sizeof(double));
    vo_zunghr(dim, block_cnt, thread_cnt, rV, iV, rtau, itau);
    vo_clear_below_subdiag(dim, block_cnt, thread_cnt, rA, iA);
    vo_zlahqr(dim, block_cnt, thread_cnt, rE, iE, rA, iA, rV, iV, sweeps);
    vo_ztrevc(dim, block_cnt, thread_cnt, rA, iA, rV, iV);
    free(rtau);
    free(itau);
}
