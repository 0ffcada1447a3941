/*
 * oracle.c — CPU restatement of the netlib BLAS semantics on the intercepted
 * path, plus double-double accuracy checkers.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  The shipped library never links or
 * calls this file.  Build with -ffp-contract=off so that x86 and Arm hosts
 * round every operation the same way and the error-free transformations stay
 * exact.
 *
 * Reference anchors (paths inside the reference project):
 *   DGEMM  argument checks and quick returns  blas_level3/gemm.cc:87-127
 *   DTRSM  argument checks, alpha==0 zeroing  blas_level3/trsm.cc:76-132
 *   DSYRK  argument checks, alpha==0 scaling  blas_level3/syrk.cc:78-146
 *   DTRMM  argument checks                    blas_level3/trmm.cc:82-137
 *   DGEMV  CBLAS wrapper (dead code)          blas_level2/gemv.cc:11-98
 *   DAXPY/DDOT/DNRM2/IDAMAX/IDAMIN wrappers   blas_level1/axpy.cc:10-50,
 *          dot.cc:9-48, nrm2.cc:9-41, amax.cc:32-43, amin.cc:32-43
 *   CPU BLAS fallback that actually runs      runtime-blas.c:60-69,
 *                                             gemm.cc:129-141
 * The arithmetic the reference finally executes is the CPU BLAS's; the loop
 * orders below are the netlib reference-BLAS ones for that arithmetic.
 */
#include "oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

static int up(char c) { return (c >= 'a' && c <= 'z') ? c - 32 : c; }
static int same(char a, char b) { return up(a) == up(b); }
static int imax(int a, int b) { return a > b ? a : b; }

/* ------------------------------------------------------------------------ */
/* SplitMix64 (Steele, Lea, Flood 2014)                                      */
/* ------------------------------------------------------------------------ */
uint64_t orc_splitmix64_next(uint64_t *state)
{
    uint64_t z = (*state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static double u01(uint64_t *s) { return (double)(orc_splitmix64_next(s) >> 11) * 0x1.0p-53; }
static double um11(uint64_t *s) { return 2.0 * u01(s) - 1.0; }

uint64_t orc_fill_uniform(uint64_t state, double *out, size_t n)
{
    for (size_t i = 0; i < n; i++) out[i] = um11(&state);
    return state;
}

uint64_t orc_fill_matrix(uint64_t state, double *a, int m, int n, int ld)
{
    for (int j = 0; j < n; j++) {
        for (int i = 0; i < m; i++) a[(size_t)j * ld + i] = um11(&state);
        for (int i = m; i < ld; i++) a[(size_t)j * ld + i] = 0.0;
    }
    return state;
}

uint64_t orc_fill_trsm_matrix(uint64_t state, double *a, int n, int ld)
{
    for (int j = 0; j < n; j++)
        for (int i = 0; i < ld; i++) {
            if (i >= n) { a[(size_t)j * ld + i] = 0.0; continue; }
            double v = um11(&state);
            a[(size_t)j * ld + i] = (i == j) ? 1.5 + 0.5 * v : v / (double)n;
        }
    return state;
}

uint64_t orc_fill_spread(uint64_t state, double *a, size_t n, int s)
{
    for (size_t i = 0; i < n; i++) {
        double u = um11(&state);
        int e = 0;
        if (s > 0) {
            uint64_t r = orc_splitmix64_next(&state);
            e = (int)(r % (uint64_t)(2 * s + 1)) - s;
        }
        a[i] = ldexp(u, e);
    }
    return state;
}

/* ------------------------------------------------------------------------ */
/* Level 1                                                                   */
/* ------------------------------------------------------------------------ */
/* element i (0-based) of a strided vector, netlib convention for inc < 0 */
static size_t vidx(int i, int n, int inc)
{
    return inc >= 0 ? (size_t)i * inc : (size_t)(n - 1 - i) * (size_t)(-inc);
}

void orc_daxpy(int n, double alpha, const double *x, int incx, double *y, int incy)
{
    if (n <= 0 || alpha == 0.0) return;
    for (int i = 0; i < n; i++) y[vidx(i, n, incy)] += alpha * x[vidx(i, n, incx)];
}

double orc_ddot(int n, const double *x, int incx, const double *y, int incy)
{
    double s = 0.0;
    if (n <= 0) return 0.0;
    for (int i = 0; i < n; i++) s += x[vidx(i, n, incx)] * y[vidx(i, n, incy)];
    return s;
}

/* ---- double-double helpers (Knuth TwoSum, FMA TwoProduct; Ogita, Rump and
 *      Oishi, "Accurate sum and dot product", SISC 2005) ------------------ */
typedef struct { double hi, lo; } dd;
static inline void two_sum(double a, double b, double *s, double *e)
{
    double x = a + b, bb = x - a;
    *s = x; *e = (a - (x - bb)) + (b - bb);
}
static inline void two_prod(double a, double b, double *p, double *e)
{
    *p = a * b; *e = fma(a, b, -*p);
}
static inline dd dd_add_d(dd a, double b)
{
    double s, e; two_sum(a.hi, b, &s, &e);
    e += a.lo;
    dd r; two_sum(s, e, &r.hi, &r.lo); return r;
}
static inline dd dd_add(dd a, dd b)
{
    double s, e; two_sum(a.hi, b.hi, &s, &e);
    e += a.lo + b.lo;
    dd r; two_sum(s, e, &r.hi, &r.lo); return r;
}
static inline dd dd_fma(dd acc, double a, double b) /* acc + a*b */
{
    double p, pe; two_prod(a, b, &p, &pe);
    double s, e; two_sum(acc.hi, p, &s, &e);
    e += acc.lo + pe;
    dd r; two_sum(s, e, &r.hi, &r.lo); return r;
}
static inline dd dd_mul_d(dd a, double b)
{
    double p, pe; two_prod(a.hi, b, &p, &pe);
    pe += a.lo * b;
    dd r; two_sum(p, pe, &r.hi, &r.lo); return r;
}
static inline double dd_to_d(dd a) { return a.hi + a.lo; }

double orc_dnrm2(int n, const double *x, int incx)
{
    /* Two-pass scaling: find max |x|, scale by the power of two nearest to it
     * (exact), accumulate the squares in double-double, unscale. */
    if (n < 1 || incx < 1) return 0.0;
    double amax = 0.0;
    for (int i = 0; i < n; i++) {
        double v = fabs(x[(size_t)i * incx]);
        if (isnan(v)) return v;
        if (v > amax) amax = v;
    }
    if (amax == 0.0 || isinf(amax)) return amax;
    int e; frexp(amax, &e);
    dd s = {0.0, 0.0};
    for (int i = 0; i < n; i++) {
        double v = ldexp(x[(size_t)i * incx], -e);
        s = dd_fma(s, v, v);
    }
    /* sqrt of a double-double: one Newton step from sqrt(hi) */
    double r = sqrt(s.hi);
    if (r > 0.0) {
        double p, pe; two_prod(r, r, &p, &pe);
        double corr = ((s.hi - p) - pe + s.lo) / (2.0 * r);
        r = r + corr;
    }
    return ldexp(r, e);
}

int orc_idamax(int n, const double *x, int incx)
{
    if (n < 1 || incx <= 0) return 0;
    int best = 1;
    double m = fabs(x[0]);
    for (int i = 1; i < n; i++) {
        double v = fabs(x[(size_t)i * incx]);
        if (v > m) { m = v; best = i + 1; }
    }
    return best;
}

int orc_idamin(int n, const double *x, int incx)
{
    if (n < 1 || incx <= 0) return 0;
    int best = 1;
    double m = fabs(x[0]);
    for (int i = 1; i < n; i++) {
        double v = fabs(x[(size_t)i * incx]);
        if (v < m) { m = v; best = i + 1; }
    }
    return best;
}

double orc_ddot_dd(int n, const double *x, int incx, const double *y, int incy)
{
    dd s = {0.0, 0.0};
    if (n <= 0) return 0.0;
    for (int i = 0; i < n; i++) s = dd_fma(s, x[vidx(i, n, incx)], y[vidx(i, n, incy)]);
    return dd_to_d(s);
}

/* ------------------------------------------------------------------------ */
/* Level 2                                                                   */
/* ------------------------------------------------------------------------ */
int orc_check_dgemv(char trans, int m, int n, int lda, int incx, int incy)
{
    if (!same(trans, 'N') && !same(trans, 'T') && !same(trans, 'C')) return 1;
    if (m < 0) return 2;
    if (n < 0) return 3;
    if (lda < imax(1, m)) return 6;
    if (incx == 0) return 8;
    if (incy == 0) return 11;
    return 0;
}

void orc_dgemv(char trans, int m, int n, double alpha, const double *a, int lda,
               const double *x, int incx, double beta, double *y, int incy)
{
    if (orc_check_dgemv(trans, m, n, lda, incx, incy)) return;
    if (m == 0 || n == 0 || (alpha == 0.0 && beta == 1.0)) return;
    int notr = same(trans, 'N');
    int lenx = notr ? n : m, leny = notr ? m : n;
    if (beta != 1.0)
        for (int i = 0; i < leny; i++) {
            size_t iy = vidx(i, leny, incy);
            y[iy] = (beta == 0.0) ? 0.0 : beta * y[iy];
        }
    if (alpha == 0.0) return;
    if (notr) {
        for (int j = 0; j < n; j++) {
            double t = alpha * x[vidx(j, lenx, incx)];
            for (int i = 0; i < m; i++) y[vidx(i, leny, incy)] += t * a[(size_t)j * lda + i];
        }
    } else {
        for (int j = 0; j < n; j++) {
            double t = 0.0;
            for (int i = 0; i < m; i++) t += a[(size_t)j * lda + i] * x[vidx(i, lenx, incx)];
            y[vidx(j, leny, incy)] += alpha * t;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Level 3                                                                   */
/* ------------------------------------------------------------------------ */
#define A_(i, j) a[(size_t)(j) * lda + (i)]
#define B_(i, j) b[(size_t)(j) * ldb + (i)]
#define C_(i, j) c[(size_t)(j) * ldc + (i)]

int orc_check_dgemm(char ta, char tb, int m, int n, int k, int lda, int ldb, int ldc)
{
    int nota = same(ta, 'N'), notb = same(tb, 'N');
    int nrowa = nota ? m : k, nrowb = notb ? k : n;
    if (!nota && !same(ta, 'C') && !same(ta, 'T')) return 1;
    if (!notb && !same(tb, 'C') && !same(tb, 'T')) return 2;
    if (m < 0) return 3;
    if (n < 0) return 4;
    if (k < 0) return 5;
    if (lda < imax(1, nrowa)) return 8;
    if (ldb < imax(1, nrowb)) return 10;
    if (ldc < imax(1, m)) return 13;
    return 0;
}

void orc_dgemm(char ta, char tb, int m, int n, int k, double alpha,
               const double *a, int lda, const double *b, int ldb,
               double beta, double *c, int ldc)
{
    if (orc_check_dgemm(ta, tb, m, n, k, lda, ldb, ldc)) return;
    if (m == 0 || n == 0 || ((alpha == 0.0 || k == 0) && beta == 1.0)) return;
    int nota = same(ta, 'N'), notb = same(tb, 'N');
    if (alpha == 0.0) {
        for (int j = 0; j < n; j++)
            for (int i = 0; i < m; i++) C_(i, j) = (beta == 0.0) ? 0.0 : beta * C_(i, j);
        return;
    }
    if (nota) {
        /* C(:,j) = beta*C(:,j) + sum_l (alpha*opB(l,j)) * A(:,l) */
        for (int j = 0; j < n; j++) {
            if (beta == 0.0) for (int i = 0; i < m; i++) C_(i, j) = 0.0;
            else if (beta != 1.0) for (int i = 0; i < m; i++) C_(i, j) *= beta;
            for (int l = 0; l < k; l++) {
                double t = alpha * (notb ? B_(l, j) : B_(j, l));
                for (int i = 0; i < m; i++) C_(i, j) += t * A_(i, l);
            }
        }
    } else {
        /* C(i,j) = alpha * sum_l A(l,i)*opB(l,j) + beta*C(i,j) */
        for (int j = 0; j < n; j++)
            for (int i = 0; i < m; i++) {
                double t = 0.0;
                for (int l = 0; l < k; l++) t += A_(l, i) * (notb ? B_(l, j) : B_(j, l));
                C_(i, j) = (beta == 0.0) ? alpha * t : alpha * t + beta * C_(i, j);
            }
    }
}

/* complex helpers on interleaved pairs */
typedef struct { double re, im; } zc;
static inline zc zld(const double *p) { zc r = {p[0], p[1]}; return r; }
static inline zc zmul(zc a, zc b) { zc r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }
static inline zc zadd(zc a, zc b) { zc r = {a.re + b.re, a.im + b.im}; return r; }
static inline zc zconj(zc a) { zc r = {a.re, -a.im}; return r; }

static zc zop(const double *m, int ld, int i, int j, char t)
{
    /* element (i,j) of op(M) */
    if (same(t, 'N')) return zld(m + 2 * ((size_t)j * ld + i));
    zc v = zld(m + 2 * ((size_t)i * ld + j));
    return same(t, 'C') ? zconj(v) : v;
}

void orc_zgemm(char ta, char tb, int m, int n, int k, const double *alpha,
               const double *a, int lda, const double *b, int ldb,
               const double *beta, double *c, int ldc)
{
    if (orc_check_dgemm(ta, tb, m, n, k, lda, ldb, ldc)) return;
    zc al = {alpha[0], alpha[1]}, be = {beta[0], beta[1]};
    int alpha0 = al.re == 0.0 && al.im == 0.0, beta0 = be.re == 0.0 && be.im == 0.0;
    int beta1 = be.re == 1.0 && be.im == 0.0;
    if (m == 0 || n == 0 || ((alpha0 || k == 0) && beta1)) return;
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            double *cp = c + 2 * ((size_t)j * ldc + i);
            zc t = {0.0, 0.0};
            if (!alpha0)
                for (int l = 0; l < k; l++) t = zadd(t, zmul(zop(a, lda, i, l, ta), zop(b, ldb, l, j, tb)));
            zc r = zmul(al, t);
            if (!beta0) r = zadd(r, zmul(be, zld(cp)));
            cp[0] = r.re; cp[1] = r.im;
        }
}

int orc_check_dsyrk(char uplo, char trans, int n, int k, int lda, int ldc)
{
    int nrowa = same(trans, 'N') ? n : k;
    if (!same(uplo, 'U') && !same(uplo, 'L')) return 1;
    if (!same(trans, 'N') && !same(trans, 'T') && !same(trans, 'C')) return 2;
    if (n < 0) return 3;
    if (k < 0) return 4;
    if (lda < imax(1, nrowa)) return 7;
    if (ldc < imax(1, n)) return 10;
    return 0;
}

void orc_dsyrk(char uplo, char trans, int n, int k, double alpha,
               const double *a, int lda, double beta, double *c, int ldc)
{
    if (orc_check_dsyrk(uplo, trans, n, k, lda, ldc)) return;
    if (n == 0 || ((alpha == 0.0 || k == 0) && beta == 1.0)) return;
    int upper = same(uplo, 'U'), notr = same(trans, 'N');
    for (int j = 0; j < n; j++) {
        int i0 = upper ? 0 : j, i1 = upper ? j + 1 : n;
        if (alpha == 0.0) {
            for (int i = i0; i < i1; i++) C_(i, j) = (beta == 0.0) ? 0.0 : beta * C_(i, j);
            continue;
        }
        if (notr) {
            if (beta == 0.0) for (int i = i0; i < i1; i++) C_(i, j) = 0.0;
            else if (beta != 1.0) for (int i = i0; i < i1; i++) C_(i, j) *= beta;
            for (int l = 0; l < k; l++) {
                double t = alpha * A_(j, l);
                for (int i = i0; i < i1; i++) C_(i, j) += t * A_(i, l);
            }
        } else {
            for (int i = i0; i < i1; i++) {
                double t = 0.0;
                for (int l = 0; l < k; l++) t += A_(l, i) * A_(l, j);
                C_(i, j) = (beta == 0.0) ? alpha * t : alpha * t + beta * C_(i, j);
            }
        }
    }
}

int orc_check_dtrsm(char side, char uplo, char ta, char diag, int m, int n, int lda, int ldb)
{
    int lside = same(side, 'L');
    int nrowa = lside ? m : n;
    if (!lside && !same(side, 'R')) return 1;
    if (!same(uplo, 'U') && !same(uplo, 'L')) return 2;
    if (!same(ta, 'N') && !same(ta, 'T') && !same(ta, 'C')) return 3;
    if (!same(diag, 'U') && !same(diag, 'N')) return 4;
    if (m < 0) return 5;
    if (n < 0) return 6;
    if (lda < imax(1, nrowa)) return 9;
    if (ldb < imax(1, m)) return 11;
    return 0;
}

/* Explicit op(A) as a dense na×na matrix, zero outside the effective triangle,
 * unit diagonal when diag == 'U'.  Returns 1 if op(A) is lower triangular. */
static int explicit_tri(char uplo, char ta, char diag, int na, const double *a, int lda, double *t)
{
    int upper = same(uplo, 'U'), notr = same(ta, 'N'), unit = same(diag, 'U');
    for (int j = 0; j < na; j++)
        for (int i = 0; i < na; i++) {
            int ai = notr ? i : j, aj = notr ? j : i;     /* A element backing op(A)(i,j) */
            int in_tri = upper ? (ai <= aj) : (ai >= aj);
            double v = in_tri ? A_(ai, aj) : 0.0;
            if (i == j && unit) v = 1.0;
            t[(size_t)j * na + i] = v;
        }
    return upper ? !notr : notr;
}

void orc_dtrsm(char side, char uplo, char ta, char diag, int m, int n,
               double alpha, const double *a, int lda, double *b, int ldb)
{
    if (orc_check_dtrsm(side, uplo, ta, diag, m, n, lda, ldb)) return;
    if (m == 0 || n == 0) return;
    if (alpha == 0.0) {
        for (int j = 0; j < n; j++) for (int i = 0; i < m; i++) B_(i, j) = 0.0;
        return;
    }
    int lside = same(side, 'L'), unit = same(diag, 'U');
    int na = lside ? m : n;
    double *t = (double *)malloc(sizeof(double) * (size_t)na * na);
    int lower = explicit_tri(uplo, ta, diag, na, a, lda, t);
#define T_(i, j) t[(size_t)(j) * na + (i)]
    for (int j = 0; j < n; j++) for (int i = 0; i < m; i++) B_(i, j) *= alpha;
    if (lside) {
        for (int j = 0; j < n; j++) {
            if (lower) {
                for (int kk = 0; kk < m; kk++) {
                    if (!unit) B_(kk, j) /= T_(kk, kk);
                    for (int i = kk + 1; i < m; i++) B_(i, j) -= B_(kk, j) * T_(i, kk);
                }
            } else {
                for (int kk = m - 1; kk >= 0; kk--) {
                    if (!unit) B_(kk, j) /= T_(kk, kk);
                    for (int i = 0; i < kk; i++) B_(i, j) -= B_(kk, j) * T_(i, kk);
                }
            }
        }
    } else {
        /* X * T = alpha*B, column by column */
        if (!lower) {
            for (int j = 0; j < n; j++) {
                for (int kk = 0; kk < j; kk++)
                    for (int i = 0; i < m; i++) B_(i, j) -= T_(kk, j) * B_(i, kk);
                if (!unit) for (int i = 0; i < m; i++) B_(i, j) /= T_(j, j);
            }
        } else {
            for (int j = n - 1; j >= 0; j--) {
                for (int kk = j + 1; kk < n; kk++)
                    for (int i = 0; i < m; i++) B_(i, j) -= T_(kk, j) * B_(i, kk);
                if (!unit) for (int i = 0; i < m; i++) B_(i, j) /= T_(j, j);
            }
        }
    }
#undef T_
    free(t);
}

void orc_dtrmm(char side, char uplo, char ta, char diag, int m, int n,
               double alpha, const double *a, int lda, double *b, int ldb)
{
    if (orc_check_dtrsm(side, uplo, ta, diag, m, n, lda, ldb)) return;
    if (m == 0 || n == 0) return;
    if (alpha == 0.0) {
        for (int j = 0; j < n; j++) for (int i = 0; i < m; i++) B_(i, j) = 0.0;
        return;
    }
    int lside = same(side, 'L');
    int na = lside ? m : n;
    double *t = (double *)malloc(sizeof(double) * (size_t)na * na);
    double *r = (double *)malloc(sizeof(double) * (size_t)m * n);
    explicit_tri(uplo, ta, diag, na, a, lda, t);
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            double s = 0.0;
            if (lside) for (int l = 0; l < m; l++) s += t[(size_t)l * na + i] * B_(l, j);
            else       for (int l = 0; l < n; l++) s += B_(i, l) * t[(size_t)j * na + l];
            r[(size_t)j * m + i] = alpha * s;
        }
    for (int j = 0; j < n; j++) for (int i = 0; i < m; i++) B_(i, j) = r[(size_t)j * m + i];
    free(r); free(t);
}

/* ------------------------------------------------------------------------ */
/* DGER, DSYMV, DTRSV (netlib dger.f, dsymv.f, dtrsv.f loop orders; the      */
/* reference's CBLAS bodies blas_level2/ger.cc:86-94, symv.cc:88-96,         */
/* trsv.cc:81-87 forward to cuBLAS)                                          */
/* ------------------------------------------------------------------------ */
int orc_check_dger(int m, int n, int incx, int incy, int lda)
{
    if (m < 0) return 1;
    if (n < 0) return 2;
    if (incx == 0) return 5;
    if (incy == 0) return 7;
    if (lda < imax(1, m)) return 9;
    return 0;
}

void orc_dger(int m, int n, double alpha, const double *x, int incx, const double *y, int incy, double *a, int lda)
{
    if (orc_check_dger(m, n, incx, incy, lda)) return;
    if (m == 0 || n == 0 || alpha == 0.0) return;
    for (int j = 0; j < n; j++) {
        double yj = y[vidx(j, n, incy)];
        if (yj == 0.0) continue;
        double t = alpha * yj;
        for (int i = 0; i < m; i++) A_(i, j) += x[vidx(i, m, incx)] * t;
    }
}

int orc_check_dsymv(char uplo, int n, int lda, int incx, int incy)
{
    if (!same(uplo, 'U') && !same(uplo, 'L')) return 1;
    if (n < 0) return 2;
    if (lda < imax(1, n)) return 5;
    if (incx == 0) return 7;
    if (incy == 0) return 10;
    return 0;
}

void orc_dsymv(char uplo, int n, double alpha, const double *a, int lda, const double *x, int incx, double beta,
               double *y, int incy)
{
    if (orc_check_dsymv(uplo, n, lda, incx, incy)) return;
    if (n == 0 || (alpha == 0.0 && beta == 1.0)) return;
    int upper = same(uplo, 'U');
    for (int i = 0; i < n; i++) {
        double s = 0.0;
        if (alpha != 0.0)
            for (int j = 0; j < n; j++) {
                int stored = upper ? (i <= j) : (i >= j);
                s += (stored ? A_(i, j) : A_(j, i)) * x[vidx(j, n, incx)];
            }
        double *yp = &y[vidx(i, n, incy)];
        *yp = (beta == 0.0) ? alpha * s : alpha * s + beta * *yp;
    }
}

int orc_check_dtrsv(char uplo, char trans, char diag, int n, int lda, int incx)
{
    if (!same(uplo, 'U') && !same(uplo, 'L')) return 1;
    if (!same(trans, 'N') && !same(trans, 'T') && !same(trans, 'C')) return 2;
    if (!same(diag, 'U') && !same(diag, 'N')) return 3;
    if (n < 0) return 4;
    if (lda < imax(1, n)) return 6;
    if (incx == 0) return 8;
    return 0;
}

void orc_dtrsv(char uplo, char trans, char diag, int n, const double *a, int lda, double *x, int incx)
{
    if (orc_check_dtrsv(uplo, trans, diag, n, lda, incx)) return;
    if (n == 0) return;
    double *t = (double *)malloc(sizeof(double) * (size_t)n * n);
    int lower = explicit_tri(uplo, trans, diag, n, a, lda, t), unit = same(diag, 'U');
    double *v = (double *)malloc(sizeof(double) * (size_t)n);
    for (int i = 0; i < n; i++) v[i] = x[vidx(i, n, incx)];
    if (lower) {
        for (int i = 0; i < n; i++) {
            double s = v[i];
            for (int j = 0; j < i; j++) s -= t[(size_t)j * n + i] * v[j];
            v[i] = unit ? s : s / t[(size_t)i * n + i];
        }
    } else {
        for (int i = n - 1; i >= 0; i--) {
            double s = v[i];
            for (int j = i + 1; j < n; j++) s -= t[(size_t)j * n + i] * v[j];
            v[i] = unit ? s : s / t[(size_t)i * n + i];
        }
    }
    for (int i = 0; i < n; i++) x[vidx(i, n, incx)] = v[i];
    free(v);
    free(t);
}

/* ------------------------------------------------------------------------ */
/* The rest of the Level-3 set in complex double: xSYMM/xHEMM, xSYRK/xHERK,  */
/* xSYR2K/xHER2K, complex xTRMM/xTRSM.  Real (S, D) and single-precision     */
/* (S, C) routines are checked against these with zero imaginary parts and   */
/* inputs widened to double.  Semantics follow the netlib reference BLAS     */
/* (zsymm.f, zhemm.f, zsyrk.f, zherk.f, zsyr2k.f, zher2k.f, ztrmm.f,         */
/* ztrsm.f), which is what the reference's wrappers reproduce              */
/* (blas_level3/symm.cc, hemm.cc, syrk.cc, herk.cc, syr2k.cc, her2k.cc,      */
/* trmm.cc, trsm.cc argument checks) before handing the call to cuBLAS.      */
/* ------------------------------------------------------------------------ */
static inline zc zget(const double *m, int ld, int i, int j) { return zld(m + 2 * ((size_t)j * ld + i)); }
static inline void zput(double *m, int ld, int i, int j, zc v)
{
    m[2 * ((size_t)j * ld + i)] = v.re;
    m[2 * ((size_t)j * ld + i) + 1] = v.im;
}
static inline int zis(const double *a, double re) { return a[0] == re && a[1] == 0.0; }

int orc_check_symm(char side, char uplo, int m, int n, int lda, int ldb, int ldc)
{
    int nrowa = same(side, 'L') ? m : n;
    if (!same(side, 'L') && !same(side, 'R')) return 1;
    if (!same(uplo, 'U') && !same(uplo, 'L')) return 2;
    if (m < 0) return 3;
    if (n < 0) return 4;
    if (lda < imax(1, nrowa)) return 7;
    if (ldb < imax(1, m)) return 9;
    if (ldc < imax(1, m)) return 12;
    return 0;
}

/* element (i,j) of the symmetric / Hermitian matrix stored in one triangle */
static zc sym_elem(const double *a, int lda, char uplo, int i, int j, int herm)
{
    int stored = same(uplo, 'U') ? (i <= j) : (i >= j);
    zc v = stored ? zget(a, lda, i, j) : zget(a, lda, j, i);
    if (herm) {
        if (!stored) v = zconj(v);
        if (i == j) v.im = 0.0;
    }
    return v;
}

void orc_zsymm(char side, char uplo, int m, int n, const double *alpha, const double *a, int lda,
               const double *b, int ldb, const double *beta, double *c, int ldc, int herm)
{
    if (orc_check_symm(side, uplo, m, n, lda, ldb, ldc)) return;
    zc al = zld(alpha), be = zld(beta);
    int alpha0 = zis(alpha, 0.0), beta0 = zis(beta, 0.0), beta1 = zis(beta, 1.0);
    if (m == 0 || n == 0 || (alpha0 && beta1)) return;
    int lside = same(side, 'L');
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            zc t = {0.0, 0.0};
            if (!alpha0) {
                if (lside) for (int l = 0; l < m; l++) t = zadd(t, zmul(sym_elem(a, lda, uplo, i, l, herm), zget(b, ldb, l, j)));
                else       for (int l = 0; l < n; l++) t = zadd(t, zmul(zget(b, ldb, i, l), sym_elem(a, lda, uplo, l, j, herm)));
            }
            zc r = zmul(al, t);
            if (!beta0) r = zadd(r, zmul(be, zget(c, ldc, i, j)));
            zput(c, ldc, i, j, r);
        }
}

/* transposition letters: 1 N, 2 T, 4 C (real routines take all three) */
static int trans_ok(char t, int allowed)
{
    return (same(t, 'N') && (allowed & 1)) || (same(t, 'T') && (allowed & 2)) || (same(t, 'C') && (allowed & 4));
}

int orc_check_rank_k(char uplo, char trans, int allowed, int n, int k, int lda, int ldc)
{
    int nrowa = same(trans, 'N') ? n : k;
    if (!same(uplo, 'U') && !same(uplo, 'L')) return 1;
    if (!trans_ok(trans, allowed)) return 2;
    if (n < 0) return 3;
    if (k < 0) return 4;
    if (lda < imax(1, nrowa)) return 7;
    if (ldc < imax(1, n)) return 10;
    return 0;
}

int orc_check_rank_2k(char uplo, char trans, int allowed, int n, int k, int lda, int ldb, int ldc)
{
    int nrowa = same(trans, 'N') ? n : k;
    if (!same(uplo, 'U') && !same(uplo, 'L')) return 1;
    if (!trans_ok(trans, allowed)) return 2;
    if (n < 0) return 3;
    if (k < 0) return 4;
    if (lda < imax(1, nrowa)) return 7;
    if (ldb < imax(1, nrowa)) return 9;
    if (ldc < imax(1, n)) return 12;
    return 0;
}

/* op(X)(i,l) for a rank-k operand: N -> X(i,l); T -> X(l,i); C -> conj X(l,i) */
static zc rk_op(const double *x, int ld, int i, int l, char trans, int herm)
{
    if (same(trans, 'N')) return zget(x, ld, i, l);
    zc v = zget(x, ld, l, i);
    return herm ? zconj(v) : v;
}
/* op(X)'(l,j), the transposed (herm: conjugate-transposed) factor */
static zc rk_opt(const double *x, int ld, int l, int j, char trans, int herm)
{
    if (!same(trans, 'N')) return zget(x, ld, l, j);
    zc v = zget(x, ld, j, l);
    return herm ? zconj(v) : v;
}

/* C = alpha op(A) op(A)' + beta C on the uplo triangle; herm: ' = ^H, alpha
 * and beta real (imaginary parts ignored), diagonal of C made real */
void orc_zsyrk(char uplo, char trans, int allowed, int n, int k, const double *alpha, const double *a, int lda,
               const double *beta, double *c, int ldc, int herm)
{
    if (orc_check_rank_k(uplo, trans, allowed, n, k, lda, ldc)) return;
    zc al = zld(alpha), be = zld(beta);
    if (herm) { al.im = 0.0; be.im = 0.0; }
    int alpha0 = al.re == 0.0 && al.im == 0.0, beta0 = be.re == 0.0 && be.im == 0.0;
    int beta1 = be.re == 1.0 && be.im == 0.0;
    if (n == 0 || ((alpha0 || k == 0) && beta1)) return;
    int upper = same(uplo, 'U');
    for (int j = 0; j < n; j++)
        for (int i = upper ? 0 : j; i < (upper ? j + 1 : n); i++) {
            zc t = {0.0, 0.0};
            if (!alpha0)
                for (int l = 0; l < k; l++)
                    t = zadd(t, zmul(rk_op(a, lda, i, l, trans, herm), rk_opt(a, lda, l, j, trans, herm)));
            zc r = zmul(al, t);
            if (!beta0) r = zadd(r, zmul(be, zget(c, ldc, i, j)));
            if (herm && i == j) r.im = 0.0;
            zput(c, ldc, i, j, r);
        }
}

/* C = alpha op(A) op(B)' + alpha' op(B) op(A)' + beta C; alpha' = alpha
 * (symmetric) or conj(alpha) (herm, beta real, diagonal made real) */
void orc_zsyr2k(char uplo, char trans, int allowed, int n, int k, const double *alpha, const double *a, int lda,
                const double *b, int ldb, const double *beta, double *c, int ldc, int herm)
{
    if (orc_check_rank_2k(uplo, trans, allowed, n, k, lda, ldb, ldc)) return;
    zc al = zld(alpha), be = zld(beta);
    if (herm) be.im = 0.0;
    zc al2 = herm ? zconj(al) : al;
    int alpha0 = al.re == 0.0 && al.im == 0.0, beta0 = be.re == 0.0 && be.im == 0.0;
    int beta1 = be.re == 1.0 && be.im == 0.0;
    if (n == 0 || ((alpha0 || k == 0) && beta1)) return;
    int upper = same(uplo, 'U');
    for (int j = 0; j < n; j++)
        for (int i = upper ? 0 : j; i < (upper ? j + 1 : n); i++) {
            zc t1 = {0.0, 0.0}, t2 = {0.0, 0.0};
            if (!alpha0)
                for (int l = 0; l < k; l++) {
                    t1 = zadd(t1, zmul(rk_op(a, lda, i, l, trans, herm), rk_opt(b, ldb, l, j, trans, herm)));
                    t2 = zadd(t2, zmul(rk_op(b, ldb, i, l, trans, herm), rk_opt(a, lda, l, j, trans, herm)));
                }
            zc r = zadd(zmul(al, t1), zmul(al2, t2));
            if (!beta0) r = zadd(r, zmul(be, zget(c, ldc, i, j)));
            if (herm && i == j) r.im = 0.0;
            zput(c, ldc, i, j, r);
        }
}

static zc zdiv(zc a, zc b)
{
    double d = b.re * b.re + b.im * b.im;
    zc r = {(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
    return r;
}

/* explicit op(A) (na x na, complex) for TRMM/TRSM; returns 1 if lower */
static int zexplicit_tri(char uplo, char ta, char diag, int na, const double *a, int lda, zc *t)
{
    int upper = same(uplo, 'U'), notr = same(ta, 'N'), unit = same(diag, 'U'), cj = same(ta, 'C');
    for (int j = 0; j < na; j++)
        for (int i = 0; i < na; i++) {
            int ai = notr ? i : j, aj = notr ? j : i;
            int in_tri = upper ? (ai <= aj) : (ai >= aj);
            zc v = {0.0, 0.0};
            if (in_tri) v = zget(a, lda, ai, aj);
            if (cj) v = zconj(v);
            if (i == j && unit) { v.re = 1.0; v.im = 0.0; }
            t[(size_t)j * na + i] = v;
        }
    return upper ? !notr : notr;
}

void orc_ztrmm(char side, char uplo, char ta, char diag, int m, int n, const double *alpha, const double *a,
               int lda, double *b, int ldb)
{
    if (orc_check_dtrsm(side, uplo, ta, diag, m, n, lda, ldb)) return;
    if (m == 0 || n == 0) return;
    zc al = zld(alpha);
    int lside = same(side, 'L'), na = lside ? m : n;
    zc *t = (zc *)malloc(sizeof(zc) * (size_t)na * na);
    zc *r = (zc *)malloc(sizeof(zc) * (size_t)m * n);
    zexplicit_tri(uplo, ta, diag, na, a, lda, t);
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            zc s2 = {0.0, 0.0};
            if (lside) for (int l = 0; l < m; l++) s2 = zadd(s2, zmul(t[(size_t)l * na + i], zget(b, ldb, l, j)));
            else       for (int l = 0; l < n; l++) s2 = zadd(s2, zmul(zget(b, ldb, i, l), t[(size_t)j * na + l]));
            r[(size_t)j * m + i] = zmul(al, s2);
        }
    if (al.re == 0.0 && al.im == 0.0)
        for (size_t q = 0; q < (size_t)m * n; q++) { r[q].re = 0.0; r[q].im = 0.0; }
    for (int j = 0; j < n; j++) for (int i = 0; i < m; i++) zput(b, ldb, i, j, r[(size_t)j * m + i]);
    free(r); free(t);
}

void orc_ztrsm(char side, char uplo, char ta, char diag, int m, int n, const double *alpha, const double *a,
               int lda, double *b, int ldb)
{
    if (orc_check_dtrsm(side, uplo, ta, diag, m, n, lda, ldb)) return;
    if (m == 0 || n == 0) return;
    zc al = zld(alpha);
    if (al.re == 0.0 && al.im == 0.0) {
        zc z = {0.0, 0.0};
        for (int j = 0; j < n; j++) for (int i = 0; i < m; i++) zput(b, ldb, i, j, z);
        return;
    }
    int lside = same(side, 'L'), unit = same(diag, 'U'), na = lside ? m : n;
    zc *t = (zc *)malloc(sizeof(zc) * (size_t)na * na);
    int lower = zexplicit_tri(uplo, ta, diag, na, a, lda, t);
#define ZT(i, j) t[(size_t)(j) * na + (i)]
#define ZB(i, j) zget(b, ldb, i, j)
#define ZSET(i, j, v) zput(b, ldb, i, j, v)
    for (int j = 0; j < n; j++) for (int i = 0; i < m; i++) ZSET(i, j, zmul(al, ZB(i, j)));
    if (lside) {
        for (int j = 0; j < n; j++) {
            if (lower) {
                for (int kk = 0; kk < m; kk++) {
                    if (!unit) ZSET(kk, j, zdiv(ZB(kk, j), ZT(kk, kk)));
                    for (int i = kk + 1; i < m; i++) {
                        zc p = zmul(ZB(kk, j), ZT(i, kk));
                        zc v = ZB(i, j); v.re -= p.re; v.im -= p.im; ZSET(i, j, v);
                    }
                }
            } else {
                for (int kk = m - 1; kk >= 0; kk--) {
                    if (!unit) ZSET(kk, j, zdiv(ZB(kk, j), ZT(kk, kk)));
                    for (int i = 0; i < kk; i++) {
                        zc p = zmul(ZB(kk, j), ZT(i, kk));
                        zc v = ZB(i, j); v.re -= p.re; v.im -= p.im; ZSET(i, j, v);
                    }
                }
            }
        }
    } else if (!lower) {
        for (int j = 0; j < n; j++) {
            for (int kk = 0; kk < j; kk++)
                for (int i = 0; i < m; i++) {
                    zc p = zmul(ZT(kk, j), ZB(i, kk));
                    zc v = ZB(i, j); v.re -= p.re; v.im -= p.im; ZSET(i, j, v);
                }
            if (!unit) for (int i = 0; i < m; i++) ZSET(i, j, zdiv(ZB(i, j), ZT(j, j)));
        }
    } else {
        for (int j = n - 1; j >= 0; j--) {
            for (int kk = j + 1; kk < n; kk++)
                for (int i = 0; i < m; i++) {
                    zc p = zmul(ZT(kk, j), ZB(i, kk));
                    zc v = ZB(i, j); v.re -= p.re; v.im -= p.im; ZSET(i, j, v);
                }
            if (!unit) for (int i = 0; i < m; i++) ZSET(i, j, zdiv(ZB(i, j), ZT(j, j)));
        }
    }
#undef ZT
#undef ZB
#undef ZSET
    free(t);
}

/* ------------------------------------------------------------------------ */
/* double-double checkers                                                    */
/* ------------------------------------------------------------------------ */
static double opd(const double *m, int ld, int i, int j, char t)
{
    return same(t, 'N') ? m[(size_t)j * ld + i] : m[(size_t)i * ld + j];
}

static double dgemm_dd_one(char ta, char tb, int k, double alpha, const double *a, int lda,
                           const double *b, int ldb, double beta, double cij, int i, int j)
{
    dd s = {0.0, 0.0};
    for (int l = 0; l < k; l++) s = dd_fma(s, opd(a, lda, i, l, ta), opd(b, ldb, l, j, tb));
    dd r = dd_mul_d(s, alpha);
    if (beta != 0.0) {
        double p, pe; two_prod(beta, cij, &p, &pe);
        dd t = {p, pe};
        r = dd_add(r, t);
    }
    return dd_to_d(r);
}

void orc_dgemm_dd(char ta, char tb, int m, int n, int k, double alpha,
                  const double *a, int lda, const double *b, int ldb,
                  double beta, const double *c, int ldc, double *out, int ldo)
{
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++)
            out[(size_t)j * ldo + i] = dgemm_dd_one(ta, tb, k, alpha, a, lda, b, ldb, beta,
                                                    beta != 0.0 ? C_(i, j) : 0.0, i, j);
}

void orc_dgemm_dd_sample(char ta, char tb, int k, double alpha,
                         const double *a, int lda, const double *b, int ldb,
                         double beta, const double *c, int ldc,
                         int nsample, const int *rows, const int *cols, double *out)
{
    for (int s = 0; s < nsample; s++) {
        int i = rows[s], j = cols[s];
        out[s] = dgemm_dd_one(ta, tb, k, alpha, a, lda, b, ldb, beta,
                              beta != 0.0 ? C_(i, j) : 0.0, i, j);
    }
}

void orc_zgemm_dd_sample(char ta, char tb, int k, const double *alpha,
                         const double *a, int lda, const double *b, int ldb,
                         const double *beta, const double *c, int ldc,
                         int nsample, const int *rows, const int *cols, double *out)
{
    for (int s = 0; s < nsample; s++) {
        int i = rows[s], j = cols[s];
        dd re = {0.0, 0.0}, im = {0.0, 0.0};
        for (int l = 0; l < k; l++) {
            zc x = zop(a, lda, i, l, ta), y = zop(b, ldb, l, j, tb);
            re = dd_fma(re, x.re, y.re); re = dd_fma(re, -x.im, y.im);
            im = dd_fma(im, x.re, y.im); im = dd_fma(im, x.im, y.re);
        }
        /* alpha * t */
        dd rr = dd_add(dd_mul_d(re, alpha[0]), dd_mul_d(im, -alpha[1]));
        dd ri = dd_add(dd_mul_d(im, alpha[0]), dd_mul_d(re, alpha[1]));
        if (beta[0] != 0.0 || beta[1] != 0.0) {
            zc cv = zld(c + 2 * ((size_t)j * ldc + i));
            rr = dd_fma(rr, beta[0], cv.re); rr = dd_fma(rr, -beta[1], cv.im);
            ri = dd_fma(ri, beta[0], cv.im); ri = dd_fma(ri, beta[1], cv.re);
        }
        out[2 * s] = dd_to_d(rr);
        out[2 * s + 1] = dd_to_d(ri);
    }
}

double orc_dtrsm_residual(char side, char uplo, char ta, char diag, int m, int n,
                          double alpha, const double *a, int lda,
                          const double *b0, int ldb0, const double *x, int ldx)
{
    int lside = same(side, 'L');
    int na = lside ? m : n;
    double *t = (double *)malloc(sizeof(double) * (size_t)na * na);
    explicit_tri(uplo, ta, diag, na, a, lda, t);
    dd rn = {0.0, 0.0}, tn = {0.0, 0.0}, xn = {0.0, 0.0}, bn = {0.0, 0.0};
    for (size_t q = 0; q < (size_t)na * na; q++) tn = dd_fma(tn, t[q], t[q]);
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            double xv = x[(size_t)j * ldx + i], bv = b0[(size_t)j * ldb0 + i];
            xn = dd_fma(xn, xv, xv);
            bn = dd_fma(bn, bv, bv);
            dd s = {0.0, 0.0};
            if (lside) for (int l = 0; l < m; l++) s = dd_fma(s, t[(size_t)l * na + i], x[(size_t)j * ldx + l]);
            else       for (int l = 0; l < n; l++) s = dd_fma(s, x[(size_t)l * ldx + i], t[(size_t)j * na + l]);
            double p, pe; two_prod(-alpha, bv, &p, &pe);
            dd q = {p, pe};
            double r = dd_to_d(dd_add(s, q));
            rn = dd_fma(rn, r, r);
        }
    free(t);
    double den = sqrt(dd_to_d(tn)) * sqrt(dd_to_d(xn)) + fabs(alpha) * sqrt(dd_to_d(bn));
    return den > 0.0 ? sqrt(dd_to_d(rn)) / den : sqrt(dd_to_d(rn));
}

/* Componentwise backward error of a triangular solve (Oettli-Prager):
 * max over entries of |op(A) X - alpha B0| / (|op(A)| |X| + |alpha| |B0|),
 * side L (op(A) X) or R (X op(A)), residual and denominators in
 * double-double.  A substitution solve keeps it near n*u whatever the
 * conditioning; it is the measure under which inverse-based solves can lose. */
double orc_dtrsm_residual_cw(char side, char uplo, char ta, char diag, int m, int n,
                             double alpha, const double *a, int lda,
                             const double *b0, int ldb0, const double *x, int ldx)
{
    int lside = same(side, 'L');
    int na = lside ? m : n;
    double *t = (double *)malloc(sizeof(double) * (size_t)na * na);
    explicit_tri(uplo, ta, diag, na, a, lda, t);
    double worst = 0.0;
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            double bv = b0[(size_t)j * ldb0 + i];
            dd s = {0.0, 0.0}, w = {0.0, 0.0};
            if (lside)
                for (int l = 0; l < m; l++) {
                    double tv = t[(size_t)l * na + i], xv = x[(size_t)j * ldx + l];
                    s = dd_fma(s, tv, xv);
                    w = dd_fma(w, fabs(tv), fabs(xv));
                }
            else
                for (int l = 0; l < n; l++) {
                    double tv = t[(size_t)j * na + l], xv = x[(size_t)l * ldx + i];
                    s = dd_fma(s, xv, tv);
                    w = dd_fma(w, fabs(xv), fabs(tv));
                }
            double p, pe; two_prod(-alpha, bv, &p, &pe);
            dd q = {p, pe};
            double r = fabs(dd_to_d(dd_add(s, q)));
            double den = dd_to_d(w) + fabs(alpha) * fabs(bv);
            double ratio = den > 0.0 ? r / den : (r > 0.0 ? INFINITY : 0.0);
            if (ratio > worst || ratio != ratio) worst = ratio;
        }
    free(t);
    return worst;
}

double orc_rel_fro(int m, int n, const double *x, int ldx, const double *ref, int ldr)
{
    dd num = {0.0, 0.0}, den = {0.0, 0.0};
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            double r = ref[(size_t)j * ldr + i], d = x[(size_t)j * ldx + i] - r;
            num = dd_fma(num, d, d);
            den = dd_fma(den, r, r);
        }
    double dn = dd_to_d(den);
    return dn > 0.0 ? sqrt(dd_to_d(num) / dn) : sqrt(dd_to_d(num));
}
