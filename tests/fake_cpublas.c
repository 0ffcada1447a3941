/*
 * fake_cpublas.c — a stand-in CPU BLAS for the forwarding test of the
 * allocation interposer (OBJTRACKER_OPTIONS=blas_libs=<this library>).
 * Plain netlib-semantics loops for the few routines the test program calls;
 * each call also writes "fake <routine>" to stderr, so the test sees which
 * library ran it.  Column-major, no argument checks (the caller's are valid).
 */
#include <math.h>
#include <string.h>
#include <unistd.h>

static void mark(const char *name)
{
    char buf[64];
    size_t n = strlen(name);
    memcpy(buf, "fake ", 5);
    memcpy(buf + 5, name, n);
    buf[5 + n] = '\n';
    if (write(2, buf, n + 6) < 0) { /* nothing to do */ }
}

void dgemm_(const char *ta, const char *tb, const int *m, const int *n, const int *k, const double *alpha,
            const double *a, const int *lda, const double *b, const int *ldb, const double *beta, double *c,
            const int *ldc)
{
    mark("dgemm_");
    const int nota = (*ta == 'N' || *ta == 'n'), notb = (*tb == 'N' || *tb == 'n');
    for (int j = 0; j < *n; j++)
        for (int i = 0; i < *m; i++) {
            double s = 0.0;
            for (int l = 0; l < *k; l++)
                s += (nota ? a[l * *lda + i] : a[i * *lda + l]) * (notb ? b[j * *ldb + l] : b[l * *ldb + j]);
            c[j * *ldc + i] = *alpha * s + (*beta == 0.0 ? 0.0 : *beta * c[j * *ldc + i]);
        }
}

void dsymm_(const char *side, const char *uplo, const int *m, const int *n, const double *alpha, const double *a,
            const int *lda, const double *b, const int *ldb, const double *beta, double *c, const int *ldc)
{
    mark("dsymm_");
    const int left = (*side == 'L' || *side == 'l'), upper = (*uplo == 'U' || *uplo == 'u');
    const int na = left ? *m : *n;
    for (int j = 0; j < *n; j++)
        for (int i = 0; i < *m; i++) {
            double s = 0.0;
            for (int l = 0; l < na; l++) {
                const int r = left ? i : l, q = left ? l : j;          /* A(r, q) */
                const int rr = (upper ? r <= q : r >= q) ? r : q, qq = rr == r ? q : r;
                const double av = a[qq * *lda + rr];
                s += left ? av * b[j * *ldb + l] : b[l * *ldb + i] * av;
            }
            c[j * *ldc + i] = *alpha * s + (*beta == 0.0 ? 0.0 : *beta * c[j * *ldc + i]);
        }
}

double ddot_(const int *n, const double *x, const int *incx, const double *y, const int *incy)
{
    mark("ddot_");
    double s = 0.0;
    for (int i = 0; i < *n; i++) s += x[i * *incx] * y[i * *incy];
    return s;
}

int idamax_(const int *n, const double *x, const int *incx)
{
    mark("idamax_");
    if (*n < 1 || *incx <= 0) return 0;
    int best = 1;
    for (int i = 1; i < *n; i++)
        if (fabs(x[i * *incx]) > fabs(x[(best - 1) * *incx])) best = i + 1;
    return best;
}
