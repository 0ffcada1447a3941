/*
 * oracle.h — CPU restatement of the BLAS routines on the intercepted path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this code; only tests/, the smoke check and bench.py's CPU-baseline
 * leg use it, and only as the checker.
 *
 * Semantics follow the netlib reference BLAS, which is what the reference's
 * argument checks replicate (blas_level3/gemm.cc:87-127, trsm.cc:76-132,
 * syrk.cc:78-146, trmm.cc:82-137) and what its runnable path finally executes
 * (the CPU BLAS reached through dlsym(RTLD_NEXT), runtime-blas.c:60-69,
 * gemm.cc:129-141).  Column-major storage, 1-based indices for i?amax/i?amin.
 *
 * Pinning: the restatement is checked against golden vectors produced by
 * OpenBLAS (tests/golden/make_golden.py) and against OpenBLAS run live in the
 * CPU test suite.
 */
#ifndef GBX_ORACLE_H
#define GBX_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- seeded inputs: SplitMix64 mapped to uniform[-1,1] ------------------ */
uint64_t orc_splitmix64_next(uint64_t *state);
/* Fill n doubles: v = 2*((x>>11) * 2^-53) - 1.  Returns the new state. */
uint64_t orc_fill_uniform(uint64_t state, double *out, size_t n);
/* Column-major m×n matrix with leading dimension ld; padding rows get 0. */
uint64_t orc_fill_matrix(uint64_t state, double *a, int m, int n, int ld);
/* Triangular test matrix for DTRSM: diag uniform[1,2], off-diagonal
 * uniform[-1,1]/n (draws one value per entry, column-major, whole square). */
uint64_t orc_fill_trsm_matrix(uint64_t state, double *a, int n, int ld);
/* u * 2^e with u uniform[-1,1], e uniform integer in [-s, s] (Ozaki inputs) */
uint64_t orc_fill_spread(uint64_t state, double *a, size_t n, int s);

/* ---- Level 1 ----------------------------------------------------------- */
void   orc_daxpy(int n, double alpha, const double *x, int incx, double *y, int incy);
double orc_ddot(int n, const double *x, int incx, const double *y, int incy);
double orc_dnrm2(int n, const double *x, int incx);
int    orc_idamax(int n, const double *x, int incx);
int    orc_idamin(int n, const double *x, int incx);

/* ---- Level 2 ----------------------------------------------------------- */
void orc_dgemv(char trans, int m, int n, double alpha, const double *a, int lda,
               const double *x, int incx, double beta, double *y, int incy);

/* ---- Level 3 ----------------------------------------------------------- */
void orc_dgemm(char ta, char tb, int m, int n, int k, double alpha,
               const double *a, int lda, const double *b, int ldb,
               double beta, double *c, int ldc);
/* complex: interleaved (re, im) pairs, ld in complex elements */
void orc_zgemm(char ta, char tb, int m, int n, int k, const double *alpha,
               const double *a, int lda, const double *b, int ldb,
               const double *beta, double *c, int ldc);
void orc_dsyrk(char uplo, char trans, int n, int k, double alpha,
               const double *a, int lda, double beta, double *c, int ldc);
void orc_dtrmm(char side, char uplo, char transa, char diag, int m, int n,
               double alpha, const double *a, int lda, double *b, int ldb);
void orc_dtrsm(char side, char uplo, char transa, char diag, int m, int n,
               double alpha, const double *a, int lda, double *b, int ldb);

/* DGER / DSYMV / DTRSV (vectors follow netlib's increment rules) */
void orc_dger(int m, int n, double alpha, const double *x, int incx, const double *y, int incy, double *a,
              int lda);
void orc_dsymv(char uplo, int n, double alpha, const double *a, int lda, const double *x, int incx, double beta,
               double *y, int incy);
void orc_dtrsv(char uplo, char trans, char diag, int n, const double *a, int lda, double *x, int incx);
int orc_check_dger(int m, int n, int incx, int incy, int lda);
int orc_check_dsymv(char uplo, int n, int lda, int incx, int incy);
int orc_check_dtrsv(char uplo, char trans, char diag, int n, int lda, int incx);

/* The rest of the Level-3 set, complex double (real and single-precision
 * routines are checked through these with zero imaginary parts).  allowed:
 * transposition letters the routine takes, 1 N | 2 T | 4 C.  herm selects
 * the Hermitian form (xHEMM, xHERK, xHER2K). */
void orc_zsymm(char side, char uplo, int m, int n, const double *alpha, const double *a, int lda,
               const double *b, int ldb, const double *beta, double *c, int ldc, int herm);
void orc_zsyrk(char uplo, char trans, int allowed, int n, int k, const double *alpha, const double *a,
               int lda, const double *beta, double *c, int ldc, int herm);
void orc_zsyr2k(char uplo, char trans, int allowed, int n, int k, const double *alpha, const double *a,
                int lda, const double *b, int ldb, const double *beta, double *c, int ldc, int herm);
void orc_ztrmm(char side, char uplo, char ta, char diag, int m, int n, const double *alpha,
               const double *a, int lda, double *b, int ldb);
void orc_ztrsm(char side, char uplo, char ta, char diag, int m, int n, const double *alpha,
               const double *a, int lda, double *b, int ldb);
int orc_check_symm(char side, char uplo, int m, int n, int lda, int ldb, int ldc);
int orc_check_rank_k(char uplo, char trans, int allowed, int n, int k, int lda, int ldc);
int orc_check_rank_2k(char uplo, char trans, int allowed, int n, int k, int lda, int ldb, int ldc);

/* ---- argument checks (netlib INFO numbering; 0 = valid) ----------------- */
int orc_check_dgemm(char ta, char tb, int m, int n, int k, int lda, int ldb, int ldc);
int orc_check_dtrsm(char side, char uplo, char ta, char diag, int m, int n, int lda, int ldb);
int orc_check_dsyrk(char uplo, char trans, int n, int k, int lda, int ldc);
int orc_check_dgemv(char trans, int m, int n, int lda, int incx, int incy);

/* ---- double-double accuracy checkers ------------------------------------ */
/* alpha*op(A)*op(B) + beta*C evaluated in double-double, rounded to double. */
void orc_dgemm_dd(char ta, char tb, int m, int n, int k, double alpha,
                  const double *a, int lda, const double *b, int ldb,
                  double beta, const double *c, int ldc, double *out, int ldo);
/* The same at nsample (row, col) pairs only: out[s] for (rows[s], cols[s]). */
void orc_dgemm_dd_sample(char ta, char tb, int k, double alpha,
                         const double *a, int lda, const double *b, int ldb,
                         double beta, const double *c, int ldc,
                         int nsample, const int *rows, const int *cols, double *out);
/* complex variant: out interleaved */
void orc_zgemm_dd_sample(char ta, char tb, int k, const double *alpha,
                         const double *a, int lda, const double *b, int ldb,
                         const double *beta, const double *c, int ldc,
                         int nsample, const int *rows, const int *cols, double *out);
/* ||op(A)*X - alpha*B0||_F / (||A||_F*||X||_F + |alpha|*||B0||_F), dd residual
 * of a triangular solve (side L: op(A) X; side R: X op(A)). */
double orc_dtrsm_residual(char side, char uplo, char transa, char diag, int m, int n,
                          double alpha, const double *a, int lda,
                          const double *b0, int ldb0, const double *x, int ldx);
/* max |op(A)*X - alpha*B0| / (|op(A)|*|X| + |alpha|*|B0|) entrywise, dd
 * (componentwise backward error of a triangular solve). */
double orc_dtrsm_residual_cw(char side, char uplo, char transa, char diag, int m, int n,
                             double alpha, const double *a, int lda,
                             const double *b0, int ldb0, const double *x, int ldx);
/* dd dot product rounded to double */
double orc_ddot_dd(int n, const double *x, int incx, const double *y, int incy);

/* relative Frobenius error ||x - ref||_F / ||ref||_F over an m×n block */
double orc_rel_fro(int m, int n, const double *x, int ldx, const double *ref, int ldr);

#ifdef __cplusplus
}
#endif
#endif
