/*
 * gbxblas_f77.h — the drop-in symbols exported by libgbxblas.so.
 *
 * Fortran ABI (LP64): every argument by reference, option characters as
 * const char*, 32-bit integers.  Trailing hidden character-length arguments
 * that gfortran passes are accepted and ignored (they are not read).
 * Column-major storage.  Every call is synchronous: the result is in the
 * caller's memory when the function returns.  Invalid arguments call
 * xerbla_("NAME  ", &info) with the netlib parameter position and return.
 *
 * Each declaration names the reference interface it replaces.
 */
#ifndef GBXBLAS_F77_H
#define GBXBLAS_F77_H

#include "gbxblas.h"

#ifdef __cplusplus
extern "C" {
#endif

/* F77_gemm(d, double)  blas.h:202-215, body blas_level3/gemm.cc:162-179 */
void dgemm_(const char *transa, const char *transb, const int *m, const int *n, const int *k,
            const double *alpha, const double *a, const int *lda, const double *b, const int *ldb,
            const double *beta, double *c, const int *ldc);
/* F77_gemm(z, double _Complex)  blas.h:202-215, body blas_level3/gemm.cc:200-216 */
void zgemm_(const char *transa, const char *transb, const int *m, const int *n, const int *k,
            const double *alpha, const double *a, const int *lda, const double *b, const int *ldb,
            const double *beta, double *c, const int *ldc);
/* F77_syrk(d, double)  blas.h:268-274, body blas_level3/syrk.cc:165-180 */
void dsyrk_(const char *uplo, const char *trans, const int *n, const int *k, const double *alpha,
            const double *a, const int *lda, const double *beta, double *c, const int *ldc);
/* F77_trsm(d, double)  blas.h:303-314, body blas_level3/trsm.cc:154-172 */
void dtrsm_(const char *side, const char *uplo, const char *transa, const char *diag,
            const int *m, const int *n, const double *alpha, const double *a, const int *lda,
            double *b, const int *ldb);
/* F77_trmm(d, double)  blas.h:290-301, body blas_level3/trmm.cc:158-175 (disabled there) */
void dtrmm_(const char *side, const char *uplo, const char *transa, const char *diag,
            const int *m, const int *n, const double *alpha, const double *a, const int *lda,
            double *b, const int *ldb);
/* The other precisions and Level-3 routines the reference exports
 * (prototypes blas.h:202-314, bodies blas_level3/<routine>.cc).  Complex scalars and
 * matrices are (re, im) pairs; Hermitian routines take the real alpha/beta
 * netlib gives them. */
/* F77_gemm(s|c)  gemm.cc:143-160, 181-198 */
void sgemm_(const char *transa, const char *transb, const int *m, const int *n, const int *k, const float *alpha,
            const float *a, const int *lda, const float *b, const int *ldb, const float *beta, float *c,
            const int *ldc);
void cgemm_(const char *transa, const char *transb, const int *m, const int *n, const int *k, const float *alpha,
            const float *a, const int *lda, const float *b, const int *ldb, const float *beta, float *c,
            const int *ldc);
/* F77_symm(s|d|c|z)  blas.h:254-266, symm.cc:124-200 */
void ssymm_(const char *side, const char *uplo, const int *m, const int *n, const float *alpha, const float *a,
            const int *lda, const float *b, const int *ldb, const float *beta, float *c, const int *ldc);
void dsymm_(const char *side, const char *uplo, const int *m, const int *n, const double *alpha, const double *a,
            const int *lda, const double *b, const int *ldb, const double *beta, double *c, const int *ldc);
void csymm_(const char *side, const char *uplo, const int *m, const int *n, const float *alpha, const float *a,
            const int *lda, const float *b, const int *ldb, const float *beta, float *c, const int *ldc);
void zsymm_(const char *side, const char *uplo, const int *m, const int *n, const double *alpha, const double *a,
            const int *lda, const double *b, const int *ldb, const double *beta, double *c, const int *ldc);
/* F77_hemm(c|z)  blas.h:217-227, hemm.cc:120-154 */
void chemm_(const char *side, const char *uplo, const int *m, const int *n, const float *alpha, const float *a,
            const int *lda, const float *b, const int *ldb, const float *beta, float *c, const int *ldc);
void zhemm_(const char *side, const char *uplo, const int *m, const int *n, const double *alpha, const double *a,
            const int *lda, const double *b, const int *ldb, const double *beta, double *c, const int *ldc);
/* F77_syrk(s|c|z)  blas.h:268-274, syrk.cc:148-216 */
void ssyrk_(const char *uplo, const char *trans, const int *n, const int *k, const float *alpha, const float *a,
            const int *lda, const float *beta, float *c, const int *ldc);
void csyrk_(const char *uplo, const char *trans, const int *n, const int *k, const float *alpha, const float *a,
            const int *lda, const float *beta, float *c, const int *ldc);
void zsyrk_(const char *uplo, const char *trans, const int *n, const int *k, const double *alpha, const double *a,
            const int *lda, const double *beta, double *c, const int *ldc);
/* F77_herk(c|z)  blas.h:230-239, herk.cc:131-163 (alpha, beta real) */
void cherk_(const char *uplo, const char *trans, const int *n, const int *k, const float *alpha, const float *a,
            const int *lda, const float *beta, float *c, const int *ldc);
void zherk_(const char *uplo, const char *trans, const int *n, const int *k, const double *alpha, const double *a,
            const int *lda, const double *beta, double *c, const int *ldc);
/* F77_syr2k(s|d|c|z)  blas.h:276-288, syr2k.cc:146-218 */
void ssyr2k_(const char *uplo, const char *trans, const int *n, const int *k, const float *alpha, const float *a,
             const int *lda, const float *b, const int *ldb, const float *beta, float *c, const int *ldc);
void dsyr2k_(const char *uplo, const char *trans, const int *n, const int *k, const double *alpha,
             const double *a, const int *lda, const double *b, const int *ldb, const double *beta, double *c,
             const int *ldc);
void csyr2k_(const char *uplo, const char *trans, const int *n, const int *k, const float *alpha, const float *a,
             const int *lda, const float *b, const int *ldb, const float *beta, float *c, const int *ldc);
void zsyr2k_(const char *uplo, const char *trans, const int *n, const int *k, const double *alpha,
             const double *a, const int *lda, const double *b, const int *ldb, const double *beta, double *c,
             const int *ldc);
/* F77_her2k(c|z)  blas.h:242-252, her2k.cc:141-183 (beta real) */
void cher2k_(const char *uplo, const char *trans, const int *n, const int *k, const float *alpha, const float *a,
             const int *lda, const float *b, const int *ldb, const float *beta, float *c, const int *ldc);
void zher2k_(const char *uplo, const char *trans, const int *n, const int *k, const double *alpha,
             const double *a, const int *lda, const double *b, const int *ldb, const double *beta, double *c,
             const int *ldc);
/* F77_trmm(s|c|z)  blas.h:290-301, trmm.cc:139-215 (disabled in the reference's build) */
void strmm_(const char *side, const char *uplo, const char *transa, const char *diag, const int *m, const int *n,
            const float *alpha, const float *a, const int *lda, float *b, const int *ldb);
void ctrmm_(const char *side, const char *uplo, const char *transa, const char *diag, const int *m, const int *n,
            const float *alpha, const float *a, const int *lda, float *b, const int *ldb);
void ztrmm_(const char *side, const char *uplo, const char *transa, const char *diag, const int *m, const int *n,
            const double *alpha, const double *a, const int *lda, double *b, const int *ldb);
/* F77_trsm(s|c|z)  blas.h:303-314, trsm.cc:134-215 */
void strsm_(const char *side, const char *uplo, const char *transa, const char *diag, const int *m, const int *n,
            const float *alpha, const float *a, const int *lda, float *b, const int *ldb);
void ctrsm_(const char *side, const char *uplo, const char *transa, const char *diag, const int *m, const int *n,
            const float *alpha, const float *a, const int *lda, float *b, const int *ldb);
void ztrsm_(const char *side, const char *uplo, const char *transa, const char *diag, const int *m, const int *n,
            const double *alpha, const double *a, const int *lda, double *b, const int *ldb);

/* F77_gemv(d, double)  blas.h:85-92 (no body in the reference) */
void dgemv_(const char *trans, const int *m, const int *n, const double *alpha, const double *a,
            const int *lda, const double *x, const int *incx, const double *beta, double *y,
            const int *incy);
/* F77_ger(d, double)  blas.h:94-100; CBLAS body blas_level2/ger.cc:86-94 (not built there) */
void dger_(const int *m, const int *n, const double *alpha, const double *x, const int *incx, const double *y,
           const int *incy, double *a, const int *lda);
/* F77_symv(d, double)  blas.h:134-142; CBLAS body blas_level2/symv.cc:88-96 (not built there) */
void dsymv_(const char *uplo, const int *n, const double *alpha, const double *a, const int *lda,
            const double *x, const int *incx, const double *beta, double *y, const int *incy);
/* F77_trsv(d, double)  blas.h:193-200; CBLAS body blas_level2/trsv.cc:81-87 (not built there) */
void dtrsv_(const char *uplo, const char *trans, const char *diag, const int *n, const double *a, const int *lda,
            double *x, const int *incx);
/* F77_axpy(d, double)  blas.h:20-31 */
void daxpy_(const int *n, const double *alpha, const double *x, const int *incx, double *y,
            const int *incy);
/* F77_dot(d, double)  blas.h:45-51 (declared void there; returns double here) */
double ddot_(const int *n, const double *x, const int *incx, const double *y, const int *incy);
/* F77_nrm2(d, double)  blas.h:33-36 (declared void there; returns double here) */
double dnrm2_(const int *n, const double *x, const int *incx);
/* i?amax / i?amin: 1-based index, 0 when n < 1 or incx <= 0.
 * CBLAS bodies blas_level1/amax.cc:32-43, amin.cc:32-43 */
int idamax_(const int *n, const double *x, const int *incx);
int idamin_(const int *n, const double *x, const int *incx);

/* Error handler (weak; an application or tester may supply its own).
 * The reference forwards to the CPU BLAS's xerbla_ (runtime-blas.c:34-37). */
void xerbla_(const char *srname, const int *info, size_t len);
/* Case-insensitive character compare (weak), runtime-blas.c:55-58. */
int lsame_(const char *ca, const char *cb);

/* ---- CBLAS (enum values of cblas.h:21-25) ---------------------------------- */
enum GBX_CBLAS_LAYOUT { GbxRowMajor = 101, GbxColMajor = 102 };
enum GBX_CBLAS_TRANSPOSE { GbxNoTrans = 111, GbxTrans = 112, GbxConjTrans = 113 };
enum GBX_CBLAS_UPLO { GbxUpper = 121, GbxLower = 122 };
enum GBX_CBLAS_DIAG { GbxNonUnit = 131, GbxUnit = 132 };
enum GBX_CBLAS_SIDE { GbxLeft = 141, GbxRight = 142 };

/* The standard C interface: complex scalars by pointer (the reference's
 * cblas.h:661-822 declares them by value but defines no Level-3 CBLAS
 * bodies); Hermitian real scalars by value. */
/* cblas_?gemm  cblas.h:661-679 */
void cblas_dgemm(int layout, int transa, int transb, int m, int n, int k, double alpha,
                 const double *a, int lda, const double *b, int ldb, double beta, double *c,
                 int ldc);
void cblas_zgemm(int layout, int transa, int transb, int m, int n, int k, const void *alpha,
                 const void *a, int lda, const void *b, int ldb, const void *beta, void *c,
                 int ldc);
void cblas_sgemm(int layout, int transa, int transb, int m, int n, int k, float alpha, const void *a, int lda,
                 const void *b, int ldb, float beta, void *c, int ldc);
void cblas_cgemm(int layout, int transa, int transb, int m, int n, int k, const void *alpha, const void *a,
                 int lda, const void *b, int ldb, const void *beta, void *c, int ldc);
/* cblas_?syrk  cblas.h:750-766; cblas_?trsm 806-822; cblas_?trmm 787-804 */
void cblas_dsyrk(int layout, int uplo, int trans, int n, int k, double alpha, const double *a,
                 int lda, double beta, double *c, int ldc);
void cblas_dtrsm(int layout, int side, int uplo, int transa, int diag, int m, int n, double alpha,
                 const double *a, int lda, double *b, int ldb);
void cblas_dtrmm(int layout, int side, int uplo, int transa, int diag, int m, int n, double alpha,
                 const double *a, int lda, double *b, int ldb);
/* cblas_?symm cblas.h:731-748, cblas_?hemm 681-696 */
void cblas_ssymm(int layout, int side, int uplo, int m, int n, float alpha, const void *a, int lda,
                 const void *b, int ldb, float beta, void *c, int ldc);
void cblas_dsymm(int layout, int side, int uplo, int m, int n, double alpha, const void *a, int lda,
                 const void *b, int ldb, double beta, void *c, int ldc);
void cblas_csymm(int layout, int side, int uplo, int m, int n, const void *alpha, const void *a, int lda,
                 const void *b, int ldb, const void *beta, void *c, int ldc);
void cblas_zsymm(int layout, int side, int uplo, int m, int n, const void *alpha, const void *a, int lda,
                 const void *b, int ldb, const void *beta, void *c, int ldc);
void cblas_chemm(int layout, int side, int uplo, int m, int n, const void *alpha, const void *a, int lda,
                 const void *b, int ldb, const void *beta, void *c, int ldc);
void cblas_zhemm(int layout, int side, int uplo, int m, int n, const void *alpha, const void *a, int lda,
                 const void *b, int ldb, const void *beta, void *c, int ldc);
/* cblas_?syrk cblas.h:750-766, cblas_?herk 698-712 */
void cblas_ssyrk(int layout, int uplo, int trans, int n, int k, float alpha, const void *a, int lda, float beta,
                 void *c, int ldc);
void cblas_csyrk(int layout, int uplo, int trans, int n, int k, const void *alpha, const void *a, int lda,
                 const void *beta, void *c, int ldc);
void cblas_zsyrk(int layout, int uplo, int trans, int n, int k, const void *alpha, const void *a, int lda,
                 const void *beta, void *c, int ldc);
void cblas_cherk(int layout, int uplo, int trans, int n, int k, float alpha, const void *a, int lda, float beta,
                 void *c, int ldc);
void cblas_zherk(int layout, int uplo, int trans, int n, int k, double alpha, const void *a, int lda,
                 double beta, void *c, int ldc);
/* cblas_?syr2k cblas.h:768-785, cblas_?her2k 714-729 */
void cblas_ssyr2k(int layout, int uplo, int trans, int n, int k, float alpha, const void *a, int lda,
                  const void *b, int ldb, float beta, void *c, int ldc);
void cblas_dsyr2k(int layout, int uplo, int trans, int n, int k, double alpha, const void *a, int lda,
                  const void *b, int ldb, double beta, void *c, int ldc);
void cblas_csyr2k(int layout, int uplo, int trans, int n, int k, const void *alpha, const void *a, int lda,
                  const void *b, int ldb, const void *beta, void *c, int ldc);
void cblas_zsyr2k(int layout, int uplo, int trans, int n, int k, const void *alpha, const void *a, int lda,
                  const void *b, int ldb, const void *beta, void *c, int ldc);
void cblas_cher2k(int layout, int uplo, int trans, int n, int k, const void *alpha, const void *a, int lda,
                  const void *b, int ldb, float beta, void *c, int ldc);
void cblas_zher2k(int layout, int uplo, int trans, int n, int k, const void *alpha, const void *a, int lda,
                  const void *b, int ldb, double beta, void *c, int ldc);
/* cblas_?trmm cblas.h:787-804, cblas_?trsm 806-822 */
void cblas_strmm(int layout, int side, int uplo, int transa, int diag, int m, int n, float alpha, const void *a,
                 int lda, void *b, int ldb);
void cblas_ctrmm(int layout, int side, int uplo, int transa, int diag, int m, int n, const void *alpha,
                 const void *a, int lda, void *b, int ldb);
void cblas_ztrmm(int layout, int side, int uplo, int transa, int diag, int m, int n, const void *alpha,
                 const void *a, int lda, void *b, int ldb);
void cblas_strsm(int layout, int side, int uplo, int transa, int diag, int m, int n, float alpha, const void *a,
                 int lda, void *b, int ldb);
void cblas_ctrsm(int layout, int side, int uplo, int transa, int diag, int m, int n, const void *alpha,
                 const void *a, int lda, void *b, int ldb);
void cblas_ztrsm(int layout, int side, int uplo, int transa, int diag, int m, int n, const void *alpha,
                 const void *a, int lda, void *b, int ldb);
/* cblas.h:283-297 */
void cblas_dgemv(int layout, int trans, int m, int n, double alpha, const double *a, int lda,
                 const double *x, int incx, double beta, double *y, int incy);
/* cblas_?ger cblas.h:301-314, cblas_?symv 506-521, cblas_?trsv 640-655 */
void cblas_dger(int layout, int m, int n, double alpha, const double *x, int incx, const double *y, int incy,
                double *a, int lda);
void cblas_dsymv(int layout, int uplo, int n, double alpha, const double *a, int lda, const double *x, int incx,
                 double beta, double *y, int incy);
void cblas_dtrsv(int layout, int uplo, int trans, int diag, int n, const double *a, int lda, double *x, int incx);
void cblas_daxpy(int n, double alpha, const double *x, int incx, double *y, int incy);
double cblas_ddot(int n, const double *x, int incx, const double *y, int incy);
double cblas_dnrm2(int n, const double *x, int incx);
/* 0-based index (CBLAS_INDEX, cblas.h:18) */
int cblas_idamax(int n, const double *x, int incx);
int cblas_idamin(int n, const double *x, int incx);

/* ---- library statistics (the reference writes statistics.csv at exit,
 *      blas2cuda.c:266-273) -------------------------------------------------- */
void gbx_stats(uint64_t *calls, uint64_t *hits, uint64_t *misses, uint64_t *bytes_h2d,
               uint64_t *bytes_d2h);

#ifdef __cplusplus
}
#endif
#endif
