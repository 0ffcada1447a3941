// level3.cu — the Level-3 BLAS on the SIMT GEMM core, for S, D, C and Z:
// xGEMM, xSYMM, xHEMM, xSYRK, xHERK, xSYR2K, xHER2K and xTRMM (xTRSM is in
// trsm.cu).  These are the routines the reference exports from
// blas_level3/{gemm,symm,hemm,syrk,herk,syr2k,her2k,trmm}.cc, each of which
// forwards to the matching cuBLAS call after its argument check (for
// example gemm.cc:143-216, symm.cc:124-200, herk.cc:131-163).
//
// Every routine is one or two launches of gemm_simt_kernel:
//   * xSYMM / xHEMM read the symmetric operand from its stored triangle (the
//     loader mirrors, and conjugates for Hermitian, the other half);
//   * xSYRK / xHERK and xSYR2K / xHER2K run on the triangular tile grid of C;
//     the rank-2k forms are two passes (alpha op(A) op(B)' + beta C, then
//     alpha' op(B) op(A)' + C);
//   * Hermitian results get a real diagonal, as netlib sets it;
//   * xTRMM masks the triangular operand and forms the product out of place.
// Quick returns and beta == 0 follow netlib: beta == 0 sets C to zero.
#include "gbx_internal.h"
#include "gemm_host.h"

#include <cuda_runtime.h>

using namespace gbx_gemm;

namespace {

inline cudaStream_t S(gbx_ctx *ctx) { return (cudaStream_t)gbx_ctx_get_stream(ctx); }

// host-side scalar traits
template <typename T> struct H;
template <> struct H<float> {
    using R = float;
    static bool zero(float a) { return a == 0.0f; }
    static bool one(float a) { return a == 1.0f; }
    static float conj(float a) { return a; }
    static float real(float r) { return r; }
};
template <> struct H<double> {
    using R = double;
    static bool zero(double a) { return a == 0.0; }
    static bool one(double a) { return a == 1.0; }
    static double conj(double a) { return a; }
    static double real(double r) { return r; }
};
template <> struct H<fcplx> {
    using R = float;
    static bool zero(fcplx a) { return a.x == 0.0f && a.y == 0.0f; }
    static bool one(fcplx a) { return a.x == 1.0f && a.y == 0.0f; }
    static fcplx conj(fcplx a) { return {a.x, -a.y}; }
    static fcplx real(float r) { return {r, 0.0f}; }
};
template <> struct H<dcplx> {
    using R = double;
    static bool zero(dcplx a) { return a.x == 0.0 && a.y == 0.0; }
    static bool one(dcplx a) { return a.x == 1.0 && a.y == 0.0; }
    static dcplx conj(dcplx a) { return {a.x, -a.y}; }
    static dcplx real(double r) { return {r, 0.0}; }
};

template <typename T> T scalar(const typename H<T>::R *p) { return T{p[0], p[1]}; }

template <typename T>
gbx_status gemm_t(gbx_ctx *ctx, const char *nm, char ta, char tb, int m, int n, int k, T alpha, const T *A,
                  int lda, const T *B, int ldb, T beta, T *C, int ldc)
{
    if (!ctx) return GBX_ERR_ARG;
    const int info = gbx_check_gemm_args(ta, tb, m, n, k, lda, ldb, ldc);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "%s parameter %d", nm, info);
    if (m == 0 || n == 0 || ((H<T>::zero(alpha) || k == 0) && H<T>::one(beta))) return GBX_OK;
    if (H<T>::zero(alpha) || k == 0) return scale_matrix<T>(ctx, m, n, beta, C, ldc, C_FULL);
    GemmArgs<T> p{};
    p.m = m; p.n = n; p.k = k;
    p.A = A; p.lda = lda; p.ta = !gbx_lsame(ta, 'N'); p.conja = gbx_lsame(ta, 'C');
    p.B = B; p.ldb = ldb; p.tb = !gbx_lsame(tb, 'N'); p.conjb = gbx_lsame(tb, 'C');
    p.alpha = alpha; p.beta = beta;
    p.C = C; p.ldc = ldc;
    return launch_gemm<T>(ctx, p, nm);
}

template <typename T>
gbx_status symm_t(gbx_ctx *ctx, const char *nm, bool herm, char side, char uplo, int m, int n, T alpha,
                  const T *A, int lda, const T *B, int ldb, T beta, T *C, int ldc)
{
    if (!ctx) return GBX_ERR_ARG;
    const int info = gbx_check_symm_args(side, uplo, m, n, lda, ldb, ldc);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "%s parameter %d", nm, info);
    if (m == 0 || n == 0 || (H<T>::zero(alpha) && H<T>::one(beta))) return GBX_OK;
    if (H<T>::zero(alpha)) return scale_matrix<T>(ctx, m, n, beta, C, ldc, C_FULL);
    const int sym = (gbx_lsame(uplo, 'L') ? SYM_LOWER : SYM_UPPER) | (herm ? SYM_HERM : 0);
    GemmArgs<T> p{};
    p.m = m; p.n = n;
    p.alpha = alpha; p.beta = beta;
    p.C = C; p.ldc = ldc;
    if (gbx_lsame(side, 'L')) {   // C = alpha A B + beta C, A m x m
        p.k = m;
        p.A = A; p.lda = lda; p.sym_a = sym;
        p.B = B; p.ldb = ldb;
    } else {                      // C = alpha B A + beta C, A n x n
        p.k = n;
        p.A = B; p.lda = ldb;
        p.B = A; p.ldb = lda; p.sym_b = sym;
    }
    return launch_gemm<T>(ctx, p, nm);
}

// C = alpha op(A) op(A)' + beta C on one triangle; ' is ^T (symmetric) or
// ^H (Hermitian, alpha and beta real).
template <typename T>
gbx_status syrk_t(gbx_ctx *ctx, const char *nm, bool herm, int allowed, char uplo, char trans, int n, int k,
                  T alpha, const T *A, int lda, T beta, T *C, int ldc)
{
    if (!ctx) return GBX_ERR_ARG;
    const int info = gbx_check_rank_k_args(uplo, trans, allowed, n, k, lda, ldc);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "%s parameter %d", nm, info);
    if (n == 0 || ((H<T>::zero(alpha) || k == 0) && H<T>::one(beta))) return GBX_OK;
    const int part = gbx_lsame(uplo, 'U') ? C_UPPER : C_LOWER;
    if (H<T>::zero(alpha) || k == 0) return scale_matrix<T>(ctx, n, n, beta, C, ldc, part, herm);
    const bool notr = gbx_lsame(trans, 'N');
    GemmArgs<T> p{};
    p.m = n; p.n = n; p.k = k;
    p.A = A; p.lda = lda; p.ta = !notr; p.conja = herm && !notr;   // N: op(A) = A;   T/C: A^T / A^H
    p.B = A; p.ldb = lda; p.tb = notr; p.conjb = herm && notr;     // N: A^T / A^H;   T/C: A
    p.alpha = alpha; p.beta = beta;
    p.C = C; p.ldc = ldc;
    p.c_part = part;
    p.c_herm = herm;
    return launch_gemm<T>(ctx, p, nm);
}

// C = alpha op(A) op(B)' + alpha' op(B) op(A)' + beta C on one triangle;
// alpha' = alpha (symmetric) or conj(alpha) (Hermitian, beta real).
template <typename T>
gbx_status syr2k_t(gbx_ctx *ctx, const char *nm, bool herm, int allowed, char uplo, char trans, int n, int k,
                   T alpha, const T *A, int lda, const T *B, int ldb, T beta, T *C, int ldc)
{
    if (!ctx) return GBX_ERR_ARG;
    const int info = gbx_check_rank_2k_args(uplo, trans, allowed, n, k, lda, ldb, ldc);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "%s parameter %d", nm, info);
    if (n == 0 || ((H<T>::zero(alpha) || k == 0) && H<T>::one(beta))) return GBX_OK;
    const int part = gbx_lsame(uplo, 'U') ? C_UPPER : C_LOWER;
    if (H<T>::zero(alpha) || k == 0) return scale_matrix<T>(ctx, n, n, beta, C, ldc, part, herm);
    const bool notr = gbx_lsame(trans, 'N');
    GemmArgs<T> p{};
    p.m = n; p.n = n; p.k = k;
    p.ta = !notr; p.conja = herm && !notr;
    p.tb = notr; p.conjb = herm && notr;
    p.C = C; p.ldc = ldc;
    p.c_part = part;
    p.c_herm = herm;
    p.A = A; p.lda = lda; p.B = B; p.ldb = ldb;
    p.alpha = alpha; p.beta = beta;
    gbx_status st = launch_gemm<T>(ctx, p, nm);
    if (st != GBX_OK) return st;
    p.A = B; p.lda = ldb; p.B = A; p.ldb = lda;
    p.alpha = herm ? H<T>::conj(alpha) : alpha;
    p.beta = H<T>::real(1);
    return launch_gemm<T>(ctx, p, nm);
}

// B = alpha op(A) B or alpha B op(A), A triangular; formed out of place from
// a copy of B in workspace.
template <typename T>
gbx_status trmm_t(gbx_ctx *ctx, const char *nm, char side, char uplo, char ta, char diag, int m, int n, T alpha,
                  const T *A, int lda, T *B, int ldb)
{
    if (!ctx) return GBX_ERR_ARG;
    const int info = gbx_check_trxm_args(side, uplo, ta, diag, m, n, lda, ldb);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "%s parameter %d", nm, info);
    if (m == 0 || n == 0) return GBX_OK;
    if (H<T>::zero(alpha)) return scale_matrix<T>(ctx, m, n, alpha, B, ldb, C_FULL);
    T *Bc;
    gbx_status st = gbx_ws(ctx, GBX_WS_TMP0, sizeof(T) * (size_t)m * n, (void **)&Bc);
    if (st != GBX_OK) return st;
    cudaError_t e = cudaMemcpy2DAsync(Bc, sizeof(T) * (size_t)m, B, sizeof(T) * (size_t)ldb, sizeof(T) * (size_t)m,
                                      n, cudaMemcpyDeviceToDevice, S(ctx));
    if (e != cudaSuccess) return gbx_fail(ctx, GBX_ERR_CUDA, "%s copy: %s", nm, cudaGetErrorString(e));
    const int tri = gbx_op_tri(uplo, ta, diag);
    const bool tr = !gbx_lsame(ta, 'N'), cj = gbx_lsame(ta, 'C');
    GemmArgs<T> p{};
    p.m = m; p.n = n;
    p.alpha = alpha; p.beta = T{};
    p.C = B; p.ldc = ldb;
    if (gbx_lsame(side, 'L')) {
        p.k = m;
        p.A = A; p.lda = lda; p.ta = tr; p.conja = cj; p.tri_a = tri;
        p.B = Bc; p.ldb = m; p.tb = 0;
    } else {
        p.k = n;
        p.A = Bc; p.lda = m; p.ta = 0;
        p.B = A; p.ldb = lda; p.tb = tr; p.conjb = cj; p.tri_b = tri;
    }
    return launch_gemm<T>(ctx, p, nm);
}

}  // namespace

// ------------------------------------------------------------------- GEMM
extern "C" gbx_status gbx_sgemm(gbx_ctx *ctx, char ta, char tb, int m, int n, int k, float alpha, const float *A,
                                int lda, const float *B, int ldb, float beta, float *C, int ldc)
{
    return gemm_t<float>(ctx, "SGEMM", ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

extern "C" gbx_status gbx_dgemm(gbx_ctx *ctx, char ta, char tb, int m, int n, int k, double alpha,
                                const double *A, int lda, const double *B, int ldb, double beta, double *C,
                                int ldc)
{
    return gemm_t<double>(ctx, "DGEMM", ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

extern "C" gbx_status gbx_cgemm(gbx_ctx *ctx, char ta, char tb, int m, int n, int k, const float *alpha,
                                const float *A, int lda, const float *B, int ldb, const float *beta, float *C,
                                int ldc)
{
    if (!alpha || !beta) return GBX_ERR_ARG;
    return gemm_t<fcplx>(ctx, "CGEMM", ta, tb, m, n, k, scalar<fcplx>(alpha), (const fcplx *)A, lda,
                         (const fcplx *)B, ldb, scalar<fcplx>(beta), (fcplx *)C, ldc);
}

extern "C" gbx_status gbx_zgemm(gbx_ctx *ctx, char ta, char tb, int m, int n, int k, const double *alpha,
                                const double *A, int lda, const double *B, int ldb, const double *beta,
                                double *C, int ldc)
{
    if (!alpha || !beta) return GBX_ERR_ARG;
    return gemm_t<dcplx>(ctx, "ZGEMM", ta, tb, m, n, k, scalar<dcplx>(alpha), (const dcplx *)A, lda,
                         (const dcplx *)B, ldb, scalar<dcplx>(beta), (dcplx *)C, ldc);
}

// ------------------------------------------------------------ SYMM / HEMM
extern "C" gbx_status gbx_ssymm(gbx_ctx *ctx, char side, char uplo, int m, int n, float alpha, const float *A,
                                int lda, const float *B, int ldb, float beta, float *C, int ldc)
{
    return symm_t<float>(ctx, "SSYMM", false, side, uplo, m, n, alpha, A, lda, B, ldb, beta, C, ldc);
}

extern "C" gbx_status gbx_dsymm(gbx_ctx *ctx, char side, char uplo, int m, int n, double alpha, const double *A,
                                int lda, const double *B, int ldb, double beta, double *C, int ldc)
{
    return symm_t<double>(ctx, "DSYMM", false, side, uplo, m, n, alpha, A, lda, B, ldb, beta, C, ldc);
}

#define GBX_COMPLEX_SYMM(NAME, LABEL, T, R, HERM)                                                                \
    extern "C" gbx_status NAME(gbx_ctx *ctx, char side, char uplo, int m, int n, const R *alpha, const R *A,     \
                               int lda, const R *B, int ldb, const R *beta, R *C, int ldc)                      \
    {                                                                                                            \
        if (!alpha || !beta) return GBX_ERR_ARG;                                                                 \
        return symm_t<T>(ctx, LABEL, HERM, side, uplo, m, n, scalar<T>(alpha), (const T *)A, lda, (const T *)B, \
                         ldb, scalar<T>(beta), (T *)C, ldc);                                                     \
    }
GBX_COMPLEX_SYMM(gbx_csymm, "CSYMM", fcplx, float, false)
GBX_COMPLEX_SYMM(gbx_zsymm, "ZSYMM", dcplx, double, false)
GBX_COMPLEX_SYMM(gbx_chemm, "CHEMM", fcplx, float, true)
GBX_COMPLEX_SYMM(gbx_zhemm, "ZHEMM", dcplx, double, true)
#undef GBX_COMPLEX_SYMM

// ------------------------------------------------------------ SYRK / HERK
extern "C" gbx_status gbx_ssyrk(gbx_ctx *ctx, char uplo, char trans, int n, int k, float alpha, const float *A,
                                int lda, float beta, float *C, int ldc)
{
    return syrk_t<float>(ctx, "SSYRK", false, GBX_TR_N | GBX_TR_T | GBX_TR_C, uplo, trans, n, k, alpha, A, lda,
                         beta, C, ldc);
}

extern "C" gbx_status gbx_dsyrk(gbx_ctx *ctx, char uplo, char trans, int n, int k, double alpha, const double *A,
                                int lda, double beta, double *C, int ldc)
{
    return syrk_t<double>(ctx, "DSYRK", false, GBX_TR_N | GBX_TR_T | GBX_TR_C, uplo, trans, n, k, alpha, A, lda,
                          beta, C, ldc);
}

extern "C" gbx_status gbx_csyrk(gbx_ctx *ctx, char uplo, char trans, int n, int k, const float *alpha,
                                const float *A, int lda, const float *beta, float *C, int ldc)
{
    if (!alpha || !beta) return GBX_ERR_ARG;
    return syrk_t<fcplx>(ctx, "CSYRK", false, GBX_TR_N | GBX_TR_T, uplo, trans, n, k, scalar<fcplx>(alpha),
                         (const fcplx *)A, lda, scalar<fcplx>(beta), (fcplx *)C, ldc);
}

extern "C" gbx_status gbx_zsyrk(gbx_ctx *ctx, char uplo, char trans, int n, int k, const double *alpha,
                                const double *A, int lda, const double *beta, double *C, int ldc)
{
    if (!alpha || !beta) return GBX_ERR_ARG;
    return syrk_t<dcplx>(ctx, "ZSYRK", false, GBX_TR_N | GBX_TR_T, uplo, trans, n, k, scalar<dcplx>(alpha),
                         (const dcplx *)A, lda, scalar<dcplx>(beta), (dcplx *)C, ldc);
}

extern "C" gbx_status gbx_cherk(gbx_ctx *ctx, char uplo, char trans, int n, int k, float alpha, const float *A,
                                int lda, float beta, float *C, int ldc)
{
    return syrk_t<fcplx>(ctx, "CHERK", true, GBX_TR_N | GBX_TR_C, uplo, trans, n, k, H<fcplx>::real(alpha),
                         (const fcplx *)A, lda, H<fcplx>::real(beta), (fcplx *)C, ldc);
}

extern "C" gbx_status gbx_zherk(gbx_ctx *ctx, char uplo, char trans, int n, int k, double alpha, const double *A,
                                int lda, double beta, double *C, int ldc)
{
    return syrk_t<dcplx>(ctx, "ZHERK", true, GBX_TR_N | GBX_TR_C, uplo, trans, n, k, H<dcplx>::real(alpha),
                         (const dcplx *)A, lda, H<dcplx>::real(beta), (dcplx *)C, ldc);
}

// ---------------------------------------------------------- SYR2K / HER2K
extern "C" gbx_status gbx_ssyr2k(gbx_ctx *ctx, char uplo, char trans, int n, int k, float alpha, const float *A,
                                 int lda, const float *B, int ldb, float beta, float *C, int ldc)
{
    return syr2k_t<float>(ctx, "SSYR2K", false, GBX_TR_N | GBX_TR_T | GBX_TR_C, uplo, trans, n, k, alpha, A, lda,
                          B, ldb, beta, C, ldc);
}

extern "C" gbx_status gbx_dsyr2k(gbx_ctx *ctx, char uplo, char trans, int n, int k, double alpha,
                                 const double *A, int lda, const double *B, int ldb, double beta, double *C,
                                 int ldc)
{
    return syr2k_t<double>(ctx, "DSYR2K", false, GBX_TR_N | GBX_TR_T | GBX_TR_C, uplo, trans, n, k, alpha, A,
                           lda, B, ldb, beta, C, ldc);
}

extern "C" gbx_status gbx_csyr2k(gbx_ctx *ctx, char uplo, char trans, int n, int k, const float *alpha,
                                 const float *A, int lda, const float *B, int ldb, const float *beta, float *C,
                                 int ldc)
{
    if (!alpha || !beta) return GBX_ERR_ARG;
    return syr2k_t<fcplx>(ctx, "CSYR2K", false, GBX_TR_N | GBX_TR_T, uplo, trans, n, k, scalar<fcplx>(alpha),
                          (const fcplx *)A, lda, (const fcplx *)B, ldb, scalar<fcplx>(beta), (fcplx *)C, ldc);
}

extern "C" gbx_status gbx_zsyr2k(gbx_ctx *ctx, char uplo, char trans, int n, int k, const double *alpha,
                                 const double *A, int lda, const double *B, int ldb, const double *beta,
                                 double *C, int ldc)
{
    if (!alpha || !beta) return GBX_ERR_ARG;
    return syr2k_t<dcplx>(ctx, "ZSYR2K", false, GBX_TR_N | GBX_TR_T, uplo, trans, n, k, scalar<dcplx>(alpha),
                          (const dcplx *)A, lda, (const dcplx *)B, ldb, scalar<dcplx>(beta), (dcplx *)C, ldc);
}

extern "C" gbx_status gbx_cher2k(gbx_ctx *ctx, char uplo, char trans, int n, int k, const float *alpha,
                                 const float *A, int lda, const float *B, int ldb, float beta, float *C, int ldc)
{
    if (!alpha) return GBX_ERR_ARG;
    return syr2k_t<fcplx>(ctx, "CHER2K", true, GBX_TR_N | GBX_TR_C, uplo, trans, n, k, scalar<fcplx>(alpha),
                          (const fcplx *)A, lda, (const fcplx *)B, ldb, H<fcplx>::real(beta), (fcplx *)C, ldc);
}

extern "C" gbx_status gbx_zher2k(gbx_ctx *ctx, char uplo, char trans, int n, int k, const double *alpha,
                                 const double *A, int lda, const double *B, int ldb, double beta, double *C,
                                 int ldc)
{
    if (!alpha) return GBX_ERR_ARG;
    return syr2k_t<dcplx>(ctx, "ZHER2K", true, GBX_TR_N | GBX_TR_C, uplo, trans, n, k, scalar<dcplx>(alpha),
                          (const dcplx *)A, lda, (const dcplx *)B, ldb, H<dcplx>::real(beta), (dcplx *)C, ldc);
}

// ------------------------------------------------------------------- TRMM
extern "C" gbx_status gbx_strmm(gbx_ctx *ctx, char side, char uplo, char ta, char diag, int m, int n, float alpha,
                                const float *A, int lda, float *B, int ldb)
{
    return trmm_t<float>(ctx, "STRMM", side, uplo, ta, diag, m, n, alpha, A, lda, B, ldb);
}

extern "C" gbx_status gbx_dtrmm(gbx_ctx *ctx, char side, char uplo, char ta, char diag, int m, int n,
                                double alpha, const double *A, int lda, double *B, int ldb)
{
    return trmm_t<double>(ctx, "DTRMM", side, uplo, ta, diag, m, n, alpha, A, lda, B, ldb);
}

extern "C" gbx_status gbx_ctrmm(gbx_ctx *ctx, char side, char uplo, char ta, char diag, int m, int n,
                                const float *alpha, const float *A, int lda, float *B, int ldb)
{
    if (!alpha) return GBX_ERR_ARG;
    return trmm_t<fcplx>(ctx, "CTRMM", side, uplo, ta, diag, m, n, scalar<fcplx>(alpha), (const fcplx *)A, lda,
                         (fcplx *)B, ldb);
}

extern "C" gbx_status gbx_ztrmm(gbx_ctx *ctx, char side, char uplo, char ta, char diag, int m, int n,
                                const double *alpha, const double *A, int lda, double *B, int ldb)
{
    if (!alpha) return GBX_ERR_ARG;
    return trmm_t<dcplx>(ctx, "ZTRMM", side, uplo, ta, diag, m, n, scalar<dcplx>(alpha), (const dcplx *)A, lda,
                         (dcplx *)B, ldb);
}
