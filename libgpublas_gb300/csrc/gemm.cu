// gemm.cu — plain FP64 Level-3 routines on the DFMA GEMM core:
// gbx_dgemm, gbx_zgemm, gbx_dsyrk, gbx_dtrmm.
//
// Argument checks use the netlib INFO numbering that the reference's wrappers
// replicate (blas_level3/gemm.cc:87-127, syrk.cc:78-146, trmm.cc:82-137); on
// the device layer an invalid argument returns GBX_ERR_ARG and the position
// is recorded in the context's error text.  Unlike gemm.cc:121-125, beta == 0
// overwrites C, as the netlib specification requires.
#include "gbx_internal.h"
#include "gemm_simt.cuh"
#include "gemm_host.h"

#include <cuda_runtime.h>
#include <algorithm>

using namespace gbx_gemm;

namespace {

inline cudaStream_t S(gbx_ctx *ctx) { return (cudaStream_t)gbx_ctx_get_stream(ctx); }

template <typename T>
__global__ void scale_matrix_kernel(int m, int n, T beta, T *C, long long ldc, int part)
{
    const long long total = (long long)m * n;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % m), j = (int)(t / m);
        if (part == C_LOWER && i < j) continue;
        if (part == C_UPPER && i > j) continue;
        T *cp = C + (long long)j * ldc + i;
        *cp = Ops<T>::is_zero(beta) ? Ops<T>::zero() : Ops<T>::mul(beta, *cp);
    }
}

}  // namespace

namespace gbx_gemm {

template <typename T>
gbx_status scale_matrix(gbx_ctx *ctx, int m, int n, T beta, T *C, long long ldc, int part)
{
    if (m <= 0 || n <= 0) return GBX_OK;
    long long total = (long long)m * n;
    long long g = std::min<long long>((total + 255) / 256, (long long)gbx_ctx_sms(ctx) * 8);
    scale_matrix_kernel<T><<<(int)g, 256, 0, S(ctx)>>>(m, n, beta, C, ldc, part);
    gbx_count_launch(ctx, 1);
    return gbx_check_launch(ctx, "scale_matrix");
}
template gbx_status scale_matrix<double>(gbx_ctx *, int, int, double, double *, long long, int);
template gbx_status scale_matrix<dcplx>(gbx_ctx *, int, int, dcplx, dcplx *, long long, int);

template <typename T, int TM>
gbx_status launch_gemm_tile(gbx_ctx *ctx, GemmArgs<T> p, const char *what)
{
    constexpr int TN = TM, BK = 8;
    constexpr int BM = 16 * TM, BN = 16 * TN;
    p.tiles_m = (p.m + BM - 1) / BM;
    p.tiles_n = (p.n + BN - 1) / BN;
    long long blocks;
    if (p.c_part == C_FULL) blocks = (long long)p.tiles_m * p.tiles_n;
    else {
        if (p.m != p.n) return gbx_fail(ctx, GBX_ERR_ARG, "%s: triangular C must be square", what);
        blocks = (long long)p.tiles_m * (p.tiles_m + 1) / 2;
    }
    if (blocks > 0x7fffffffLL) return gbx_fail(ctx, GBX_ERR_UNSUPPORTED, "%s: grid too large", what);
    gbx_timer_begin(ctx, GBX_TIMER_GEMM_FP64);
    gemm_simt_kernel<T, TM, TN, BK><<<(unsigned)blocks, GEMM_THREADS, 0, S(ctx)>>>(p);
    gbx_timer_end(ctx);
    gbx_count_launch(ctx, 1);
    return gbx_check_launch(ctx, what);
}

// Tile choice: the largest block tile that still gives every SM two tiles;
// 128x128 (8x8 per thread) for large problems, 64x64 and 32x32 for the
// skinny and small products that DTRSM's recursion and small calls produce
// (with few large tiles most SMs would idle).  Complex uses 64x64 / 32x32.
template <typename T>
gbx_status launch_gemm(gbx_ctx *ctx, GemmArgs<T> p, const char *what)
{
    if (p.m <= 0 || p.n <= 0) return GBX_OK;
    const long long want = 2LL * gbx_ctx_sms(ctx);
    auto tiles = [&](int bm) {
        const long long tm = (p.m + bm - 1) / bm, tn = (p.n + bm - 1) / bm;
        return p.c_part == C_FULL ? tm * tn : tm * (tm + 1) / 2;
    };
    if constexpr (sizeof(T) == 8) {
        if (tiles(128) >= want) return launch_gemm_tile<T, 8>(ctx, p, what);
        if (tiles(64) >= want) return launch_gemm_tile<T, 4>(ctx, p, what);
        return launch_gemm_tile<T, 2>(ctx, p, what);
    } else {
        if (tiles(64) >= want) return launch_gemm_tile<T, 4>(ctx, p, what);
        return launch_gemm_tile<T, 2>(ctx, p, what);
    }
}
template gbx_status launch_gemm<double>(gbx_ctx *, GemmArgs<double>, const char *);
template gbx_status launch_gemm<dcplx>(gbx_ctx *, GemmArgs<dcplx>, const char *);

}  // namespace gbx_gemm

// ------------------------------------------------------------------ checks
extern "C" int gbx_check_gemm_args(char ta, char tb, int m, int n, int k, int lda, int ldb, int ldc)
{
    const int nota = gbx_lsame(ta, 'N'), notb = gbx_lsame(tb, 'N');
    const int nrowa = nota ? m : k, nrowb = notb ? k : n;
    if (!nota && !gbx_lsame(ta, 'C') && !gbx_lsame(ta, 'T')) return 1;
    if (!notb && !gbx_lsame(tb, 'C') && !gbx_lsame(tb, 'T')) return 2;
    if (m < 0) return 3;
    if (n < 0) return 4;
    if (k < 0) return 5;
    if (lda < std::max(1, nrowa)) return 8;
    if (ldb < std::max(1, nrowb)) return 10;
    if (ldc < std::max(1, m)) return 13;
    return 0;
}

extern "C" int gbx_check_syrk_args(char uplo, char trans, int n, int k, int lda, int ldc)
{
    const int nrowa = gbx_lsame(trans, 'N') ? n : k;
    if (!gbx_lsame(uplo, 'U') && !gbx_lsame(uplo, 'L')) return 1;
    if (!gbx_lsame(trans, 'N') && !gbx_lsame(trans, 'T') && !gbx_lsame(trans, 'C')) return 2;
    if (n < 0) return 3;
    if (k < 0) return 4;
    if (lda < std::max(1, nrowa)) return 7;
    if (ldc < std::max(1, n)) return 10;
    return 0;
}

extern "C" int gbx_check_trxm_args(char side, char uplo, char ta, char diag, int m, int n, int lda,
                                   int ldb)
{
    const int lside = gbx_lsame(side, 'L');
    const int nrowa = lside ? m : n;
    if (!lside && !gbx_lsame(side, 'R')) return 1;
    if (!gbx_lsame(uplo, 'U') && !gbx_lsame(uplo, 'L')) return 2;
    if (!gbx_lsame(ta, 'N') && !gbx_lsame(ta, 'T') && !gbx_lsame(ta, 'C')) return 3;
    if (!gbx_lsame(diag, 'U') && !gbx_lsame(diag, 'N')) return 4;
    if (m < 0) return 5;
    if (n < 0) return 6;
    if (lda < std::max(1, nrowa)) return 9;
    if (ldb < std::max(1, m)) return 11;
    return 0;
}

// ------------------------------------------------------------------- DGEMM
extern "C" gbx_status gbx_dgemm(gbx_ctx *ctx, char ta, char tb, int m, int n, int k, double alpha,
                                const double *A, int lda, const double *B, int ldb, double beta,
                                double *C, int ldc)
{
    if (!ctx) return GBX_ERR_ARG;
    int info = gbx_check_gemm_args(ta, tb, m, n, k, lda, ldb, ldc);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "DGEMM parameter %d", info);
    if (m == 0 || n == 0 || ((alpha == 0.0 || k == 0) && beta == 1.0)) return GBX_OK;
    if (alpha == 0.0 || k == 0) return scale_matrix<double>(ctx, m, n, beta, C, ldc, C_FULL);
    GemmArgs<double> p{};
    p.m = m; p.n = n; p.k = k;
    p.A = A; p.lda = lda; p.ta = !gbx_lsame(ta, 'N');
    p.B = B; p.ldb = ldb; p.tb = !gbx_lsame(tb, 'N');
    p.alpha = alpha; p.beta = beta;
    p.C = C; p.ldc = ldc;
    return launch_gemm<double>(ctx, p, "dgemm");
}

// ------------------------------------------------------------------- ZGEMM
extern "C" gbx_status gbx_zgemm(gbx_ctx *ctx, char ta, char tb, int m, int n, int k,
                                const double *alpha, const double *A, int lda, const double *B,
                                int ldb, const double *beta, double *C, int ldc)
{
    if (!ctx || !alpha || !beta) return GBX_ERR_ARG;
    int info = gbx_check_gemm_args(ta, tb, m, n, k, lda, ldb, ldc);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "ZGEMM parameter %d", info);
    const dcplx al{alpha[0], alpha[1]}, be{beta[0], beta[1]};
    const bool alpha0 = al.x == 0.0 && al.y == 0.0, beta1 = be.x == 1.0 && be.y == 0.0;
    if (m == 0 || n == 0 || ((alpha0 || k == 0) && beta1)) return GBX_OK;
    if (alpha0 || k == 0) return scale_matrix<dcplx>(ctx, m, n, be, (dcplx *)C, ldc, C_FULL);
    GemmArgs<dcplx> p{};
    p.m = m; p.n = n; p.k = k;
    p.A = (const dcplx *)A; p.lda = lda; p.ta = !gbx_lsame(ta, 'N'); p.conja = gbx_lsame(ta, 'C');
    p.B = (const dcplx *)B; p.ldb = ldb; p.tb = !gbx_lsame(tb, 'N'); p.conjb = gbx_lsame(tb, 'C');
    p.alpha = al; p.beta = be;
    p.C = (dcplx *)C; p.ldc = ldc;
    return launch_gemm<dcplx>(ctx, p, "zgemm");
}

// ------------------------------------------------------------------- DSYRK
extern "C" gbx_status gbx_dsyrk(gbx_ctx *ctx, char uplo, char trans, int n, int k, double alpha,
                                const double *A, int lda, double beta, double *C, int ldc)
{
    if (!ctx) return GBX_ERR_ARG;
    int info = gbx_check_syrk_args(uplo, trans, n, k, lda, ldc);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "DSYRK parameter %d", info);
    if (n == 0 || ((alpha == 0.0 || k == 0) && beta == 1.0)) return GBX_OK;
    const int part = gbx_lsame(uplo, 'U') ? C_UPPER : C_LOWER;
    if (alpha == 0.0 || k == 0) return scale_matrix<double>(ctx, n, n, beta, C, ldc, part);
    const bool notr = gbx_lsame(trans, 'N');
    GemmArgs<double> p{};
    p.m = n; p.n = n; p.k = k;
    p.A = A; p.lda = lda; p.ta = !notr;   // N: op(A) = A (n x k);  T: op(A) = A^T
    p.B = A; p.ldb = lda; p.tb = notr;    // N: op(B) = A^T;        T: op(B) = A (k x n)
    p.alpha = alpha; p.beta = beta;
    p.C = C; p.ldc = ldc;
    p.c_part = part;
    return launch_gemm<double>(ctx, p, "dsyrk");
}

// ------------------------------------------------------------------- DTRMM
// Effective triangle of op(A): transposing swaps lower and upper.
extern "C" int gbx_op_tri(char uplo, char transa, char diag)
{
    const bool lower = gbx_lsame(uplo, 'L');
    const bool notr = gbx_lsame(transa, 'N');
    int t = (lower == notr) ? TRI_LOWER : TRI_UPPER;
    if (gbx_lsame(diag, 'U')) t |= TRI_UNIT;
    return t;
}

extern "C" gbx_status gbx_dtrmm(gbx_ctx *ctx, char side, char uplo, char ta, char diag, int m,
                                int n, double alpha, const double *A, int lda, double *B, int ldb)
{
    if (!ctx) return GBX_ERR_ARG;
    int info = gbx_check_trxm_args(side, uplo, ta, diag, m, n, lda, ldb);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "DTRMM parameter %d", info);
    if (m == 0 || n == 0) return GBX_OK;
    if (alpha == 0.0) return scale_matrix<double>(ctx, m, n, 0.0, B, ldb, C_FULL);
    // The product is formed out of place: B is copied to workspace first.
    double *Bc;
    gbx_status st = gbx_ws(ctx, 0, sizeof(double) * (size_t)m * n, (void **)&Bc);
    if (st != GBX_OK) return st;
    cudaError_t e = cudaMemcpy2DAsync(Bc, sizeof(double) * (size_t)m, B, sizeof(double) * (size_t)ldb,
                                      sizeof(double) * (size_t)m, n, cudaMemcpyDeviceToDevice, S(ctx));
    if (e != cudaSuccess) return gbx_fail(ctx, GBX_ERR_CUDA, "dtrmm copy: %s", cudaGetErrorString(e));
    const int tri = gbx_op_tri(uplo, ta, diag);
    const bool tr = !gbx_lsame(ta, 'N');
    GemmArgs<double> p{};
    p.m = m; p.n = n;
    p.alpha = alpha; p.beta = 0.0;
    p.C = B; p.ldc = ldb;
    if (gbx_lsame(side, 'L')) {
        p.k = m;
        p.A = A; p.lda = lda; p.ta = tr; p.tri_a = tri;
        p.B = Bc; p.ldb = m; p.tb = 0;
    } else {
        p.k = n;
        p.A = Bc; p.lda = m; p.ta = 0;
        p.B = A; p.ldb = lda; p.tb = tr; p.tri_b = tri;
    }
    return launch_gemm<double>(ctx, p, "dtrmm");
}
