// potrf.cu — Cholesky factorisation of one diagonal block, lower triangle.
// Not a BLAS routine: it is the diagonal step of the blocked right-looking
// Cholesky that drives the serving trace (the other steps are the
// intercepted dtrsm_/dsyrk_/dgemm_ calls).
//
// Blocked in 64-column steps.  On GB300 one SM does about 4 GFLOP/s of FP64,
// so a factorisation of a 256 x 256 block confined to one CTA costs over a
// millisecond; here only the 64 x 64 diagonal factorisations are serial:
//   * potrf_step(j0): every CTA factors the 64 x 64 diagonal block at j0 in
//     shared memory (redundantly: 44k FMAs), CTA 0 writes it back, and each
//     CTA solves 16 rows of the panel below against it (x L^T = a, 16
//     threads per row);
//   * the trailing update A22 -= A21 A21^T is one DSYRK on the GEMM core.
// A non-positive pivot sets *info to its 1-based column (LAPACK convention,
// first failure wins); the rest of the block is then unspecified.
#include "gbx_internal.h"

#include <cuda_runtime.h>

extern "C" gbx_status gbx_dsyrk(gbx_ctx *ctx, char uplo, char trans, int n, int k, double alpha, const double *A,
                                int lda, double beta, double *C, int ldc);

namespace {

constexpr int PB = 64;          // panel width
constexpr int PT_THREADS = 256;
constexpr int PR = 16;          // panel rows per CTA (16 threads per row)

// One step j0: the diagonal block factor and the panel rows of this CTA.
// FP64 arithmetic retires two lanes per clock per SM on this part, so the
// step is spread thin: the 64 x 64 factor (about 44k FMAs) is repeated by
// every CTA and the panel below is split 16 rows per CTA; divisions and
// square roots, long dependent FP64 sequences, are replaced by one rsqrt per
// column (L_kk = d * rsqrt(d), the column and the panel scaled by rsqrt(d)).
__global__ void __launch_bounds__(PT_THREADS)
potrf_step(int n, int j0, double *__restrict__ A, long long lda, int *__restrict__ info, unsigned *done)
{
    extern __shared__ double sm[];
    double(*L)[PB + 1] = (double(*)[PB + 1])sm;                   // diagonal block
    double(*X)[PB + 1] = (double(*)[PB + 1])(sm + PB * (PB + 1));  // this CTA's panel rows
    __shared__ double rinv[PB];
    __shared__ int s_bad, s_last;
    const int tid = threadIdx.x;
    const int b = min(PB, n - j0);
    for (int t = tid; t < PB * PB; t += PT_THREADS) {
        const int i = t % PB, k = t / PB;
        L[i][k] = (i < b && k < b && i >= k) ? A[(long long)(j0 + k) * lda + j0 + i] : (i == k ? 1.0 : 0.0);
    }
    // the panel rows are loaded now too (they do not depend on the factor)
    const int r0 = j0 + b + blockIdx.x * PR;
    for (int t = tid; t < PR * PB; t += PT_THREADS) {
        const int rr = t % PR, k = t / PR;
        X[rr][k] = (r0 + rr < n && k < b) ? A[(long long)(j0 + k) * lda + r0 + rr] : 0.0;
    }
    if (tid == 0) s_bad = 0;
    __syncthreads();
    // right-looking factorisation of the diagonal block in shared memory
    for (int k = 0; k < b; k++) {
        if (tid == 0) {
            const double d = L[k][k];
            if (!(d > 0.0)) {
                s_bad = k + 1;
            } else {
                const double y = rsqrt(d);
                L[k][k] = d * y;
                rinv[k] = y;
            }
        }
        __syncthreads();
        if (s_bad) break;
        const double y = rinv[k];
        for (int i = k + 1 + tid; i < b; i += PT_THREADS) L[i][k] *= y;
        __syncthreads();
        const int m = b - k - 1;
        for (int t = tid; t < m * m; t += PT_THREADS) {
            const int i = k + 1 + t % m, j = k + 1 + t / m;
            if (j <= i) L[i][j] = fma(-L[i][k], L[j][k], L[i][j]);
        }
        __syncthreads();
    }
    if (!s_bad) {   // uniform over the CTA
        // panel: x L11^T = a for this CTA's rows, right-looking; 16 threads
        // per row (a half warp) share the updates, column j to thread j % 16
        const int rr = tid >> 4, c = tid & 15;
        for (int k = 0; k < b; k++) {
            const double xk = X[rr][k] * rinv[k];
            for (int j = k + 1 + ((c - k - 1) & 15); j < b; j += 16) X[rr][j] = fma(-xk, L[j][k], X[rr][j]);
            __syncwarp();
            if (c == (k & 15)) X[rr][k] = xk;
            __syncwarp();
        }
        __syncthreads();
        for (int t = tid; t < PR * PB; t += PT_THREADS) {
            const int q = t % PR, k = t / PR;
            if (r0 + q < n && k < b) A[(long long)(j0 + k) * lda + r0 + q] = X[q][k];
        }
    }
    // The factored diagonal block goes back to A only when every CTA has
    // read the original (the last CTA to finish writes it; all CTAs hold the
    // same factor), so no CTA can read a half-written block.
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        s_last = atomicAdd(done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    if (tid == 0) *done = 0u;
    if (s_bad) {
        if (tid == 0) atomicCAS(info, 0, j0 + s_bad);
        return;
    }
    for (int t = tid; t < b * b; t += PT_THREADS) {
        const int i = t % b, k = t / b;
        if (i >= k) A[(long long)(j0 + k) * lda + j0 + i] = L[i][k];
    }
}

}  // namespace

extern "C" gbx_status gbx_dpotrf_small(gbx_ctx *ctx, char uplo, int n, double *A, int lda, int *info)
{
    if (!ctx || !info) return GBX_ERR_ARG;
    if (!gbx_lsame(uplo, 'L')) return gbx_fail(ctx, GBX_ERR_UNSUPPORTED, "dpotrf_small: lower only");
    if (n < 0 || n > 256 || lda < (n > 1 ? n : 1))
        return gbx_fail(ctx, GBX_ERR_ARG, "dpotrf_small: n = %d (<= 256), lda = %d", n, lda);
    cudaStream_t s = (cudaStream_t)gbx_ctx_get_stream(ctx);
    int *words, *mirror;
    gbx_status st = gbx_ctx_status(ctx, &words, &mirror);   // word 12: the step's finish counter
    if (st != GBX_OK) return st;
    unsigned *done = (unsigned *)(words + 12);
    cudaMemsetAsync(info, 0, sizeof(int), s);
    constexpr size_t SMEM = 2 * sizeof(double) * PB * (PB + 1);
    cudaFuncSetAttribute(potrf_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM);
    for (int j0 = 0; j0 < n; j0 += PB) {
        const int b = n - j0 < PB ? n - j0 : PB;
        const int rows = n - j0 - b;
        const int grid = rows > 0 ? (rows + PR - 1) / PR : 1;
        potrf_step<<<grid, PT_THREADS, SMEM, s>>>(n, j0, A, lda, info, done);
        gbx_count_launch(ctx, 1);
        if ((st = gbx_check_launch(ctx, "dpotrf_small")) != GBX_OK) return st;
        if (rows > 0) {
            double *A21 = A + (long long)j0 * lda + j0 + b;
            double *A22 = A + (long long)(j0 + b) * lda + j0 + b;
            if ((st = gbx_dsyrk(ctx, 'L', 'N', rows, b, -1.0, A21, lda, 1.0, A22, lda)) != GBX_OK) return st;
        }
    }
    return GBX_OK;
}
