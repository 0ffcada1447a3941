// potrf.cu — Cholesky factorisation of one diagonal block, lower triangle.
// Not a BLAS routine: it is the diagonal step of the blocked right-looking
// Cholesky that drives the serving trace (the other steps are the
// intercepted dtrsm_/dsyrk_/dgemm_ calls).
//
// Blocked in 32-column steps.  On GB300 one SM does about 4 GFLOP/s of FP64,
// so a factorisation of a 256 x 256 block confined to one CTA costs over a
// millisecond; here only the 32 x 32 diagonal factorisations are serial:
//   * potrf_step(j0): every CTA factors the 32 x 32 diagonal block at j0 in
//     shared memory (redundantly: 5.5k FMAs), the last CTA to finish writes
//     it back, and each CTA solves 8 rows of the panel below against it
//     (x L^T = a, one warp per row);
//   * potrf_syrk(j0): the trailing update A22 -= A21 A21^T, one 16 x 16
//     lower tile per CTA (8k FMAs each).  The GEMM core would put this
//     product on one or two 128 x 128 tiles, i.e. one or two SMs: 63 µs for
//     a 64 x 64 x 64 update, most of the old 64-column version's 250 µs per
//     128 x 128 block.
// A non-positive pivot sets *info to its 1-based column (LAPACK convention,
// first failure wins); the rest of the block is then unspecified.
#include "gbx_internal.h"

#include <cuda_runtime.h>

namespace {

constexpr int PB = 32;          // panel width
constexpr int PT_THREADS = 256;
constexpr int PR = 8;           // panel rows per CTA (one warp per row)
static_assert(PB == 32 && PR * 32 == PT_THREADS, "the panel solve maps lane j to column j, one warp per row");

// One step j0: the diagonal block factor and the panel rows of this CTA.
// FP64 arithmetic retires two lanes per clock per SM on this part, so the
// step is spread thin: the 32 x 32 factor (about 5.5k FMAs) is repeated by
// every CTA and the panel below is split 8 rows per CTA; divisions and
// square roots, long dependent FP64 sequences, are replaced by one rsqrt per
// column (L_kk = d * rsqrt(d), the column and the panel scaled by rsqrt(d)).
// An FP64 warp instruction holds the SM's 2-lane FP64 pipe for 16 cycles
// whatever its predicate, so the trailing update of each column walks only
// the live triangle (a table of (row, column) pairs).
__global__ void __launch_bounds__(PT_THREADS)
potrf_step(int n, int j0, double *__restrict__ A, long long lda, int *__restrict__ info, unsigned *done)
{
    extern __shared__ double sm[];
    double(*L)[PB + 1] = (double(*)[PB + 1])sm;                   // diagonal block
    double(*X)[PB + 1] = (double(*)[PB + 1])(sm + PB * (PB + 1));  // this CTA's panel rows
    __shared__ double rinv[PB];
    __shared__ unsigned short tri[PB * (PB - 1) / 2];   // (r << 8 | c), c <= r < PB - 1, by r(r+1)/2 + c
    __shared__ int s_bad, s_last;
    const int tid = threadIdx.x;
    const int b = min(PB, n - j0);
    for (int t = tid; t < PB * (PB - 1) / 2; t += PT_THREADS) {
        int r = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
        while ((r + 1) * (r + 2) / 2 <= t) r++;
        while (r * (r + 1) / 2 > t) r--;
        tri[t] = (unsigned short)((r << 8) | (t - r * (r + 1) / 2));
    }
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
    // Right-looking factorisation of the diagonal block in shared memory,
    // one barrier per column.  The pivot of column k + 1 is formed by the
    // thread that finishes its last update (the first pair of column k's
    // update is (k+1, k+1)), the update of column k uses the unscaled column
    // times y^2, and column k is scaled during the next column's update
    // (which reads only column k + 1).
    auto pivot = [&](int k, double d) {
        if (!(d > 0.0)) {
            s_bad = k + 1;
        } else {
            const double y = rsqrt(d);
            L[k][k] = d * y;
            rinv[k] = y;
        }
    };
    if (tid == 0) pivot(0, L[0][0]);
    __syncthreads();
    for (int k = 0; k < b; k++) {
        if (s_bad) break;   // uniform: read after a barrier
        if (k > 0) {
            const double yp = rinv[k - 1];
            for (int i = k + tid; i < b; i += PT_THREADS) L[i][k - 1] *= yp;
        }
        const double y = rinv[k], y2 = y * y;
        const int m = b - k - 1;
        for (int t = tid; t < m * (m + 1) / 2; t += PT_THREADS) {
            const int rc = tri[t];
            const int i = k + 1 + (rc >> 8), j = k + 1 + (rc & 255);
            const double v = fma(-L[i][k] * y2, L[j][k], L[i][j]);
            L[i][j] = v;
            if (t == 0) pivot(k + 1, v);
        }
        __syncthreads();
    }
    __syncthreads();
    if (!s_bad) {   // uniform over the CTA
        // panel: x L11^T = a for this CTA's rows, right-looking; one warp per
        // row, lane j owning column j (PB = 32)
        const int rr = tid >> 5, c = tid & 31;
        for (int k = 0; k < b; k++) {
            const double xk = X[rr][k] * rinv[k];
            if (c > k && c < b) X[rr][c] = fma(-xk, L[c][k], X[rr][c]);
            __syncwarp();
            if (c == k) X[rr][k] = xk;
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

// A22 (m x m, lower) -= A21 A21^T with A21 m x PB: one 16 x 16 tile of the
// lower triangle per CTA, blockIdx.x enumerating the tiles (ti >= tj) row by
// row; the two 16 x PB row blocks of A21 are staged in shared memory.
__global__ void __launch_bounds__(256)
potrf_syrk(int m, const double *__restrict__ A21, double *__restrict__ A22, long long lda)
{
    __shared__ double Li[16][PB + 1], Lj[16][PB + 1];
    const int b = blockIdx.x;
    int ti = (int)((sqrtf(8.0f * (float)b + 1.0f) - 1.0f) * 0.5f);
    while ((ti + 1) * (ti + 2) / 2 <= b) ti++;
    while (ti * (ti + 1) / 2 > b) ti--;
    const int tj = b - ti * (ti + 1) / 2;
    const int i0 = ti * 16, j0 = tj * 16;
    for (int t = threadIdx.x; t < 16 * PB; t += blockDim.x) {
        const int r = t & 15, k = t >> 4;
        Li[r][k] = i0 + r < m ? A21[(long long)k * lda + i0 + r] : 0.0;
        Lj[r][k] = j0 + r < m ? A21[(long long)k * lda + j0 + r] : 0.0;
    }
    __syncthreads();
    const int r = threadIdx.x & 15, c = threadIdx.x >> 4;
    const int gi = i0 + r, gj = j0 + c;
    if (gi >= m || gj > gi) return;
    double acc = 0.0;
#pragma unroll 8
    for (int k = 0; k < PB; k++) acc = fma(Li[r][k], Lj[c][k], acc);
    A22[(long long)gj * lda + gi] -= acc;
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
            const double *A21 = A + (long long)j0 * lda + j0 + b;
            double *A22 = A + (long long)(j0 + b) * lda + j0 + b;
            const int nt = (rows + 15) / 16;
            potrf_syrk<<<nt * (nt + 1) / 2, 256, 0, s>>>(rows, A21, A22, lda);
            gbx_count_launch(ctx, 1);
            if ((st = gbx_check_launch(ctx, "dpotrf_small update")) != GBX_OK) return st;
        }
    }
    return GBX_OK;
}
