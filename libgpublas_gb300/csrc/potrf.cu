// potrf.cu — Cholesky factorisation of one small diagonal block (n <= 256),
// lower triangle, in one CTA.  Not a BLAS routine: it is the diagonal step of
// the blocked right-looking Cholesky that drives the serving trace (the
// other steps are the intercepted dtrsm_/dsyrk_/dgemm_ calls).
//
// Right-looking, column by column, in place in global memory (the block is
// small and stays in L1/L2): a_kk = sqrt(a_kk); a_ik /= a_kk; a_ij -= a_ik a_jk
// for i >= j > k.  A non-positive pivot sets *info = k+1 (1-based, LAPACK
// convention) and stops.
#include "gbx_internal.h"

#include <cuda_runtime.h>

namespace {

constexpr int PT_THREADS = 256;

__global__ void __launch_bounds__(PT_THREADS)
potrf_small_lower(int n, double *__restrict__ A, long long lda, int *__restrict__ info)
{
    __shared__ double s_piv;
    __shared__ int s_bad;
    if (threadIdx.x == 0) s_bad = 0;
    __syncthreads();
    for (int k = 0; k < n; k++) {
        if (threadIdx.x == 0) {
            const double d = A[(long long)k * lda + k];
            if (!(d > 0.0)) {
                s_bad = k + 1;
            } else {
                const double r = sqrt(d);
                A[(long long)k * lda + k] = r;
                s_piv = r;
            }
        }
        __syncthreads();
        if (s_bad) break;
        const double piv = s_piv;
        for (int i = k + 1 + threadIdx.x; i < n; i += PT_THREADS) A[(long long)k * lda + i] /= piv;
        __syncthreads();
        // trailing update of the lower triangle, one (i, j) pair per step
        const int m = n - k - 1;
        const long long pairs = (long long)m * (m + 1) / 2;
        for (long long t = threadIdx.x; t < pairs; t += PT_THREADS) {
            // t -> (jj, ii) with ii >= jj, column-major over the trailing triangle
            int jj = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
            while ((long long)(jj + 1) * (jj + 2) / 2 <= t) jj++;
            while ((long long)jj * (jj + 1) / 2 > t) jj--;
            const int ii = (int)(t - (long long)jj * (jj + 1) / 2);
            // map (jj, ii) with ii <= jj to row = k+1+jj, col = k+1+ii (row >= col)
            const int row = k + 1 + jj, col = k + 1 + ii;
            A[(long long)col * lda + row] =
                fma(-A[(long long)k * lda + row], A[(long long)k * lda + col], A[(long long)col * lda + row]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *info = s_bad;
}

}  // namespace

extern "C" gbx_status gbx_dpotrf_small(gbx_ctx *ctx, char uplo, int n, double *A, int lda, int *info)
{
    if (!ctx || !info) return GBX_ERR_ARG;
    if (!gbx_lsame(uplo, 'L')) return gbx_fail(ctx, GBX_ERR_UNSUPPORTED, "dpotrf_small: lower only");
    if (n < 0 || n > 256 || lda < (n > 1 ? n : 1))
        return gbx_fail(ctx, GBX_ERR_ARG, "dpotrf_small: n = %d (<= 256), lda = %d", n, lda);
    if (n == 0) {
        cudaMemsetAsync(info, 0, sizeof(int), (cudaStream_t)gbx_ctx_get_stream(ctx));
        return GBX_OK;
    }
    potrf_small_lower<<<1, PT_THREADS, 0, (cudaStream_t)gbx_ctx_get_stream(ctx)>>>(n, A, lda, info);
    gbx_count_launch(ctx, 1);
    return gbx_check_launch(ctx, "dpotrf_small");
}
