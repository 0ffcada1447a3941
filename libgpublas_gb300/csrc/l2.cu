// l2.cu — gbx_dgemv: y := alpha*op(A)*x + beta*y, HBM-bound streaming kernels.
//
// Replaces the reference's dead CBLAS wrapper blas_level2/gemv.cc:11-98 (which
// transposed row-major inputs through cublasDgeam before cublasDgemv).  The
// matrix is read exactly once:
//   * 'N': a 2-D grid of (512-row tile) x (column chunk) blocks; each thread
//     owns two adjacent rows (one 128-bit load per column when the columns are
//     16-byte aligned) and walks its chunk of columns; per-chunk partial
//     results are combined in a fixed order by a second kernel that also
//     applies alpha and beta (deterministic);
//   * 'T'/'C': one warp per column (contiguous in memory) with 128-bit loads
//     and a shuffle reduction, or one block per column when there are too few
//     columns to fill the GPU.
#include "gbx_internal.h"

#include <cuda_runtime.h>
#include <stdint.h>
#include <algorithm>

namespace {

constexpr int GEMV_THREADS = 256;
constexpr int ROWS_PER_BLOCK = 2 * GEMV_THREADS;

inline cudaStream_t S(gbx_ctx *ctx) { return (cudaStream_t)gbx_ctx_get_stream(ctx); }
inline long long base_off(int n, int inc) { return inc >= 0 ? 0 : (long long)(n - 1) * (-inc); }

__global__ void __launch_bounds__(GEMV_THREADS)
gemv_n_partial(int m, int n, int chunk, const double *__restrict__ A, long long lda,
               const double *__restrict__ x, int incx, double *__restrict__ part, int vec)
{
    const int r = blockIdx.x * ROWS_PER_BLOCK + 2 * threadIdx.x;
    const int c0 = blockIdx.y * chunk;
    const int c1 = min(n, c0 + chunk);
    double s0 = 0.0, s1 = 0.0, t0 = 0.0, t1 = 0.0;
    if (vec && r + 1 < m) {
        const double *ap = A + (long long)c0 * lda + r;
        int c = c0;
        for (; c + 4 <= c1; c += 4) {
            const double2 a0 = __ldg((const double2 *)(ap));
            const double2 a1 = __ldg((const double2 *)(ap + lda));
            const double2 a2 = __ldg((const double2 *)(ap + 2 * lda));
            const double2 a3 = __ldg((const double2 *)(ap + 3 * lda));
            const double x0 = __ldg(x + (long long)c * incx), x1 = __ldg(x + (long long)(c + 1) * incx);
            const double x2 = __ldg(x + (long long)(c + 2) * incx), x3 = __ldg(x + (long long)(c + 3) * incx);
            // two chains per row: the FP64 pipe is the bound, so its
            // dependent-latency gaps must be covered within the warp
            s0 = fma(a0.x, x0, s0); s1 = fma(a0.y, x0, s1);
            t0 = fma(a1.x, x1, t0); t1 = fma(a1.y, x1, t1);
            s0 = fma(a2.x, x2, s0); s1 = fma(a2.y, x2, s1);
            t0 = fma(a3.x, x3, t0); t1 = fma(a3.y, x3, t1);
            ap += 4 * lda;
        }
        s0 += t0;
        s1 += t1;
        for (; c < c1; c++) {
            const double2 a0 = __ldg((const double2 *)(ap));
            const double xv = __ldg(x + (long long)c * incx);
            s0 = fma(a0.x, xv, s0); s1 = fma(a0.y, xv, s1);
            ap += lda;
        }
    } else {
        for (int c = c0; c < c1; c++) {
            const double xv = __ldg(x + (long long)c * incx);
            if (r < m) s0 = fma(__ldg(A + (long long)c * lda + r), xv, s0);
            if (r + 1 < m) s1 = fma(__ldg(A + (long long)c * lda + r + 1), xv, s1);
        }
    }
    double *pp = part + (long long)blockIdx.y * m;
    if (r < m) pp[r] = s0;
    if (r + 1 < m) pp[r + 1] = s1;
}

__global__ void __launch_bounds__(GEMV_THREADS)
gemv_n_finish(int m, int nchunks, const double *__restrict__ part, double alpha, double beta,
              double *__restrict__ y, int incy)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int c = 0; c < nchunks; c++) s += part[(long long)c * m + i];
        double *yp = y + (long long)i * incy;
        *yp = (beta == 0.0) ? alpha * s : fma(beta, *yp, alpha * s);
    }
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// one warp per column
__global__ void __launch_bounds__(GEMV_THREADS)
gemv_t_warp(int m, int n, const double *__restrict__ A, long long lda, const double *__restrict__ x,
            int incx, double alpha, double beta, double *__restrict__ y, int incy, int vec)
{
    const int lane = threadIdx.x & 31;
    const int j = blockIdx.x * (GEMV_THREADS / 32) + (threadIdx.x >> 5);
    if (j >= n) return;
    const double *col = A + (long long)j * lda;
    double s0 = 0.0, s1 = 0.0;
    if (vec) {
        const int m2 = m >> 1;
        double s2 = 0.0, s3 = 0.0;
        int i = lane;
        for (; i + 32 < m2; i += 64) {
            const double2 a = __ldg((const double2 *)col + i), b = __ldg((const double2 *)col + i + 32);
            const double2 xv = __ldg((const double2 *)x + i), xw = __ldg((const double2 *)x + i + 32);
            s0 = fma(a.x, xv.x, s0);
            s1 = fma(a.y, xv.y, s1);
            s2 = fma(b.x, xw.x, s2);
            s3 = fma(b.y, xw.y, s3);
        }
        for (; i < m2; i += 32) {
            const double2 a = __ldg((const double2 *)col + i);
            const double2 xv = __ldg((const double2 *)x + i);
            s0 = fma(a.x, xv.x, s0);
            s1 = fma(a.y, xv.y, s1);
        }
        s0 += s2;
        s1 += s3;
        if ((m & 1) && lane == 0) s0 = fma(col[m - 1], x[m - 1], s0);
    } else {
        for (int i = lane; i < m; i += 32) s0 = fma(__ldg(col + i), __ldg(x + (long long)i * incx), s0);
    }
    const double s = warp_sum(s0 + s1);
    if (lane == 0) {
        double *yp = y + (long long)j * incy;
        *yp = (beta == 0.0) ? alpha * s : fma(beta, *yp, alpha * s);
    }
}

// one block per column, for short-and-tall problems
__global__ void __launch_bounds__(GEMV_THREADS)
gemv_t_block(int m, int n, const double *__restrict__ A, long long lda, const double *__restrict__ x,
             int incx, double alpha, double beta, double *__restrict__ y, int incy)
{
    __shared__ double sw[GEMV_THREADS / 32];
    const int j = blockIdx.x;
    const double *col = A + (long long)j * lda;
    double s = 0.0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) s = fma(__ldg(col + i), __ldg(x + (long long)i * incx), s);
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < GEMV_THREADS / 32 ? sw[threadIdx.x] : 0.0;
        v = warp_sum(v);
        if (threadIdx.x == 0) {
            double *yp = y + (long long)j * incy;
            *yp = (beta == 0.0) ? alpha * v : fma(beta, *yp, alpha * v);
        }
    }
}

__global__ void gemv_scale_y(int len, double beta, double *y, int incy)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) {
        double *yp = y + (long long)i * incy;
        *yp = (beta == 0.0) ? 0.0 : beta * *yp;
    }
}

}  // namespace

extern "C" int gbx_check_gemv_args(char trans, int m, int n, int lda, int incx, int incy)
{
    if (!gbx_lsame(trans, 'N') && !gbx_lsame(trans, 'T') && !gbx_lsame(trans, 'C')) return 1;
    if (m < 0) return 2;
    if (n < 0) return 3;
    if (lda < std::max(1, m)) return 6;
    if (incx == 0) return 8;
    if (incy == 0) return 11;
    return 0;
}

extern "C" gbx_status gbx_dgemv(gbx_ctx *ctx, char trans, int m, int n, double alpha,
                                const double *A, int lda, const double *x, int incx, double beta,
                                double *y, int incy)
{
    if (!ctx) return GBX_ERR_ARG;
    int info = gbx_check_gemv_args(trans, m, n, lda, incx, incy);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "DGEMV parameter %d", info);
    if (m == 0 || n == 0 || (alpha == 0.0 && beta == 1.0)) return GBX_OK;
    const bool notr = gbx_lsame(trans, 'N');
    const int lenx = notr ? n : m, leny = notr ? m : n;
    const double *xb = x + base_off(lenx, incx);
    double *yb = y + base_off(leny, incy);
    const int sms = gbx_ctx_sms(ctx);
    if (alpha == 0.0) {
        gemv_scale_y<<<std::min(sms * 4, (leny + 255) / 256), 256, 0, S(ctx)>>>(leny, beta, yb, incy);
        gbx_count_launch(ctx, 1);
        return gbx_check_launch(ctx, "dgemv");
    }
    if (notr) {
        const int rtiles = (m + ROWS_PER_BLOCK - 1) / ROWS_PER_BLOCK;
        int nchunks = std::max(1, (sms * 4 + rtiles - 1) / rtiles);
        nchunks = std::min(nchunks, std::max(1, n / 16));
        nchunks = std::min(nchunks, 65535);
        const int chunk = (n + nchunks - 1) / nchunks;
        nchunks = (n + chunk - 1) / chunk;
        double *part;
        gbx_status st = gbx_ws(ctx, GBX_WS_GEMV, sizeof(double) * (size_t)nchunks * m, (void **)&part);
        if (st != GBX_OK) return st;
        const int vec = ((((uintptr_t)A) & 15) == 0) && (lda % 2 == 0);
        dim3 g(rtiles, nchunks);
        gbx_timer_begin(ctx, GBX_TIMER_GEMV);
        gemv_n_partial<<<g, GEMV_THREADS, 0, S(ctx)>>>(m, n, chunk, A, lda, xb, incx, part, vec);
        gbx_timer_end(ctx);
        gemv_n_finish<<<std::min(sms * 4, (m + 255) / 256), 256, 0, S(ctx)>>>(m, nchunks, part, alpha,
                                                                               beta, yb, incy);
        gbx_count_launch(ctx, 2);
        return gbx_check_launch(ctx, "dgemv");
    }
    const int warps_per_block = GEMV_THREADS / 32;
    gbx_timer_begin(ctx, GBX_TIMER_GEMV);
    if (n >= sms * 4 * warps_per_block / 2) {
        const int vec = incx == 1 && ((((uintptr_t)A) & 15) == 0) && (lda % 2 == 0) &&
                        ((((uintptr_t)xb) & 15) == 0);
        gemv_t_warp<<<(n + warps_per_block - 1) / warps_per_block, GEMV_THREADS, 0, S(ctx)>>>(
            m, n, A, lda, xb, incx, alpha, beta, yb, incy, vec);
    } else {
        gemv_t_block<<<n, GEMV_THREADS, 0, S(ctx)>>>(m, n, A, lda, xb, incx, alpha, beta, yb, incy);
    }
    gbx_timer_end(ctx);
    gbx_count_launch(ctx, 1);
    return gbx_check_launch(ctx, "dgemv");
}
