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

// Exact signed sum of products on the integer pipe, for a quarter of the
// products of the streaming DGEMV kernels.  Each matrix element is used once
// with one DFMA, and the FP64 pipe (2 lanes per clock per SM) caps that at
// about 5 TB/s of matrix; products moved to the integer pipe lift the cap
// above the HBM rate.  For finite a = ma 2^(ea - 1075) and x = mx 2^(ex -
// 1075) (53-bit significands, subnormals with exponent 1 and no hidden bit)
// the product is ma mx 2^(ea + ex - 2150); the accumulator is the signed
// 128-bit sum of ma mx 2^((ea + ex) - eref - 12), eref the largest exponent
// sum seen: a product at eref adds |ma mx| >> 12 < 2^94 (2^33 of them fit),
// a smaller one drops only its bits below 2^-94 of the largest product, and
// a larger exponent shifts the sum down first.
struct ProdFix {
    unsigned long long lo;
    long long hi;
    int eref;
    __device__ __forceinline__ void init() { lo = 0ull; hi = 0; eref = 0; }
    __device__ __forceinline__ void shift_down(int d)   // arithmetic
    {
        if (d >= 127) { hi = hi >> 63; lo = (unsigned long long)hi; }
        else if (d >= 64) { lo = (unsigned long long)(hi >> (d - 64)); hi >>= 63; }
        else if (d > 0) { lo = (lo >> d) | ((unsigned long long)hi << (64 - d)); hi >>= d; }
    }
    __device__ __forceinline__ void add(double a, double x)
    {
        const unsigned long long ba = (unsigned long long)__double_as_longlong(a);
        const unsigned long long bx = (unsigned long long)__double_as_longlong(x);
        const int ea = (int)((ba >> 52) & 0x7FF), ex = (int)((bx >> 52) & 0x7FF);
        const unsigned long long ma = (ba & 0xFFFFFFFFFFFFFull) | (ea ? 0x10000000000000ull : 0ull);
        const unsigned long long mx = (bx & 0xFFFFFFFFFFFFFull) | (ex ? 0x10000000000000ull : 0ull);
        const int e = max(ea, 1) + max(ex, 1);
        if (e > eref) {
            shift_down(e - eref);
            eref = e;
        }
        const int sh = 12 + (eref - e);
        const unsigned long long plo = ma * mx, phi = __umul64hi(ma, mx);   // < 2^106
        const int s1 = min(sh, 63), s2 = min(max(sh - 64, 0), 63);
        unsigned long long clo = sh < 64 ? (plo >> s1) | (phi << (64 - s1)) : (phi >> s2);
        unsigned long long chi = sh < 64 ? (phi >> s1) : 0ull;
        if (sh >= 106) { clo = 0ull; chi = 0ull; }
        // two's complement negation when the signs differ
        const unsigned long long neg = 0ull - ((ba ^ bx) >> 63);
        clo ^= neg;
        chi ^= neg;
        const unsigned long long c1 = clo + (neg & 1ull);
        chi += (c1 < clo) ? 1ull : 0ull;
        lo += c1;
        hi += (long long)chi + (lo < c1 ? 1 : 0);
    }
    // the sum as a double: acc * 2^(eref - 2150 + 12)
    __device__ __forceinline__ double value() const
    {
        if ((lo | (unsigned long long)hi) == 0ull) return 0.0;
        const double d = (hi == ((long long)lo >> 63)) ? (double)(long long)lo : fma((double)hi, 0x1p64, (double)lo);
        return ldexp(d, eref - 2138);
    }
};

// True when every active lane's operands are finite (integer tests on the
// high words): the integer products then stand in for the DFMAs exactly.
__device__ __forceinline__ bool all_finite3(double a, double b, double c)
{
    const auto hi = [](double v) { return (unsigned)(__double_as_longlong(v) >> 32) & 0x7FF00000u; };
    const bool bad = (hi(a) == 0x7FF00000u) | (hi(b) == 0x7FF00000u) | (hi(c) == 0x7FF00000u);
    return !__any_sync(__activemask(), bad);
}

__global__ void __launch_bounds__(GEMV_THREADS)
gemv_n_partial(int m, int n, int chunk, const double *__restrict__ A, long long lda,
               const double *__restrict__ x, int incx, double *__restrict__ part, int vec)
{
    const int r = blockIdx.x * ROWS_PER_BLOCK + 2 * threadIdx.x;
    const int c0 = blockIdx.y * chunk;
    const int c1 = min(n, c0 + chunk);
    double s0 = 0.0, s1 = 0.0;
    if (vec && r + 1 < m) {
        const double *ap = A + (long long)c0 * lda + r;
        int c = c0;
        ProdFix f0, f1;
        f0.init();
        f1.init();
        for (; c + 4 <= c1; c += 4) {
            const double2 a0 = __ldg((const double2 *)(ap));
            const double2 a1 = __ldg((const double2 *)(ap + lda));
            const double2 a2 = __ldg((const double2 *)(ap + 2 * lda));
            const double2 a3 = __ldg((const double2 *)(ap + 3 * lda));
            const double x0 = __ldg(x + (long long)c * incx), x1 = __ldg(x + (long long)(c + 1) * incx);
            const double x2 = __ldg(x + (long long)(c + 2) * incx), x3 = __ldg(x + (long long)(c + 3) * incx);
            s0 = fma(a0.x, x0, s0); s1 = fma(a0.y, x0, s1);
            s0 = fma(a1.x, x1, s0); s1 = fma(a1.y, x1, s1);
            s0 = fma(a2.x, x2, s0); s1 = fma(a2.y, x2, s1);
            if (all_finite3(a3.x, a3.y, x3)) {
                // a quarter of the products on the integer pipe
                f0.add(a3.x, x3);
                f1.add(a3.y, x3);
            } else {
                s0 = fma(a3.x, x3, s0); s1 = fma(a3.y, x3, s1);
            }
            ap += 4 * lda;
        }
        s0 += f0.value();
        s1 += f1.value();
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
        ProdFix f;
        f.init();
        int i = lane;
        for (; i + 32 < m2; i += 64) {
            const double2 a = __ldg((const double2 *)col + i), b = __ldg((const double2 *)col + i + 32);
            const double2 xv = __ldg((const double2 *)x + i), xw = __ldg((const double2 *)x + i + 32);
            s0 = fma(a.x, xv.x, s0);
            s1 = fma(a.y, xv.y, s1);
            s0 = fma(b.x, xw.x, s0);
            if (all_finite3(b.y, xw.y, 0.0)) f.add(b.y, xw.y);   // a quarter on the integer pipe
            else s1 = fma(b.y, xw.y, s1);
        }
        for (; i < m2; i += 32) {
            const double2 a = __ldg((const double2 *)col + i);
            const double2 xv = __ldg((const double2 *)x + i);
            s0 = fma(a.x, xv.x, s0);
            s1 = fma(a.y, xv.y, s1);
        }
        s1 += f.value();
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
