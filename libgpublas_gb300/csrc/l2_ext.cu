// l2_ext.cu — DGER, DSYMV and DTRSV: the Level-2 routines on either side of
// a Cholesky or TRSM step (rank-1 update, symmetric matrix-vector product,
// triangular solve with one right-hand side).  The reference lists them in
// blas_level2/ger.cc, symv.cc and trsv.cc (CBLAS bodies that its build
// leaves out, meson.build:53-75; prototypes blas.h:94-100, 134-142,
// 193-200).
//
//   * DGER: A += alpha x y^T streams A once (read + write, 16 B per FMA:
//     HBM-bound); 512-row x 32-column tiles, netlib's skip of zero y_j.
//   * DSYMV: y = alpha A x + beta y reads only the stored triangle.  Each
//     64x64 tile of the triangle is staged in shared memory and used twice
//     (A_IJ x_J for rows I and A_IJ^T x_I for rows J), so the kernel does 2
//     FMAs per 8 bytes: on GB300's FP64 pipe (2 lanes per clock per SM) that
//     is the bound, not HBM.  Per-tile partial vectors are summed in a fixed
//     order by a second kernel (deterministic).
//   * DTRSV: blocked substitution in 64-row steps.  The 64x64 diagonal blocks
//     of op(A) are inverted once (trinv_blocks of trsm.cu); step J is one
//     launch whose every CTA forms x_J = inv(A_JJ) b_J from the running
//     right-hand side and subtracts op(A)_IJ x_J from its rows I beyond J.
//     The running right-hand side lives in workspace, so no CTA reads what
//     another writes in the same launch.
#include "gbx_internal.h"
#include "gemm_host.h"

#include <cuda_runtime.h>
#include <stdint.h>
#include <algorithm>

namespace {

inline cudaStream_t S(gbx_ctx *ctx) { return (cudaStream_t)gbx_ctx_get_stream(ctx); }
inline long long base_off(int n, int inc) { return inc >= 0 ? 0 : (long long)(n - 1) * (-inc); }

// ------------------------------------------------------------------- DGER
constexpr int GER_ROWS = 512, GER_COLS = 32;

__global__ void __launch_bounds__(256)
ger_kernel(int m, int n, double alpha, const double *__restrict__ x, int incx, const double *__restrict__ y,
           int incy, double *__restrict__ A, long long lda)
{
    const int c0 = blockIdx.y * GER_COLS, c1 = min(n, c0 + GER_COLS);
    for (int i = blockIdx.x * GER_ROWS + threadIdx.x; i < min(m, (blockIdx.x + 1) * GER_ROWS); i += blockDim.x) {
        const double xi = __ldg(x + (long long)i * incx);
        double *ap = A + (long long)c0 * lda + i;
#pragma unroll 4
        for (int j = c0; j < c1; j++, ap += lda) {
            const double yj = __ldg(y + (long long)j * incy);
            if (yj != 0.0) *ap = fma(xi, alpha * yj, *ap);
        }
    }
}

// ------------------------------------------------------------------ DSYMV
constexpr int SY_T = 64;

// One tile (I, J) of the stored triangle per CTA (I >= J for lower, I <= J
// for upper in block indices).  Writes the row partial (A_IJ x_J, 64 values)
// to part[I][J] and, off the diagonal, the column partial (A_IJ^T x_I) to
// part[J][I]; part[b][q] is the q-th partial of output block b.
__global__ void __launch_bounds__(256)
symv_tiles(int n, int nb, int lower, const double *__restrict__ A, long long lda, const double *__restrict__ x,
           int incx, double *__restrict__ part)
{
    __shared__ double s[SY_T][SY_T + 1];
    __shared__ double sxI[SY_T], sxJ[SY_T];
    __shared__ double red[4][SY_T];
    // tile index -> (I, J) with I >= J (lower) in row-major triangle order
    const int t = blockIdx.x;
    int I = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while ((long long)(I + 1) * (I + 2) / 2 <= t) I++;
    while ((long long)I * (I + 1) / 2 > t) I--;
    int J = t - I * (I + 1) / 2;
    if (!lower) { const int tmp = I; I = J; J = tmp; }   // upper: I <= J
    const int r0 = I * SY_T, c0 = J * SY_T;
    const int tid = threadIdx.x;
    for (int q = tid; q < SY_T * SY_T; q += blockDim.x) {
        const int i = q % SY_T, j = q / SY_T;
        const int gi = r0 + i, gj = c0 + j;
        double v = 0.0;
        if (gi < n && gj < n) {
            if (I != J) v = A[(long long)gj * lda + gi];
            else {
                const bool stored = lower ? gi >= gj : gi <= gj;
                v = stored ? A[(long long)gj * lda + gi] : A[(long long)gi * lda + gj];   // mirror
            }
        }
        s[i][j] = v;
    }
    if (tid < SY_T) {
        sxJ[tid] = (c0 + tid < n) ? x[(long long)(c0 + tid) * incx] : 0.0;
        sxI[tid] = (r0 + tid < n) ? x[(long long)(r0 + tid) * incx] : 0.0;
    }
    __syncthreads();
    const int l = tid & (SY_T - 1), part4 = tid >> 6;
    // row sums: row l over columns part4*16 .. +15
    double r = 0.0;
#pragma unroll
    for (int j = 0; j < 16; j++) r = fma(s[l][part4 * 16 + j], sxJ[part4 * 16 + j], r);
    red[part4][l] = r;
    __syncthreads();
    double *rowp = part + ((size_t)I * nb + J) * SY_T;
    if (tid < SY_T) rowp[tid] = (red[0][tid] + red[1][tid]) + (red[2][tid] + red[3][tid]);
    if (I == J) return;
    __syncthreads();
    // column sums: column l over rows part4*16 .. +15
    double c = 0.0;
#pragma unroll
    for (int i = 0; i < 16; i++) c = fma(s[part4 * 16 + i][l], sxI[part4 * 16 + i], c);
    red[part4][l] = c;
    __syncthreads();
    double *colp = part + ((size_t)J * nb + I) * SY_T;
    if (tid < SY_T) colp[tid] = (red[0][tid] + red[1][tid]) + (red[2][tid] + red[3][tid]);
}

// y_i = alpha * sum_q part[b][q][i] + beta y_i  (beta == 0 sets y)
__global__ void __launch_bounds__(256)
symv_finish(int n, int nb, const double *__restrict__ part, double alpha, double beta, double *__restrict__ y,
            int incy)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int b = i / SY_T, l = i % SY_T;
        const double *p = part + (size_t)b * nb * SY_T + l;
        double s = 0.0;
        for (int q = 0; q < nb; q++) s += p[(size_t)q * SY_T];
        double *yp = y + (long long)i * incy;
        *yp = (beta == 0.0) ? alpha * s : fma(alpha, s, beta * *yp);
    }
}

// ------------------------------------------------------------------ DTRSV
constexpr int TV_NB = 64;

__global__ void gather_vec(int n, const double *__restrict__ x, int incx, double *__restrict__ w, int npad)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npad; i += gridDim.x * blockDim.x)
        w[i] = i < n ? x[(long long)i * incx] : 0.0;
}

// Step J (solve order position): every CTA computes x_J = inv_J b_J (64 x 64
// from the inverted diagonal blocks), CTA 0 stores it to x, and each CTA
// subtracts op(A)(rows, cols J) x_J from its 256 rows of the running
// right-hand side w (rows of the not yet solved blocks only).
//   fwd: op(A) lower, blocks solved in increasing order, updated rows below;
//   otherwise upper, decreasing order, updated rows above.
//   tr:  op(A) = A^T (A read transposed: a warp per row, lanes along k).
__global__ void __launch_bounds__(256)
trsv_step(int n, int J, int fwd, int tr, const double *__restrict__ A, long long lda, const double *__restrict__ inv,
          double *__restrict__ w, double *__restrict__ x, int incx)
{
    __shared__ double sx[TV_NB];
    __shared__ double sb[TV_NB];
    const int tid = threadIdx.x;
    const int c0 = J * TV_NB;
    if (tid < TV_NB) sb[tid] = w[c0 + tid];
    __syncthreads();
    const double *iv = inv + (size_t)J * TV_NB * TV_NB;
    if (tid < TV_NB) {
        double s = 0.0;
        for (int k = 0; k < TV_NB; k++) s = fma(iv[(size_t)k * TV_NB + tid], sb[k], s);
        sx[tid] = s;
        if (blockIdx.x == 0 && c0 + tid < n) x[(long long)(c0 + tid) * incx] = s;
    }
    __syncthreads();
    const int cols = min(TV_NB, n - c0);
    // rows this CTA updates: the 256-row slab blockIdx.x of the unsolved range
    const int lo = fwd ? c0 + TV_NB : 0, hi = fwd ? n : c0;
    const int rbeg = lo + blockIdx.x * 256;
    if (rbeg >= hi) return;
    if (!tr) {
        const int i = rbeg + tid;
        if (i >= hi) return;
        const double *ap = A + (long long)c0 * lda + i;
        double s = 0.0;
#pragma unroll 8
        for (int k = 0; k < cols; k++) s = fma(ap[(long long)k * lda], sx[k], s);
        w[i] -= s;
    } else {
        const int warp = tid >> 5, lane = tid & 31;
        for (int i = rbeg + warp; i < min(hi, rbeg + 256); i += 8) {
            const double *ap = A + (long long)i * lda + c0;   // op(A)(i, c0 + k) = A(c0 + k, i)
            double s = 0.0;
            if (lane < cols) s = ap[lane] * sx[lane];
            if (lane + 32 < cols) s = fma(ap[lane + 32], sx[lane + 32], s);
#pragma unroll
            for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) w[i] -= s;
        }
    }
}

}  // namespace

// ------------------------------------------------------------------ checks
extern "C" int gbx_check_ger_args(int m, int n, int incx, int incy, int lda)
{
    if (m < 0) return 1;
    if (n < 0) return 2;
    if (incx == 0) return 5;
    if (incy == 0) return 7;
    if (lda < std::max(1, m)) return 9;
    return 0;
}

extern "C" int gbx_check_symv_args(char uplo, int n, int lda, int incx, int incy)
{
    if (!gbx_lsame(uplo, 'U') && !gbx_lsame(uplo, 'L')) return 1;
    if (n < 0) return 2;
    if (lda < std::max(1, n)) return 5;
    if (incx == 0) return 7;
    if (incy == 0) return 10;
    return 0;
}

extern "C" int gbx_check_trsv_args(char uplo, char trans, char diag, int n, int lda, int incx)
{
    if (!gbx_lsame(uplo, 'U') && !gbx_lsame(uplo, 'L')) return 1;
    if (!gbx_lsame(trans, 'N') && !gbx_lsame(trans, 'T') && !gbx_lsame(trans, 'C')) return 2;
    if (!gbx_lsame(diag, 'U') && !gbx_lsame(diag, 'N')) return 3;
    if (n < 0) return 4;
    if (lda < std::max(1, n)) return 6;
    if (incx == 0) return 8;
    return 0;
}

// ------------------------------------------------------------ entry points
extern "C" gbx_status gbx_dger(gbx_ctx *ctx, int m, int n, double alpha, const double *x, int incx,
                               const double *y, int incy, double *A, int lda)
{
    if (!ctx) return GBX_ERR_ARG;
    const int info = gbx_check_ger_args(m, n, incx, incy, lda);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "DGER parameter %d", info);
    if (m == 0 || n == 0 || alpha == 0.0) return GBX_OK;
    dim3 g((m + GER_ROWS - 1) / GER_ROWS, (n + GER_COLS - 1) / GER_COLS);
    if (g.y > 65535) return gbx_fail(ctx, GBX_ERR_UNSUPPORTED, "DGER: n too large");
    gbx_timer_begin(ctx, GBX_TIMER_GEMV);
    ger_kernel<<<g, 256, 0, S(ctx)>>>(m, n, alpha, x + base_off(m, incx), incx, y + base_off(n, incy), incy, A,
                                      lda);
    gbx_timer_end(ctx);
    gbx_count_launch(ctx, 1);
    return gbx_check_launch(ctx, "dger");
}

extern "C" gbx_status gbx_dsymv(gbx_ctx *ctx, char uplo, int n, double alpha, const double *A, int lda,
                                const double *x, int incx, double beta, double *y, int incy)
{
    if (!ctx) return GBX_ERR_ARG;
    const int info = gbx_check_symv_args(uplo, n, lda, incx, incy);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "DSYMV parameter %d", info);
    if (n == 0 || (alpha == 0.0 && beta == 1.0)) return GBX_OK;
    const double *xb = x + base_off(n, incx);
    double *yb = y + base_off(n, incy);
    const int nb = (n + SY_T - 1) / SY_T;
    double *part;
    gbx_status st = gbx_ws(ctx, GBX_WS_GEMV, sizeof(double) * (size_t)nb * nb * SY_T, (void **)&part);
    if (st != GBX_OK) return st;
    const long long tiles = (long long)nb * (nb + 1) / 2;
    if (tiles > 0x7fffffffLL) return gbx_fail(ctx, GBX_ERR_UNSUPPORTED, "DSYMV: n too large");
    if (alpha != 0.0) {
        gbx_timer_begin(ctx, GBX_TIMER_GEMV);
        symv_tiles<<<(unsigned)tiles, 256, 0, S(ctx)>>>(n, nb, gbx_lsame(uplo, 'L'), A, lda, xb, incx, part);
        gbx_timer_end(ctx);
        gbx_count_launch(ctx, 1);
    } else {
        cudaMemsetAsync(part, 0, sizeof(double) * (size_t)nb * nb * SY_T, S(ctx));
    }
    const int sms = gbx_ctx_sms(ctx);
    symv_finish<<<std::min(sms * 4, (n + 255) / 256), 256, 0, S(ctx)>>>(n, nb, part, alpha, beta, yb, incy);
    gbx_count_launch(ctx, 1);
    return gbx_check_launch(ctx, "dsymv");
}

namespace gbx_gemm {
// inverted 64x64 diagonal blocks of op(A) (trsm.cu)
gbx_status trinv_diag_blocks(gbx_ctx *ctx, int na, const double *A, long long lda, int tr, int lower, int unit,
                             double *inv);
}

extern "C" gbx_status gbx_dtrsv(gbx_ctx *ctx, char uplo, char trans, char diag, int n, const double *A, int lda,
                                double *x, int incx)
{
    if (!ctx) return GBX_ERR_ARG;
    const int info = gbx_check_trsv_args(uplo, trans, diag, n, lda, incx);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "DTRSV parameter %d", info);
    if (n == 0) return GBX_OK;
    const int tri = gbx_op_tri(uplo, trans, diag);
    const int fwd = (tri & gbx_gemm::TRI_LOWER) != 0;
    const int tr = !gbx_lsame(trans, 'N');
    const int nblk = (n + TV_NB - 1) / TV_NB, npad = nblk * TV_NB;
    double *inv, *w;
    gbx_status st;
    if ((st = gbx_ws(ctx, GBX_WS_TMP1, sizeof(double) * (size_t)nblk * TV_NB * TV_NB, (void **)&inv)) != GBX_OK)
        return st;
    if ((st = gbx_ws(ctx, GBX_WS_TMP2, sizeof(double) * (size_t)npad, (void **)&w)) != GBX_OK) return st;
    if ((st = gbx_gemm::trinv_diag_blocks(ctx, n, A, lda, tr, fwd, (tri & gbx_gemm::TRI_UNIT) != 0, inv)) !=
        GBX_OK)
        return st;
    double *xb = x + base_off(n, incx);
    const int sms = gbx_ctx_sms(ctx);
    gather_vec<<<std::min(sms * 4, (npad + 255) / 256), 256, 0, S(ctx)>>>(n, xb, incx, w, npad);
    gbx_count_launch(ctx, 1);
    gbx_timer_begin(ctx, GBX_TIMER_GEMV);
    for (int s = 0; s < nblk; s++) {
        const int J = fwd ? s : nblk - 1 - s;
        const int rows = fwd ? std::max(0, n - (J + 1) * TV_NB) : J * TV_NB;
        const int grid = std::max(1, (rows + 255) / 256);
        trsv_step<<<grid, 256, 0, S(ctx)>>>(n, J, fwd, tr, A, lda, inv, w, xb, incx);
    }
    gbx_timer_end(ctx);
    gbx_count_launch(ctx, (uint64_t)nblk);
    return gbx_check_launch(ctx, "dtrsv");
}
