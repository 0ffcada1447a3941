// trsm.cu — gbx_dtrsm: triangular solve with many right-hand sides.
//
// Replaces cublasDtrsm behind the reference's wrapper (blas_level3/trsm.cc:
// 40-73 launch, 76-132 argument checks; that file does not compile as shipped,
// trsm.cc:55).  Recursive blocked algorithm:
//   * all diagonal blocks of op(A) (64 x 64) are inverted in FP64 by one
//     launch (one CTA per block, forward/back substitution against I);
//   * the solve recurses on halves: solve the leading half, update the
//     trailing half with one large GEMM (k = half the order) on the DFMA GEMM
//     core, solve the trailing half.  Leaves multiply by the inverted block.
// The GEMM updates dominate (m^2*nrhs flops overall); the inverted-block leaves
// add 2*64^2*nrhs flops per block (about 3% at m = 8192).
#include "gbx_internal.h"
#include "gemm_host.h"

#include <cuda_runtime.h>
#include <algorithm>

using namespace gbx_gemm;

namespace {

constexpr int NB = 64;

inline cudaStream_t S(gbx_ctx *ctx) { return (cudaStream_t)gbx_ctx_get_stream(ctx); }

// Inverse of each NB x NB diagonal block of op(A) (na x na).  Blocks shorter
// than NB at the end are padded with the identity.  Inv holds the blocks one
// after another, each column-major with leading dimension NB.
__global__ void __launch_bounds__(NB)
trinv_blocks(int na, const double *__restrict__ A, long long lda, int tr, int lower, int unit,
             double *__restrict__ Inv)
{
    extern __shared__ double sm[];
    double *L = sm;                   // L[i*(NB+1) + k] = op(A)(r0+i, r0+k)
    double *X = sm + NB * (NB + 1);   // X[i*NB + j]
    const int r0 = blockIdx.x * NB;
    const int nbb = min(NB, na - r0);
    for (int t = threadIdx.x; t < NB * NB; t += blockDim.x) {
        const int i = t % NB, k = t / NB;
        double v = 0.0;
        if (i < nbb && k < nbb) {
            const bool in = lower ? (k <= i) : (k >= i);
            if (in) v = tr ? A[(long long)(r0 + i) * lda + r0 + k] : A[(long long)(r0 + k) * lda + r0 + i];
            if (i == k && unit) v = 1.0;
        } else if (i == k) {
            v = 1.0;
        }
        L[i * (NB + 1) + k] = v;
    }
    __syncthreads();
    const int j = threadIdx.x;   // this thread owns column j of the inverse
    if (lower) {
        for (int i = 0; i < NB; i++) {
            double s = (i == j) ? 1.0 : 0.0;
            for (int k = 0; k < i; k++) s = fma(-L[i * (NB + 1) + k], X[k * NB + j], s);
            X[i * NB + j] = s / L[i * (NB + 1) + i];
        }
    } else {
        for (int i = NB - 1; i >= 0; i--) {
            double s = (i == j) ? 1.0 : 0.0;
            for (int k = i + 1; k < NB; k++) s = fma(-L[i * (NB + 1) + k], X[k * NB + j], s);
            X[i * NB + j] = s / L[i * (NB + 1) + i];
        }
    }
    double *out = Inv + (long long)blockIdx.x * NB * NB;
    for (int i = 0; i < NB; i++) out[(long long)j * NB + i] = X[i * NB + j];
}

struct Trsm {
    gbx_ctx *ctx;
    int m, n, na;
    const double *A;
    long long lda;
    int tr, lower;
    double *B;
    long long ldb;
    const double *Inv;
    double *T;   // NB x n (left) or m x NB (right)

    // op(A)[r0:, c0:] as a GEMM operand: pointer and transposition flag
    const double *opA(int r0, int c0, int &t) const
    {
        t = tr;
        return tr ? A + (long long)r0 * lda + c0 : A + (long long)c0 * lda + r0;
    }

    gbx_status gemm(int mm, int nn, int kk, double alpha, const double *Ap, long long lda_, int ta,
                    const double *Bp, long long ldb_, int tb, double beta, double *Cp, long long ldc)
    {
        GemmArgs<double> p{};
        p.m = mm; p.n = nn; p.k = kk;
        p.A = Ap; p.lda = lda_; p.ta = ta;
        p.B = Bp; p.ldb = ldb_; p.tb = tb;
        p.alpha = alpha; p.beta = beta;
        p.C = Cp; p.ldc = ldc;
        return launch_gemm<double>(ctx, p, "dtrsm");
    }

    gbx_status copy_back(double *dst, long long ldd, const double *src, long long lds, int rows, int cols)
    {
        cudaError_t e = cudaMemcpy2DAsync(dst, sizeof(double) * ldd, src, sizeof(double) * lds,
                                          sizeof(double) * rows, cols, cudaMemcpyDeviceToDevice, S(ctx));
        return e == cudaSuccess ? GBX_OK : gbx_fail(ctx, GBX_ERR_CUDA, "dtrsm copy: %s", cudaGetErrorString(e));
    }

    // split point: a multiple of NB near the middle
    static int split(int len) { return std::max(NB, ((len / 2 + NB - 1) / NB) * NB); }

    // Left side: solve rows [r0, r0+len) of op(A) X = B in place.
    gbx_status left(int r0, int len)
    {
        gbx_status st;
        if (len <= NB) {
            const double *inv = Inv + (long long)(r0 / NB) * NB * NB;
            if ((st = gemm(len, n, len, 1.0, inv, NB, 0, B + r0, ldb, 0, 0.0, T, NB)) != GBX_OK) return st;
            return copy_back(B + r0, ldb, T, NB, len, n);
        }
        const int h = split(len);
        int t;
        if (lower) {
            if ((st = left(r0, h)) != GBX_OK) return st;
            const double *a = opA(r0 + h, r0, t);
            if ((st = gemm(len - h, n, h, -1.0, a, lda, t, B + r0, ldb, 0, 1.0, B + r0 + h, ldb)) != GBX_OK)
                return st;
            return left(r0 + h, len - h);
        }
        if ((st = left(r0 + h, len - h)) != GBX_OK) return st;
        const double *a = opA(r0, r0 + h, t);
        if ((st = gemm(h, n, len - h, -1.0, a, lda, t, B + r0 + h, ldb, 0, 1.0, B + r0, ldb)) != GBX_OK)
            return st;
        return left(r0, h);
    }

    // Right side: solve columns [c0, c0+len) of X op(A) = B in place.
    gbx_status right(int c0, int len)
    {
        gbx_status st;
        if (len <= NB) {
            const double *inv = Inv + (long long)(c0 / NB) * NB * NB;
            if ((st = gemm(m, len, len, 1.0, B + (long long)c0 * ldb, ldb, 0, inv, NB, 0, 0.0, T, m)) != GBX_OK)
                return st;
            return copy_back(B + (long long)c0 * ldb, ldb, T, m, m, len);
        }
        const int h = split(len);
        int t;
        if (!lower) {
            // X_2 op(A)_22 = B_2 - X_1 op(A)_12
            if ((st = right(c0, h)) != GBX_OK) return st;
            const double *a = opA(c0, c0 + h, t);
            if ((st = gemm(m, len - h, h, -1.0, B + (long long)c0 * ldb, ldb, 0, a, lda, t, 1.0,
                           B + (long long)(c0 + h) * ldb, ldb)) != GBX_OK)
                return st;
            return right(c0 + h, len - h);
        }
        // lower: X_1 op(A)_11 = B_1 - X_2 op(A)_21
        if ((st = right(c0 + h, len - h)) != GBX_OK) return st;
        const double *a = opA(c0 + h, c0, t);
        if ((st = gemm(m, h, len - h, -1.0, B + (long long)(c0 + h) * ldb, ldb, 0, a, lda, t, 1.0,
                       B + (long long)c0 * ldb, ldb)) != GBX_OK)
            return st;
        return right(c0, h);
    }
};

}  // namespace

extern "C" gbx_status gbx_dtrsm(gbx_ctx *ctx, char side, char uplo, char ta, char diag, int m,
                                int n, double alpha, const double *A, int lda, double *B, int ldb)
{
    if (!ctx) return GBX_ERR_ARG;
    int info = gbx_check_trxm_args(side, uplo, ta, diag, m, n, lda, ldb);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "DTRSM parameter %d", info);
    if (m == 0 || n == 0) return GBX_OK;
    if (alpha == 0.0) return scale_matrix<double>(ctx, m, n, 0.0, B, ldb, C_FULL);
    gbx_status st;
    if (alpha != 1.0 && (st = scale_matrix<double>(ctx, m, n, alpha, B, ldb, C_FULL)) != GBX_OK) return st;

    const bool lside = gbx_lsame(side, 'L');
    const int tri = gbx_op_tri(uplo, ta, diag);
    Trsm t;
    t.ctx = ctx; t.m = m; t.n = n; t.na = lside ? m : n;
    t.A = A; t.lda = lda; t.tr = !gbx_lsame(ta, 'N'); t.lower = (tri & TRI_LOWER) != 0;
    t.B = B; t.ldb = ldb;
    const int nblk = (t.na + NB - 1) / NB;
    double *inv, *tmp;
    if ((st = gbx_ws(ctx, 1, sizeof(double) * (size_t)nblk * NB * NB, (void **)&inv)) != GBX_OK) return st;
    if ((st = gbx_ws(ctx, 2, sizeof(double) * (size_t)NB * (lside ? n : m), (void **)&tmp)) != GBX_OK) return st;
    t.Inv = inv;
    t.T = tmp;

    const size_t smem = sizeof(double) * (NB * (NB + 1) + NB * NB);
    // a per-device function attribute; setting it is a cheap host call
    cudaFuncSetAttribute(trinv_blocks, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    trinv_blocks<<<nblk, NB, smem, S(ctx)>>>(t.na, A, lda, t.tr, t.lower, (tri & TRI_UNIT) != 0, inv);
    gbx_count_launch(ctx, 1);
    if ((st = gbx_check_launch(ctx, "dtrsm inverse")) != GBX_OK) return st;
    return lside ? t.left(0, m) : t.right(0, n);
}
