// trsm.cu — xTRSM (S, D, C, Z): triangular solve with many right-hand sides.
//
// Replaces cublas?trsm behind the reference's wrapper (blas_level3/trsm.cc:
// 40-73 launch, 76-132 argument checks, 134-213 the four precisions; that
// file does not compile as shipped, trsm.cc:55).  Recursive blocked
// algorithm:
//   * all diagonal blocks of op(A) (64 x 64) are inverted by one launch (one
//     CTA per block, forward/back substitution against I, in the routine's
//     own precision);
//   * the solve recurses on halves: solve the leading half, update the
//     trailing half with one large GEMM (k = half the order) on the SIMT GEMM
//     core, solve the trailing half.  Leaves multiply by the inverted block.
// The GEMM updates dominate (m^2*nrhs flops overall); the inverted-block leaves
// add 2*64^2*nrhs flops per block (about 3% at m = 8192).  op(A) = A^H
// (transa 'C') conjugates the inverted blocks and the GEMM operands.
#include "gbx_internal.h"
#include "gemm_host.h"

#include <cuda_runtime.h>
#include <algorithm>

using namespace gbx_gemm;

namespace {

constexpr int NB = 64;

inline cudaStream_t S(gbx_ctx *ctx) { return (cudaStream_t)gbx_ctx_get_stream(ctx); }

template <typename T> T unit_of(int v) { return T(v); }
template <> fcplx unit_of<fcplx>(int v) { return {(float)v, 0.0f}; }
template <> dcplx unit_of<dcplx>(int v) { return {(double)v, 0.0}; }

// Inverse of each NB x NB diagonal block of op(A) (na x na).  Blocks shorter
// than NB at the end are padded with the identity.  Inv holds the blocks one
// after another, each column-major with leading dimension NB.  One CTA of NB
// threads per block, one column of the inverse per thread, in the routine's
// precision; the divisions are the element type's own (IEEE for real,
// Smith's algorithm for complex).
template <typename T>
__global__ void __launch_bounds__(NB)
trinv_blocks(int na, const T *__restrict__ A, long long lda, int tr, int cj, int lower, int unit,
             T *__restrict__ Inv)
{
    extern __shared__ __align__(16) unsigned char sm_raw[];
    T *L = (T *)sm_raw;               // L[i*(NB+1) + k] = op(A)(r0+i, r0+k)
    T *X = L + NB * (NB + 1);         // X[i*NB + j]
    const int r0 = blockIdx.x * NB;
    const int nbb = min(NB, na - r0);
    for (int t = threadIdx.x; t < NB * NB; t += blockDim.x) {
        const int i = t % NB, k = t / NB;
        T v = Ops<T>::zero();
        if (i < nbb && k < nbb) {
            const bool in = lower ? (k <= i) : (k >= i);
            if (in) {
                v = tr ? A[(long long)(r0 + i) * lda + r0 + k] : A[(long long)(r0 + k) * lda + r0 + i];
                if (cj) v = Ops<T>::conj(v);
            }
            if (i == k && unit) v = Ops<T>::one();
        } else if (i == k) {
            v = Ops<T>::one();
        }
        L[i * (NB + 1) + k] = v;
    }
    __syncthreads();
    const int j = threadIdx.x;   // this thread owns column j of the inverse
    if (lower) {
        for (int i = 0; i < NB; i++) {
            T s = (i == j) ? Ops<T>::one() : Ops<T>::zero();
            for (int k = 0; k < i; k++) Ops<T>::fma_acc(s, Ops<T>::neg(L[i * (NB + 1) + k]), X[k * NB + j]);
            X[i * NB + j] = Ops<T>::div(s, L[i * (NB + 1) + i]);
        }
    } else {
        for (int i = NB - 1; i >= 0; i--) {
            T s = (i == j) ? Ops<T>::one() : Ops<T>::zero();
            for (int k = i + 1; k < NB; k++) Ops<T>::fma_acc(s, Ops<T>::neg(L[i * (NB + 1) + k]), X[k * NB + j]);
            X[i * NB + j] = Ops<T>::div(s, L[i * (NB + 1) + i]);
        }
    }
    T *out = Inv + (long long)blockIdx.x * NB * NB;
    for (int i = 0; i < NB; i++) out[(long long)j * NB + i] = X[i * NB + j];
}

template <typename T>
struct Trsm {
    gbx_ctx *ctx;
    const char *nm;
    int m, n, na;
    const T *A;
    long long lda;
    int tr, cj, lower;
    T *B;
    long long ldb;
    const T *Inv;
    T *Tw;   // NB x n (left) or m x NB (right)

    // op(A)[r0:, c0:] as a GEMM operand: pointer and transposition flag
    const T *opA(int r0, int c0, int &t) const
    {
        t = tr;
        return tr ? A + (long long)r0 * lda + c0 : A + (long long)c0 * lda + r0;
    }

    // C = alpha op(X) op(Y) + beta C; conj_x / conj_y conjugate the operand
    // (the slices of op(A) = A^H)
    gbx_status gemm(int mm, int nn, int kk, T alpha, const T *Ap, long long lda_, int ta, int ca, const T *Bp,
                    long long ldb_, int tb, int cb, T beta, T *Cp, long long ldc)
    {
        GemmArgs<T> p{};
        p.m = mm; p.n = nn; p.k = kk;
        p.A = Ap; p.lda = lda_; p.ta = ta; p.conja = ca;
        p.B = Bp; p.ldb = ldb_; p.tb = tb; p.conjb = cb;
        p.alpha = alpha; p.beta = beta;
        p.C = Cp; p.ldc = ldc;
        return launch_gemm<T>(ctx, p, nm);
    }

    gbx_status copy_back(T *dst, long long ldd, const T *src, long long lds, int rows, int cols)
    {
        cudaError_t e = cudaMemcpy2DAsync(dst, sizeof(T) * ldd, src, sizeof(T) * lds, sizeof(T) * rows, cols,
                                          cudaMemcpyDeviceToDevice, S(ctx));
        return e == cudaSuccess ? GBX_OK : gbx_fail(ctx, GBX_ERR_CUDA, "%s copy: %s", nm, cudaGetErrorString(e));
    }

    static T one() { return unit_of<T>(1); }
    static T mone() { return unit_of<T>(-1); }

    // split point: a multiple of NB near the middle
    static int split(int len) { return std::max(NB, ((len / 2 + NB - 1) / NB) * NB); }

    // Left side: solve rows [r0, r0+len) of op(A) X = B in place.
    gbx_status left(int r0, int len)
    {
        gbx_status st;
        if (len <= NB) {
            const T *inv = Inv + (long long)(r0 / NB) * NB * NB;
            if ((st = gemm(len, n, len, one(), inv, NB, 0, 0, B + r0, ldb, 0, 0, T{}, Tw, NB)) != GBX_OK) return st;
            return copy_back(B + r0, ldb, Tw, NB, len, n);
        }
        const int h = split(len);
        int t;
        if (lower) {
            if ((st = left(r0, h)) != GBX_OK) return st;
            const T *a = opA(r0 + h, r0, t);
            if ((st = gemm(len - h, n, h, mone(), a, lda, t, cj, B + r0, ldb, 0, 0, one(), B + r0 + h, ldb)) !=
                GBX_OK)
                return st;
            return left(r0 + h, len - h);
        }
        if ((st = left(r0 + h, len - h)) != GBX_OK) return st;
        const T *a = opA(r0, r0 + h, t);
        if ((st = gemm(h, n, len - h, mone(), a, lda, t, cj, B + r0 + h, ldb, 0, 0, one(), B + r0, ldb)) != GBX_OK)
            return st;
        return left(r0, h);
    }

    // Right side: solve columns [c0, c0+len) of X op(A) = B in place.
    gbx_status right(int c0, int len)
    {
        gbx_status st;
        if (len <= NB) {
            const T *inv = Inv + (long long)(c0 / NB) * NB * NB;
            if ((st = gemm(m, len, len, one(), B + (long long)c0 * ldb, ldb, 0, 0, inv, NB, 0, 0, T{}, Tw, m)) !=
                GBX_OK)
                return st;
            return copy_back(B + (long long)c0 * ldb, ldb, Tw, m, m, len);
        }
        const int h = split(len);
        int t;
        if (!lower) {
            // X_2 op(A)_22 = B_2 - X_1 op(A)_12
            if ((st = right(c0, h)) != GBX_OK) return st;
            const T *a = opA(c0, c0 + h, t);
            if ((st = gemm(m, len - h, h, mone(), B + (long long)c0 * ldb, ldb, 0, 0, a, lda, t, cj, one(),
                           B + (long long)(c0 + h) * ldb, ldb)) != GBX_OK)
                return st;
            return right(c0 + h, len - h);
        }
        // lower: X_1 op(A)_11 = B_1 - X_2 op(A)_21
        if ((st = right(c0 + h, len - h)) != GBX_OK) return st;
        const T *a = opA(c0 + h, c0, t);
        if ((st = gemm(m, h, len - h, mone(), B + (long long)(c0 + h) * ldb, ldb, 0, 0, a, lda, t, cj, one(),
                       B + (long long)c0 * ldb, ldb)) != GBX_OK)
            return st;
        return right(c0, h);
    }
};

template <typename T>
gbx_status trsm_t(gbx_ctx *ctx, const char *nm, char side, char uplo, char ta, char diag, int m, int n, T alpha,
                  bool alpha0, bool alpha1, const T *A, int lda, T *B, int ldb)
{
    if (!ctx) return GBX_ERR_ARG;
    int info = gbx_check_trxm_args(side, uplo, ta, diag, m, n, lda, ldb);
    if (info) return gbx_fail(ctx, GBX_ERR_ARG, "%s parameter %d", nm, info);
    if (m == 0 || n == 0) return GBX_OK;
    if (alpha0) return scale_matrix<T>(ctx, m, n, alpha, B, ldb, C_FULL);
    gbx_status st;
    if (!alpha1 && (st = scale_matrix<T>(ctx, m, n, alpha, B, ldb, C_FULL)) != GBX_OK) return st;

    const bool lside = gbx_lsame(side, 'L');
    const int tri = gbx_op_tri(uplo, ta, diag);
    Trsm<T> t;
    t.ctx = ctx; t.nm = nm; t.m = m; t.n = n; t.na = lside ? m : n;
    t.A = A; t.lda = lda; t.tr = !gbx_lsame(ta, 'N'); t.cj = gbx_lsame(ta, 'C');
    t.lower = (tri & TRI_LOWER) != 0;
    t.B = B; t.ldb = ldb;
    const int nblk = (t.na + NB - 1) / NB;
    T *inv, *tmp;
    if ((st = gbx_ws(ctx, GBX_WS_TMP1, sizeof(T) * (size_t)nblk * NB * NB, (void **)&inv)) != GBX_OK) return st;
    if ((st = gbx_ws(ctx, GBX_WS_TMP2, sizeof(T) * (size_t)NB * (lside ? n : m), (void **)&tmp)) != GBX_OK)
        return st;
    t.Inv = inv;
    t.Tw = tmp;

    const size_t smem = sizeof(T) * (NB * (NB + 1) + NB * NB);
    // a per-device function attribute; setting it is a cheap host call
    cudaFuncSetAttribute(trinv_blocks<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    trinv_blocks<T><<<nblk, NB, smem, S(ctx)>>>(t.na, A, lda, t.tr, t.cj, t.lower, (tri & TRI_UNIT) != 0, inv);
    gbx_count_launch(ctx, 1);
    if ((st = gbx_check_launch(ctx, nm)) != GBX_OK) return st;
    return lside ? t.left(0, m) : t.right(0, n);
}

}  // namespace

namespace gbx_gemm {
// Inverted 64x64 diagonal blocks of op(A) (na x na; lower: op(A) is lower
// triangular), for the blocked DTRSV.
gbx_status trinv_diag_blocks(gbx_ctx *ctx, int na, const double *A, long long lda, int tr, int lower, int unit,
                             double *inv)
{
    const int nblk = (na + NB - 1) / NB;
    const size_t smem = sizeof(double) * (NB * (NB + 1) + NB * NB);
    cudaFuncSetAttribute(trinv_blocks<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    trinv_blocks<double><<<nblk, NB, smem, S(ctx)>>>(na, A, lda, tr, 0, lower, unit, inv);
    gbx_count_launch(ctx, 1);
    return gbx_check_launch(ctx, "trsv inverse");
}
}  // namespace gbx_gemm

extern "C" gbx_status gbx_strsm(gbx_ctx *ctx, char side, char uplo, char ta, char diag, int m, int n, float alpha,
                                const float *A, int lda, float *B, int ldb)
{
    return trsm_t<float>(ctx, "STRSM", side, uplo, ta, diag, m, n, alpha, alpha == 0.0f, alpha == 1.0f, A, lda, B,
                         ldb);
}

extern "C" gbx_status gbx_dtrsm(gbx_ctx *ctx, char side, char uplo, char ta, char diag, int m, int n,
                                double alpha, const double *A, int lda, double *B, int ldb)
{
    return trsm_t<double>(ctx, "DTRSM", side, uplo, ta, diag, m, n, alpha, alpha == 0.0, alpha == 1.0, A, lda, B,
                          ldb);
}

extern "C" gbx_status gbx_ctrsm(gbx_ctx *ctx, char side, char uplo, char ta, char diag, int m, int n,
                                const float *alpha, const float *A, int lda, float *B, int ldb)
{
    if (!alpha) return GBX_ERR_ARG;
    const fcplx al{alpha[0], alpha[1]};
    return trsm_t<fcplx>(ctx, "CTRSM", side, uplo, ta, diag, m, n, al, al.x == 0.0f && al.y == 0.0f,
                         al.x == 1.0f && al.y == 0.0f, (const fcplx *)A, lda, (fcplx *)B, ldb);
}

extern "C" gbx_status gbx_ztrsm(gbx_ctx *ctx, char side, char uplo, char ta, char diag, int m, int n,
                                const double *alpha, const double *A, int lda, double *B, int ldb)
{
    if (!alpha) return GBX_ERR_ARG;
    const dcplx al{alpha[0], alpha[1]};
    return trsm_t<dcplx>(ctx, "ZTRSM", side, uplo, ta, diag, m, n, al, al.x == 0.0 && al.y == 0.0,
                         al.x == 1.0 && al.y == 0.0, (const dcplx *)A, lda, (dcplx *)B, ldb);
}
