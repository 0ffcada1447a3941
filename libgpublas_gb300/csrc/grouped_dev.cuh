// grouped_dev.cuh — device code shared by the grouped kernel (batched.cu)
// and the serving loop's persistent kernel (serve_loop.cu): the operation
// descriptor and the small triangular solve.
#pragma once

#include <cuda_runtime.h>

namespace gbx_grouped {

struct DevOp {
    int kind;                     // GBX_OP_GEMM / GBX_OP_TRSM
    int ta, tb;                   // GEMM transpositions; TRSM: ta = op(A) transposed
    int lower, unit, left;        // TRSM: effective triangle of the solved matrix, diag, side
    int m, n, k;
    double alpha, beta;
    const double *A;
    long long lda;
    const double *B;
    long long ldb;
    double *C;
    long long ldc;
};

// ---------------------------------------------------------------- TRSM item
// Solves T y = alpha*b for up to NSYS systems of order n (<= 256), where
// for side 'L' T = op(A) and the systems are columns of B (m x nrhs), and for
// side 'R' T = op(A)^T and the systems are rows of B.  Substitution order is
// chosen by the effective triangle of T.
template <int NSYS, int NTHREADS>
__device__ void trsm_item(const DevOp &o, int sys0, double *smem)
{
    const int n = o.left ? o.m : o.n;                 // order of T
    const int nsys_total = o.left ? o.n : o.m;
    const int nsys = min(NSYS, nsys_total - sys0);
    double *X = smem;                                  // X[i * NSYS + s]
    // element (i, s) of system vector s
    auto bidx = [&](int i, int s) -> long long {
        return o.left ? (long long)(sys0 + s) * o.ldc + i : (long long)i * o.ldc + (sys0 + s);
    };
    // T(i, j): side L: op(A)(i,j); side R: op(A)(j,i)
    auto T = [&](int i, int j) -> double {
        int r = i, c = j;
        if (!o.left) { r = j; c = i; }
        return o.ta ? o.A[(long long)r * o.lda + c] : o.A[(long long)c * o.lda + r];
    };
    for (int t = threadIdx.x; t < n * NSYS; t += NTHREADS) {
        const int i = t / NSYS, s = t % NSYS;
        X[t] = s < nsys ? o.alpha * o.C[bidx(i, s)] : 0.0;
    }
    __syncthreads();
    for (int step = 0; step < n; step++) {
        const int kk = o.lower ? step : n - 1 - step;
        if (!o.unit) {
            const double d = T(kk, kk);
            if (threadIdx.x < NSYS) X[kk * NSYS + threadIdx.x] /= d;
            __syncthreads();
        }
        // update the rows still to be solved
        const int r0 = o.lower ? kk + 1 : 0, r1 = o.lower ? n : kk;
        for (int t = threadIdx.x; t < (r1 - r0) * NSYS; t += NTHREADS) {
            const int i = r0 + t / NSYS, s = t % NSYS;
            X[i * NSYS + s] = fma(-T(i, kk), X[kk * NSYS + s], X[i * NSYS + s]);
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < n * NSYS; t += NTHREADS) {
        const int i = t / NSYS, s = t % NSYS;
        if (s < nsys) o.C[bidx(i, s)] = X[t];
    }
}

}  // namespace gbx_grouped
