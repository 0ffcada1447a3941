// gemm_host.h — host-side entry points of the GEMM core shared by the
// Level-3 translation units.
#pragma once

#include "gbx_internal.h"
#include "gemm_simt.cuh"

namespace gbx_gemm {
template <typename T>
gbx_status launch_gemm(gbx_ctx *ctx, GemmArgs<T> p, const char *what);
template <typename T>
gbx_status scale_matrix(gbx_ctx *ctx, int m, int n, T beta, T *C, long long ldc, int part);
}  // namespace gbx_gemm

extern "C" {
int gbx_check_gemm_args(char ta, char tb, int m, int n, int k, int lda, int ldb, int ldc);
int gbx_check_syrk_args(char uplo, char trans, int n, int k, int lda, int ldc);
int gbx_check_trxm_args(char side, char uplo, char ta, char diag, int m, int n, int lda, int ldb);
int gbx_op_tri(char uplo, char transa, char diag);
}
