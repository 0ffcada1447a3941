// gemm_host.h — host-side entry points of the GEMM core shared by the
// Level-3 translation units.
#pragma once

#include "gbx_internal.h"
#include "gemm_simt.cuh"

namespace gbx_gemm {
template <typename T>
gbx_status launch_gemm(gbx_ctx *ctx, GemmArgs<T> p, const char *what);
// C = beta * C on the whole matrix or one triangle (beta == 0 sets zero);
// herm: the diagonal's imaginary part is set to zero (Hermitian C).
template <typename T>
gbx_status scale_matrix(gbx_ctx *ctx, int m, int n, T beta, T *C, long long ldc, int part, int herm = 0);
}  // namespace gbx_gemm
