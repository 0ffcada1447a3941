// l1.cu — Level-1 streaming kernels: daxpy, ddot, dnrm2, idamax, idamin, dscal.
//
// Replaces the reference's (dead, never-built) cuBLAS Level-1 wrappers
// blas_level1/axpy.cc:10-50, dot.cc:9-48, nrm2.cc:9-41, amax.cc:32-43,
// amin.cc:32-43.  All of them are HBM-bound: the kernels read each element
// once with 128-bit loads when the pointers allow it, run a grid sized to a
// multiple of the SM count, and reduce deterministically in two passes (a
// fixed partition into per-block partials, then one block combining the
// partials in a fixed order), so repeated calls give bit-identical results.
#include "gbx_internal.h"
#include "l1_kernels.cuh"

#include <cuda_runtime.h>

using namespace gbx_l1;

namespace {

inline int grid_for(gbx_ctx *ctx, long long n, int per_thread)
{
    long long want = (n + (long long)L1_THREADS * per_thread - 1) / ((long long)L1_THREADS * per_thread);
    long long cap = (long long)gbx_ctx_sms(ctx) * L1_BLOCKS_PER_SM;
    if (want < 1) want = 1;
    return (int)(want < cap ? want : cap);
}

inline cudaStream_t S(gbx_ctx *ctx) { return (cudaStream_t)gbx_ctx_get_stream(ctx); }

// element offset of the first element a kernel should touch: netlib walks a
// negative-increment vector from its far end.
inline long long base_off(int n, int inc) { return inc >= 0 ? 0 : (long long)(n - 1) * (-inc); }

}  // namespace

extern "C" gbx_status gbx_daxpy(gbx_ctx *ctx, int n, double alpha, const double *x, int incx,
                                double *y, int incy)
{
    if (!ctx) return GBX_ERR_ARG;
    if (n <= 0 || alpha == 0.0) return GBX_OK;
    int g = grid_for(ctx, n, 4);
    gbx_timer_begin(ctx, GBX_TIMER_LEVEL1);
    if (incx == 1 && incy == 1) {
        axpy_unit<<<g, L1_THREADS, 0, S(ctx)>>>(n, alpha, x, y);
    } else {
        axpy_strided<<<g, L1_THREADS, 0, S(ctx)>>>(n, alpha, x + base_off(n, incx), incx,
                                                    y + base_off(n, incy), incy);
    }
    gbx_timer_end(ctx);
    gbx_count_launch(ctx, 1);
    return gbx_check_launch(ctx, "daxpy");
}

extern "C" gbx_status gbx_dscal(gbx_ctx *ctx, int n, double alpha, double *x, int incx)
{
    if (!ctx) return GBX_ERR_ARG;
    if (n <= 0 || incx <= 0 || alpha == 1.0) return GBX_OK;
    int g = grid_for(ctx, n, 4);
    scal_kernel<<<g, L1_THREADS, 0, S(ctx)>>>(n, alpha, x, incx);
    gbx_count_launch(ctx, 1);
    return gbx_check_launch(ctx, "dscal");
}

extern "C" gbx_status gbx_ddot(gbx_ctx *ctx, int n, const double *x, int incx,
                               const double *y, int incy, double *res)
{
    if (!ctx || !res) return GBX_ERR_ARG;
    int g = n > 0 ? grid_for(ctx, n, 8) : 1;
    double *part;
    gbx_status st = gbx_ws(ctx, GBX_WS_RED, sizeof(double) * (size_t)g, (void **)&part);
    if (st != GBX_OK) return st;
    if (n <= 0) {
        zero_result<<<1, 1, 0, S(ctx)>>>(res);
        gbx_count_launch(ctx, 1);
        return gbx_check_launch(ctx, "ddot");
    }
    gbx_timer_begin(ctx, GBX_TIMER_LEVEL1);
    dot_partial<<<g, L1_THREADS, 0, S(ctx)>>>(n, x + base_off(n, incx), incx,
                                              y + base_off(n, incy), incy, part);
    gbx_timer_end(ctx);
    sum_partials<<<1, L1_THREADS, 0, S(ctx)>>>(part, g, res);
    gbx_count_launch(ctx, 2);
    return gbx_check_launch(ctx, "ddot");
}

extern "C" gbx_status gbx_dnrm2(gbx_ctx *ctx, int n, const double *x, int incx, double *res)
{
    if (!ctx || !res) return GBX_ERR_ARG;
    if (n < 1 || incx < 1) {
        zero_result<<<1, 1, 0, S(ctx)>>>(res);
        gbx_count_launch(ctx, 1);
        return gbx_check_launch(ctx, "dnrm2");
    }
    int g = grid_for(ctx, n, 8);
    double *part;
    gbx_status st = gbx_ws(ctx, GBX_WS_RED, 3 * sizeof(double) * (size_t)g, (void **)&part);
    if (st != GBX_OK) return st;
    gbx_timer_begin(ctx, GBX_TIMER_LEVEL1);
    nrm2_partial<<<g, L1_THREADS, 0, S(ctx)>>>(n, x, incx, part);
    gbx_timer_end(ctx);
    nrm2_finish<<<1, L1_THREADS, 0, S(ctx)>>>(part, g, res);
    gbx_count_launch(ctx, 2);
    return gbx_check_launch(ctx, "dnrm2");
}

static gbx_status iamax_common(gbx_ctx *ctx, int n, const double *x, int incx, int *res, bool is_min)
{
    if (!ctx || !res) return GBX_ERR_ARG;
    if (n < 1 || incx <= 0) {
        zero_index<<<1, 1, 0, S(ctx)>>>(res);
        gbx_count_launch(ctx, 1);
        return gbx_check_launch(ctx, is_min ? "idamin" : "idamax");
    }
    int g = grid_for(ctx, n, 8);
    unsigned long long *keys;
    gbx_status st = gbx_ws(ctx, GBX_WS_RED, 2 * sizeof(unsigned long long) * (size_t)g,
                           (void **)&keys);
    if (st != GBX_OK) return st;
    long long *idx = (long long *)(keys + g);
    gbx_timer_begin(ctx, GBX_TIMER_LEVEL1);
    if (is_min) iamax_partial<true><<<g, L1_THREADS, 0, S(ctx)>>>(n, x, incx, keys, idx);
    else iamax_partial<false><<<g, L1_THREADS, 0, S(ctx)>>>(n, x, incx, keys, idx);
    gbx_timer_end(ctx);
    if (is_min) iamax_finish<true><<<1, L1_THREADS, 0, S(ctx)>>>(x, keys, idx, g, res);
    else iamax_finish<false><<<1, L1_THREADS, 0, S(ctx)>>>(x, keys, idx, g, res);
    gbx_count_launch(ctx, 2);
    return gbx_check_launch(ctx, is_min ? "idamin" : "idamax");
}

extern "C" gbx_status gbx_idamax(gbx_ctx *ctx, int n, const double *x, int incx, int *res)
{
    return iamax_common(ctx, n, x, incx, res, false);
}

extern "C" gbx_status gbx_idamin(gbx_ctx *ctx, int n, const double *x, int incx, int *res)
{
    return iamax_common(ctx, n, x, incx, res, true);
}
