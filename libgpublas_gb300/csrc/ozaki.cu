// ozaki.cu — Ozaki split-precision DGEMM / ZGEMM / DSYRK (placeholder until
// the tensor-core path lands; every entry reports GBX_ERR_UNSUPPORTED).
#include "gbx_internal.h"

extern "C" gbx_status gbx_dgemm_ozaki(gbx_ctx *ctx, char, char, int, int, int, double,
                                      const double *, int, const double *, int, double, double *,
                                      int, double, int, int *)
{
    return gbx_fail(ctx, GBX_ERR_UNSUPPORTED, "ozaki dgemm not built");
}

extern "C" gbx_status gbx_zgemm_ozaki(gbx_ctx *ctx, char, char, int, int, int, const double *,
                                      const double *, int, const double *, int, const double *,
                                      double *, int, double, int, int *)
{
    return gbx_fail(ctx, GBX_ERR_UNSUPPORTED, "ozaki zgemm not built");
}

extern "C" gbx_status gbx_dsyrk_ozaki(gbx_ctx *ctx, char, char, int, int, double, const double *,
                                      int, double, double *, int, double, int, int *)
{
    return gbx_fail(ctx, GBX_ERR_UNSUPPORTED, "ozaki dsyrk not built");
}
