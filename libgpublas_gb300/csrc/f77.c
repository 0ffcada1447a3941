/*
 * f77.c — the drop-in layer: Fortran-ABI and CBLAS entry points.
 *
 * Each Fortran routine follows the reference's wrapper shape
 * (blas_level3/gemm.cc:162-179: check -> quick return -> stage -> run) with
 * these differences, all deliberate:
 *   * no size cutoff to the CPU BLAS (gemm.cc:129-141): every valid call with
 *     work in it runs on the GPU; there is no CPU fallback;
 *   * beta/alpha scaling on quick paths happens on the GPU, not in a host
 *     loop (gemm.cc:121-125, syrk.cc:113-143), and beta == 0 sets C to zero;
 *   * operands resident in device or managed memory are used in place
 *     (gpuptr hits, runtime-mem.hpp:69-83); host operands are staged through
 *     per-thread workspace that persists across calls instead of a
 *     cudaMalloc/cudaFree per operand per call (runtime-mem.hpp:84-113);
 *   * every call returns only after the result is in the caller's memory,
 *     also for managed outputs (the reference can return early, §3.3 race);
 *   * ddot_/dnrm2_ return double and idamax_/idamin_ return int (blas.h:33-51
 *     declares them void).
 */
#include "gbx_internal.h"
#include "../../include/gbxblas_f77.h"

#include <pthread.h>
#include <stdatomic.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static atomic_ullong g_calls;

void gbx_stats(uint64_t *calls, uint64_t *hits, uint64_t *misses, uint64_t *h2d, uint64_t *d2h)
{
    if (calls) *calls = atomic_load(&g_calls);
    gbx_placement_counters(hits, misses, h2d, d2h);
}

/* ---- netlib-compatible error hooks (weak: applications may override) ---- */
__attribute__((weak)) void xerbla_(const char *srname, const int *info, size_t len)
{
    /* netlib's message, with the routine name trimmed as LEN_TRIM does */
    char name[16] = {0};
    size_t n = len < sizeof name - 1 ? len : sizeof name - 1;
    memcpy(name, srname, n);
    while (n > 0 && (name[n - 1] == ' ' || name[n - 1] == '\0')) name[--n] = '\0';
    fprintf(stderr, " ** On entry to %s parameter number %2d had an illegal value\n", name, *info);
}

__attribute__((weak)) int lsame_(const char *ca, const char *cb)
{
    return gbx_lsame(*ca, *cb);
}

int gbx_check_gemm_args(char ta, char tb, int m, int n, int k, int lda, int ldb, int ldc);
int gbx_check_syrk_args(char uplo, char trans, int n, int k, int lda, int ldc);
int gbx_check_trxm_args(char side, char uplo, char ta, char diag, int m, int n, int lda, int ldb);
int gbx_check_gemv_args(char trans, int m, int n, int lda, int incx, int incy);

static void report(const char *name, gbx_ctx *ctx, gbx_status st)
{
    fprintf(stderr, "gbxblas: %s failed: %s (%s)\n", name, gbx_status_string(st),
            ctx ? gbx_ctx_last_error(ctx) : "no CUDA context");
    if (gbx_get_config()->abort_on_error) abort();
}

/* trace=<file> (preload library): name every operand object of the call */
#define NOTE(fun, p)                                 \
    do {                                             \
        if (gbx_tracker_note) gbx_tracker_note(fun, p); \
    } while (0)

static gbx_ctx *ctx_or_report(const char *name)
{
    gbx_ctx *ctx = gbx_thread_ctx();
    if (!ctx) report(name, NULL, GBX_ERR_CUDA);
    atomic_fetch_add(&g_calls, 1);
    return ctx;
}

/* shared with the other Fortran/CBLAS translation unit (f77_level3.c) */
gbx_ctx *gbx_f77_ctx(const char *name) { return ctx_or_report(name); }
void gbx_f77_report(const char *name, gbx_ctx *ctx, gbx_status st) { report(name, ctx, st); }

#define TRY(expr)                                 \
    do {                                          \
        st = (expr);                              \
        if (st != GBX_OK) goto fail;              \
    } while (0)

/* ---- serve=on: Level-3 calls go through one process-wide serving loop ----
 * Calls from many application threads are then batched together on the GPU
 * (small ones into one grouped kernel).  Staging memory is reserved against
 * the server's budget before operands are placed (admission by free HBM) and
 * given back when the call returns. */
static gbx_server *g_srv;
static pthread_once_t g_srv_once = PTHREAD_ONCE_INIT;

static void srv_init(void)
{
    int dev = 0;
    const char *d = getenv("GBX_DEVICE");
    if (d) dev = atoi(d);
    if (gbx_server_create(dev, 8, 0, &g_srv) != GBX_OK) g_srv = NULL;
}

static gbx_server *server(void)
{
    if (!gbx_get_config()->serve) return NULL;
    pthread_once(&g_srv_once, srv_init);
    return g_srv;
}

/* The staged operands were copied on the calling thread's stream. */
static gbx_status served(gbx_ctx *ctx, gbx_server *srv, const gbx_op *op)
{
    gbx_status st = gbx_ctx_sync(ctx);
    if (st != GBX_OK) return st;
    return gbx_server_call(srv, op, NULL);
}

/* ---------------------------------------------------------------- DGEMM */
void dgemm_(const char *transa, const char *transb, const int *m, const int *n, const int *k,
            const double *alpha, const double *a, const int *lda, const double *b, const int *ldb,
            const double *beta, double *c, const int *ldc)
{
    int info = gbx_check_gemm_args(*transa, *transb, *m, *n, *k, *lda, *ldb, *ldc);
    if (info) { xerbla_("DGEMM ", &info, 6); return; }
    NOTE("dgemm_", a); NOTE("dgemm_", b); NOTE("dgemm_", c);
    GBX_FORWARD(dgemm_, (transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc));
    if (*m == 0 || *n == 0 || ((*alpha == 0.0 || *k == 0) && *beta == 1.0)) return;
    gbx_ctx *ctx = ctx_or_report("DGEMM");
    if (!ctx) return;
    gbx_status st;
    const int nota = gbx_lsame(*transa, 'N'), notb = gbx_lsame(*transb, 'N');
    const int work = !(*alpha == 0.0 || *k == 0);
    gbx_server *srv = server();
    const size_t bytes = 8 * ((size_t)*m * *k + (size_t)*k * *n + (size_t)*m * *n);
    if (srv && (st = gbx_server_admit(srv, bytes)) != GBX_OK) { report("DGEMM", ctx, st); return; }
    const gbx_config *cfg = gbx_get_config();
    if (!srv && work && !cfg->precision_ozaki && gbx_dgemm_pipeline_eligible(ctx, *m, *n, *k, a, b, c)) {
        /* large call on host operands: copies overlap the block products */
        TRY(gbx_dgemm_host_pipelined(ctx, *transa, *transb, *m, *n, *k, *alpha, a, *lda, b, *ldb, *beta, c, *ldc));
        TRY(gbx_ctx_sync(ctx));
        return;
    }
    /* operands left unplaced on quick paths keep the caller's (valid) ld */
    gbx_operand oa = {.ld = *lda}, ob = {.ld = *ldb}, oc = {0};
    if (work) {
        TRY(gbx_place_in(ctx, GBX_WS_STAGE_A, a, nota ? *m : *k, nota ? *k : *m, *lda, 8, 1, &oa));
        TRY(gbx_place_in(ctx, GBX_WS_STAGE_B, b, notb ? *k : *n, notb ? *n : *k, *ldb, 8, 1, &ob));
    }
    TRY(gbx_place_in(ctx, GBX_WS_STAGE_C, c, *m, *n, *ldc, 8, *beta != 0.0, &oc));
    if (srv) {
        gbx_op op = {0};
        op.kind = (work && cfg->precision_ozaki) ? GBX_OP_GEMM_OZAKI : GBX_OP_GEMM;
        op.transa = *transa; op.transb = *transb;
        op.m = *m; op.n = *n; op.k = *k; op.alpha = *alpha; op.beta = *beta;
        op.A = oa.dev; op.lda = oa.ld; op.B = ob.dev; op.ldb = ob.ld; op.C = oc.dev; op.ldc = oc.ld;
        TRY(served(ctx, srv, &op));
    } else if (work && cfg->precision_ozaki) {
        TRY(gbx_dgemm_ozaki(ctx, *transa, *transb, *m, *n, *k, *alpha, oa.dev, oa.ld, ob.dev, ob.ld,
                            *beta, oc.dev, oc.ld, cfg->ozaki_tol, 0, NULL));
    } else {
        TRY(gbx_dgemm(ctx, *transa, *transb, *m, *n, *k, *alpha, oa.dev, oa.ld, ob.dev, ob.ld,
                      *beta, oc.dev, oc.ld));
    }
    TRY(gbx_place_out(ctx, &oc, *m, *n, 8));
    TRY(gbx_ctx_sync(ctx));
    if (srv) gbx_server_release(srv, bytes);
    return;
fail:
    if (srv) gbx_server_release(srv, bytes);
    report("DGEMM", ctx, st);
}

/* ---------------------------------------------------------------- ZGEMM */
void zgemm_(const char *transa, const char *transb, const int *m, const int *n, const int *k,
            const double *alpha, const double *a, const int *lda, const double *b, const int *ldb,
            const double *beta, double *c, const int *ldc)
{
    int info = gbx_check_gemm_args(*transa, *transb, *m, *n, *k, *lda, *ldb, *ldc);
    if (info) { xerbla_("ZGEMM ", &info, 6); return; }
    NOTE("zgemm_", a); NOTE("zgemm_", b); NOTE("zgemm_", c);
    GBX_FORWARD(zgemm_, (transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc));
    const int alpha0 = alpha[0] == 0.0 && alpha[1] == 0.0;
    const int beta0 = beta[0] == 0.0 && beta[1] == 0.0;
    const int beta1 = beta[0] == 1.0 && beta[1] == 0.0;
    if (*m == 0 || *n == 0 || ((alpha0 || *k == 0) && beta1)) return;
    gbx_ctx *ctx = ctx_or_report("ZGEMM");
    if (!ctx) return;
    gbx_status st;
    const int nota = gbx_lsame(*transa, 'N'), notb = gbx_lsame(*transb, 'N');
    const int work = !(alpha0 || *k == 0);
    /* operands left unplaced on quick paths keep the caller's (valid) ld */
    gbx_operand oa = {.ld = *lda}, ob = {.ld = *ldb}, oc = {0};
    if (work) {
        TRY(gbx_place_in(ctx, GBX_WS_STAGE_A, a, nota ? *m : *k, nota ? *k : *m, *lda, 16, 1, &oa));
        TRY(gbx_place_in(ctx, GBX_WS_STAGE_B, b, notb ? *k : *n, notb ? *n : *k, *ldb, 16, 1, &ob));
    }
    TRY(gbx_place_in(ctx, GBX_WS_STAGE_C, c, *m, *n, *ldc, 16, !beta0, &oc));
    const gbx_config *cfg = gbx_get_config();
    if (work && cfg->precision_ozaki)
        TRY(gbx_zgemm_ozaki(ctx, *transa, *transb, *m, *n, *k, alpha, oa.dev, oa.ld, ob.dev, ob.ld,
                            beta, oc.dev, oc.ld, cfg->ozaki_tol, 0, NULL));
    else
        TRY(gbx_zgemm(ctx, *transa, *transb, *m, *n, *k, alpha, oa.dev, oa.ld, ob.dev, ob.ld, beta,
                      oc.dev, oc.ld));
    TRY(gbx_place_out(ctx, &oc, *m, *n, 16));
    TRY(gbx_ctx_sync(ctx));
    return;
fail:
    report("ZGEMM", ctx, st);
}

/* ---------------------------------------------------------------- DSYRK */
void dsyrk_(const char *uplo, const char *trans, const int *n, const int *k, const double *alpha,
            const double *a, const int *lda, const double *beta, double *c, const int *ldc)
{
    int info = gbx_check_syrk_args(*uplo, *trans, *n, *k, *lda, *ldc);
    if (info) { xerbla_("DSYRK ", &info, 6); return; }
    NOTE("dsyrk_", a); NOTE("dsyrk_", c);
    GBX_FORWARD(dsyrk_, (uplo, trans, n, k, alpha, a, lda, beta, c, ldc));
    if (*n == 0 || ((*alpha == 0.0 || *k == 0) && *beta == 1.0)) return;
    gbx_ctx *ctx = ctx_or_report("DSYRK");
    if (!ctx) return;
    gbx_status st;
    const int notr = gbx_lsame(*trans, 'N');
    const int work = !(*alpha == 0.0 || *k == 0);
    gbx_server *srv = server();
    const size_t bytes = 8 * ((size_t)*n * *k + (size_t)*n * *n);
    if (srv && (st = gbx_server_admit(srv, bytes)) != GBX_OK) { report("DSYRK", ctx, st); return; }
    gbx_operand oa = {.ld = *lda}, oc = {0};
    if (work)
        TRY(gbx_place_in(ctx, GBX_WS_STAGE_A, a, notr ? *n : *k, notr ? *k : *n, *lda, 8, 1, &oa));
    /* the other triangle of C must survive the round trip: always copy in */
    TRY(gbx_place_in(ctx, GBX_WS_STAGE_C, c, *n, *n, *ldc, 8, 1, &oc));
    const gbx_config *cfg = gbx_get_config();
    if (srv) {
        gbx_op op = {0};
        op.kind = (work && cfg->precision_ozaki) ? GBX_OP_SYRK_OZAKI : GBX_OP_SYRK;
        op.uplo = *uplo; op.transa = *trans; op.n = *n; op.k = *k; op.alpha = *alpha; op.beta = *beta;
        op.A = oa.dev; op.lda = oa.ld; op.C = oc.dev; op.ldc = oc.ld;
        TRY(served(ctx, srv, &op));
    } else if (work && cfg->precision_ozaki) {
        TRY(gbx_dsyrk_ozaki(ctx, *uplo, *trans, *n, *k, *alpha, oa.dev, oa.ld, *beta, oc.dev, oc.ld,
                            cfg->ozaki_tol, 0, NULL));
    } else {
        TRY(gbx_dsyrk(ctx, *uplo, *trans, *n, *k, *alpha, oa.dev, oa.ld, *beta, oc.dev, oc.ld));
    }
    TRY(gbx_place_out(ctx, &oc, *n, *n, 8));
    TRY(gbx_ctx_sync(ctx));
    if (srv) gbx_server_release(srv, bytes);
    return;
fail:
    if (srv) gbx_server_release(srv, bytes);
    report("DSYRK", ctx, st);
}

/* ------------------------------------------------------- DTRSM / DTRMM */
typedef gbx_status (*trxm_fn)(gbx_ctx *, char, char, char, char, int, int, double, const double *,
                              int, double *, int);

static void trxm(const char *name, trxm_fn fn, const char *side, const char *uplo,
                 const char *transa, const char *diag, const int *m, const int *n,
                 const double *alpha, const double *a, const int *lda, double *b, const int *ldb)
{
    int info = gbx_check_trxm_args(*side, *uplo, *transa, *diag, *m, *n, *lda, *ldb);
    if (info) { xerbla_(name, &info, 6); return; }
    NOTE(fn == gbx_dtrsm ? "dtrsm_" : "dtrmm_", a);
    NOTE(fn == gbx_dtrsm ? "dtrsm_" : "dtrmm_", b);
    if (fn == gbx_dtrsm) GBX_FORWARD(dtrsm_, (side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb));
    else GBX_FORWARD(dtrmm_, (side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb));
    if (*m == 0 || *n == 0) return;
    gbx_ctx *ctx = ctx_or_report(name);
    if (!ctx) return;
    gbx_status st;
    const int na = gbx_lsame(*side, 'L') ? *m : *n;
    gbx_server *srv = fn == gbx_dtrsm ? server() : NULL;   /* DTRMM runs directly */
    const size_t bytes = 8 * ((size_t)na * na + (size_t)*m * *n);
    if (srv && (st = gbx_server_admit(srv, bytes)) != GBX_OK) { report(name, ctx, st); return; }
    gbx_operand oa = {.ld = *lda}, ob = {0};
    if (*alpha != 0.0) TRY(gbx_place_in(ctx, GBX_WS_STAGE_A, a, na, na, *lda, 8, 1, &oa));
    TRY(gbx_place_in(ctx, GBX_WS_STAGE_B, b, *m, *n, *ldb, 8, *alpha != 0.0, &ob));
    const int ozaki = fn == gbx_dtrsm && gbx_get_config()->precision_ozaki && *alpha != 0.0;
    if (srv) {
        gbx_op op = {0};
        op.kind = ozaki ? GBX_OP_TRSM_OZAKI : GBX_OP_TRSM;
        op.side = *side; op.uplo = *uplo; op.transa = *transa; op.diag = *diag;
        op.m = *m; op.n = *n; op.alpha = *alpha;
        op.A = oa.dev; op.lda = oa.ld; op.C = ob.dev; op.ldc = ob.ld;
        TRY(served(ctx, srv, &op));
    } else if (ozaki) {
        TRY(gbx_dtrsm_ozaki(ctx, *side, *uplo, *transa, *diag, *m, *n, *alpha, oa.dev, oa.ld, ob.dev, ob.ld,
                            gbx_get_config()->ozaki_tol, 0, NULL));
    } else {
        TRY(fn(ctx, *side, *uplo, *transa, *diag, *m, *n, *alpha, oa.dev, oa.ld, ob.dev, ob.ld));
    }
    TRY(gbx_place_out(ctx, &ob, *m, *n, 8));
    TRY(gbx_ctx_sync(ctx));
    if (srv) gbx_server_release(srv, bytes);
    return;
fail:
    if (srv) gbx_server_release(srv, bytes);
    report(name, ctx, st);
}

void dtrsm_(const char *side, const char *uplo, const char *transa, const char *diag,
            const int *m, const int *n, const double *alpha, const double *a, const int *lda,
            double *b, const int *ldb)
{
    trxm("DTRSM ", gbx_dtrsm, side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb);
}

void dtrmm_(const char *side, const char *uplo, const char *transa, const char *diag,
            const int *m, const int *n, const double *alpha, const double *a, const int *lda,
            double *b, const int *ldb)
{
    trxm("DTRMM ", gbx_dtrmm, side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb);
}

/* ---------------------------------------------------------------- DGEMV */
void dgemv_(const char *trans, const int *m, const int *n, const double *alpha, const double *a,
            const int *lda, const double *x, const int *incx, const double *beta, double *y,
            const int *incy)
{
    int info = gbx_check_gemv_args(*trans, *m, *n, *lda, *incx, *incy);
    if (info) { xerbla_("DGEMV ", &info, 6); return; }
    NOTE("dgemv_", a); NOTE("dgemv_", x); NOTE("dgemv_", y);
    GBX_FORWARD(dgemv_, (trans, m, n, alpha, a, lda, x, incx, beta, y, incy));
    if (*m == 0 || *n == 0 || (*alpha == 0.0 && *beta == 1.0)) return;
    gbx_ctx *ctx = ctx_or_report("DGEMV");
    if (!ctx) return;
    gbx_status st;
    const int notr = gbx_lsame(*trans, 'N');
    const int lenx = notr ? *n : *m, leny = notr ? *m : *n;
    gbx_operand oa = {.ld = *lda}, ox = {0}, oy = {0};
    if (*alpha != 0.0) {
        TRY(gbx_place_in(ctx, GBX_WS_STAGE_A, a, *m, *n, *lda, 8, 1, &oa));
        TRY(gbx_place_vec(ctx, GBX_WS_STAGE_B, x, lenx, *incx, 8, 1, &ox));
    }
    /* strided y: the staged span has gaps that must round-trip unchanged */
    const int yin = *beta != 0.0 || (*incy != 1 && *incy != -1);
    TRY(gbx_place_vec(ctx, GBX_WS_STAGE_C, y, leny, *incy, 8, yin, &oy));
    TRY(gbx_dgemv(ctx, *trans, *m, *n, *alpha, oa.dev, oa.ld, ox.dev, *incx, *beta, oy.dev, *incy));
    TRY(gbx_place_vec_out(ctx, &oy, leny, *incy, 8));
    TRY(gbx_ctx_sync(ctx));
    return;
fail:
    report("DGEMV", ctx, st);
}

/* ----------------------------------------------- DGER / DSYMV / DTRSV */
int gbx_check_ger_args(int m, int n, int incx, int incy, int lda);
int gbx_check_symv_args(char uplo, int n, int lda, int incx, int incy);
int gbx_check_trsv_args(char uplo, char trans, char diag, int n, int lda, int incx);

void dger_(const int *m, const int *n, const double *alpha, const double *x, const int *incx, const double *y,
           const int *incy, double *a, const int *lda)
{
    int info = gbx_check_ger_args(*m, *n, *incx, *incy, *lda);
    if (info) { xerbla_("DGER  ", &info, 6); return; }
    NOTE("dger_", x); NOTE("dger_", y); NOTE("dger_", a);
    GBX_FORWARD(dger_, (m, n, alpha, x, incx, y, incy, a, lda));
    if (*m == 0 || *n == 0 || *alpha == 0.0) return;
    gbx_ctx *ctx = ctx_or_report("DGER");
    if (!ctx) return;
    gbx_status st;
    gbx_operand oa = {0}, ox = {0}, oy = {0};
    TRY(gbx_place_vec(ctx, GBX_WS_STAGE_B, x, *m, *incx, 8, 1, &ox));
    TRY(gbx_place_vec(ctx, GBX_WS_STAGE_C, y, *n, *incy, 8, 1, &oy));
    TRY(gbx_place_in(ctx, GBX_WS_STAGE_A, a, *m, *n, *lda, 8, 1, &oa));
    TRY(gbx_dger(ctx, *m, *n, *alpha, ox.dev, *incx, oy.dev, *incy, oa.dev, oa.ld));
    TRY(gbx_place_out(ctx, &oa, *m, *n, 8));
    TRY(gbx_ctx_sync(ctx));
    return;
fail:
    report("DGER", ctx, st);
}

void dsymv_(const char *uplo, const int *n, const double *alpha, const double *a, const int *lda,
            const double *x, const int *incx, const double *beta, double *y, const int *incy)
{
    int info = gbx_check_symv_args(*uplo, *n, *lda, *incx, *incy);
    if (info) { xerbla_("DSYMV ", &info, 6); return; }
    NOTE("dsymv_", a); NOTE("dsymv_", x); NOTE("dsymv_", y);
    GBX_FORWARD(dsymv_, (uplo, n, alpha, a, lda, x, incx, beta, y, incy));
    if (*n == 0 || (*alpha == 0.0 && *beta == 1.0)) return;
    gbx_ctx *ctx = ctx_or_report("DSYMV");
    if (!ctx) return;
    gbx_status st;
    gbx_operand oa = {.ld = *lda}, ox = {0}, oy = {0};
    if (*alpha != 0.0) {
        TRY(gbx_place_in(ctx, GBX_WS_STAGE_A, a, *n, *n, *lda, 8, 1, &oa));
        TRY(gbx_place_vec(ctx, GBX_WS_STAGE_B, x, *n, *incx, 8, 1, &ox));
    }
    const int yin = *beta != 0.0 || (*incy != 1 && *incy != -1);
    TRY(gbx_place_vec(ctx, GBX_WS_STAGE_C, y, *n, *incy, 8, yin, &oy));
    TRY(gbx_dsymv(ctx, *uplo, *n, *alpha, oa.dev, oa.ld, ox.dev, *incx, *beta, oy.dev, *incy));
    TRY(gbx_place_vec_out(ctx, &oy, *n, *incy, 8));
    TRY(gbx_ctx_sync(ctx));
    return;
fail:
    report("DSYMV", ctx, st);
}

void dtrsv_(const char *uplo, const char *trans, const char *diag, const int *n, const double *a, const int *lda,
            double *x, const int *incx)
{
    int info = gbx_check_trsv_args(*uplo, *trans, *diag, *n, *lda, *incx);
    if (info) { xerbla_("DTRSV ", &info, 6); return; }
    NOTE("dtrsv_", a); NOTE("dtrsv_", x);
    GBX_FORWARD(dtrsv_, (uplo, trans, diag, n, a, lda, x, incx));
    if (*n == 0) return;
    gbx_ctx *ctx = ctx_or_report("DTRSV");
    if (!ctx) return;
    gbx_status st;
    gbx_operand oa = {0}, ox = {0};
    TRY(gbx_place_in(ctx, GBX_WS_STAGE_A, a, *n, *n, *lda, 8, 1, &oa));
    TRY(gbx_place_vec(ctx, GBX_WS_STAGE_B, x, *n, *incx, 8, 1, &ox));
    TRY(gbx_dtrsv(ctx, *uplo, *trans, *diag, *n, oa.dev, oa.ld, ox.dev, *incx));
    TRY(gbx_place_vec_out(ctx, &ox, *n, *incx, 8));
    TRY(gbx_ctx_sync(ctx));
    return;
fail:
    report("DTRSV", ctx, st);
}

/* ---------------------------------------------------------------- Level 1 */
void daxpy_(const int *n, const double *alpha, const double *x, const int *incx, double *y,
            const int *incy)
{
    if (*n <= 0 || *alpha == 0.0) return;
    NOTE("daxpy_", x); NOTE("daxpy_", y);
    GBX_FORWARD(daxpy_, (n, alpha, x, incx, y, incy));
    gbx_ctx *ctx = ctx_or_report("DAXPY");
    if (!ctx) return;
    gbx_status st;
    gbx_operand ox = {0}, oy = {0};
    TRY(gbx_place_vec(ctx, GBX_WS_STAGE_A, x, *n, *incx, 8, 1, &ox));
    TRY(gbx_place_vec(ctx, GBX_WS_STAGE_B, y, *n, *incy, 8, 1, &oy));
    TRY(gbx_daxpy(ctx, *n, *alpha, ox.dev, *incx, oy.dev, *incy));
    TRY(gbx_place_vec_out(ctx, &oy, *n, *incy, 8));
    TRY(gbx_ctx_sync(ctx));
    return;
fail:
    report("DAXPY", ctx, st);
}

double ddot_(const int *n, const double *x, const int *incx, const double *y, const int *incy)
{
    if (*n <= 0) return 0.0;
    NOTE("ddot_", x); NOTE("ddot_", y);
    GBX_FORWARD_RET(ddot_, (n, x, incx, y, incy));
    gbx_ctx *ctx = ctx_or_report("DDOT");
    if (!ctx) return 0.0;
    gbx_status st;
    gbx_operand ox = {0}, oy = {0};
    double *res;
    TRY(gbx_pinned(ctx, sizeof(double), (void **)&res));
    TRY(gbx_place_vec(ctx, GBX_WS_STAGE_A, x, *n, *incx, 8, 1, &ox));
    TRY(gbx_place_vec(ctx, GBX_WS_STAGE_B, y, *n, *incy, 8, 1, &oy));
    TRY(gbx_ddot(ctx, *n, ox.dev, *incx, oy.dev, *incy, res));
    TRY(gbx_ctx_sync(ctx));
    return *res;
fail:
    report("DDOT", ctx, st);
    return 0.0;
}

double dnrm2_(const int *n, const double *x, const int *incx)
{
    if (*n < 1 || *incx < 1) return 0.0;
    NOTE("dnrm2_", x);
    GBX_FORWARD_RET(dnrm2_, (n, x, incx));
    gbx_ctx *ctx = ctx_or_report("DNRM2");
    if (!ctx) return 0.0;
    gbx_status st;
    gbx_operand ox = {0};
    double *res;
    TRY(gbx_pinned(ctx, sizeof(double), (void **)&res));
    TRY(gbx_place_vec(ctx, GBX_WS_STAGE_A, x, *n, *incx, 8, 1, &ox));
    TRY(gbx_dnrm2(ctx, *n, ox.dev, *incx, res));
    TRY(gbx_ctx_sync(ctx));
    return *res;
fail:
    report("DNRM2", ctx, st);
    return 0.0;
}

static int iamx(const char *name, int is_min, const int *n, const double *x, const int *incx)
{
    if (*n < 1 || *incx <= 0) return 0;
    NOTE(is_min ? "idamin_" : "idamax_", x);
    if (is_min) GBX_FORWARD_RET(idamin_, (n, x, incx));
    else GBX_FORWARD_RET(idamax_, (n, x, incx));
    if (*n == 1) return 1;
    gbx_ctx *ctx = ctx_or_report(name);
    if (!ctx) return 0;
    gbx_status st;
    gbx_operand ox = {0};
    int *res;
    TRY(gbx_pinned(ctx, sizeof(int), (void **)&res));
    TRY(gbx_place_vec(ctx, GBX_WS_STAGE_A, x, *n, *incx, 8, 1, &ox));
    TRY(is_min ? gbx_idamin(ctx, *n, ox.dev, *incx, res) : gbx_idamax(ctx, *n, ox.dev, *incx, res));
    TRY(gbx_ctx_sync(ctx));
    return *res;
fail:
    report(name, ctx, st);
    return 0;
}

int idamax_(const int *n, const double *x, const int *incx) { return iamx("IDAMAX", 0, n, x, incx); }
int idamin_(const int *n, const double *x, const int *incx) { return iamx("IDAMIN", 1, n, x, incx); }

/* ------------------------------------------------------------------ CBLAS
 * Row-major calls are mapped onto the column-major routines by transposing
 * the problem (C^T = op(B)^T op(A)^T, and so on), which is the standard CBLAS
 * construction.  Parameter errors are reported through xerbla_ with the
 * Fortran routine's numbering; an invalid layout reports position 1.       */
static char tch(int t) { return t == GbxNoTrans ? 'N' : t == GbxTrans ? 'T' : t == GbxConjTrans ? 'C' : '?'; }
static char uch(int u) { return u == GbxUpper ? 'U' : u == GbxLower ? 'L' : '?'; }
static char dch(int d) { return d == GbxUnit ? 'U' : d == GbxNonUnit ? 'N' : '?'; }
static char sch(int s) { return s == GbxLeft ? 'L' : s == GbxRight ? 'R' : '?'; }
static char flip_t(char t) { return t == 'N' ? 'T' : t == '?' ? '?' : 'N'; }
static char flip_u(char u) { return u == 'U' ? 'L' : u == 'L' ? 'U' : '?'; }
static char flip_s(char s) { return s == 'L' ? 'R' : s == 'R' ? 'L' : '?'; }

static int bad_layout(int layout, const char *name)
{
    if (layout == GbxRowMajor || layout == GbxColMajor) return 0;
    int info = 1;
    xerbla_(name, &info, 6);
    return 1;
}

void cblas_dgemm(int layout, int transa, int transb, int m, int n, int k, double alpha,
                 const double *a, int lda, const double *b, int ldb, double beta, double *c, int ldc)
{
    if (bad_layout(layout, "DGEMM ")) return;
    char ta = tch(transa), tb = tch(transb);
    if (layout == GbxColMajor)
        dgemm_(&ta, &tb, &m, &n, &k, &alpha, a, &lda, b, &ldb, &beta, c, &ldc);
    else
        dgemm_(&tb, &ta, &n, &m, &k, &alpha, b, &ldb, a, &lda, &beta, c, &ldc);
}

void cblas_zgemm(int layout, int transa, int transb, int m, int n, int k, const void *alpha,
                 const void *a, int lda, const void *b, int ldb, const void *beta, void *c, int ldc)
{
    if (bad_layout(layout, "ZGEMM ")) return;
    char ta = tch(transa), tb = tch(transb);
    if (layout == GbxColMajor)
        zgemm_(&ta, &tb, &m, &n, &k, alpha, a, &lda, b, &ldb, beta, c, &ldc);
    else
        zgemm_(&tb, &ta, &n, &m, &k, alpha, b, &ldb, a, &lda, beta, c, &ldc);
}

void cblas_dsyrk(int layout, int uplo, int trans, int n, int k, double alpha, const double *a,
                 int lda, double beta, double *c, int ldc)
{
    if (bad_layout(layout, "DSYRK ")) return;
    char u = uch(uplo), t = tch(trans);
    if (layout == GbxRowMajor) { u = flip_u(u); t = flip_t(t); }
    dsyrk_(&u, &t, &n, &k, &alpha, a, &lda, &beta, c, &ldc);
}

static void cblas_trxm(int trsm, int layout, int side, int uplo, int transa, int diag, int m, int n,
                       double alpha, const double *a, int lda, double *b, int ldb)
{
    if (bad_layout(layout, trsm ? "DTRSM " : "DTRMM ")) return;
    char s = sch(side), u = uch(uplo), t = tch(transa), d = dch(diag);
    if (layout == GbxRowMajor) {
        s = flip_s(s);
        u = flip_u(u);
        int tmp = m; m = n; n = tmp;
    }
    if (trsm) dtrsm_(&s, &u, &t, &d, &m, &n, &alpha, a, &lda, b, &ldb);
    else dtrmm_(&s, &u, &t, &d, &m, &n, &alpha, a, &lda, b, &ldb);
}

void cblas_dtrsm(int layout, int side, int uplo, int transa, int diag, int m, int n, double alpha,
                 const double *a, int lda, double *b, int ldb)
{
    cblas_trxm(1, layout, side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb);
}

void cblas_dtrmm(int layout, int side, int uplo, int transa, int diag, int m, int n, double alpha,
                 const double *a, int lda, double *b, int ldb)
{
    cblas_trxm(0, layout, side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb);
}

void cblas_dgemv(int layout, int trans, int m, int n, double alpha, const double *a, int lda,
                 const double *x, int incx, double beta, double *y, int incy)
{
    if (bad_layout(layout, "DGEMV ")) return;
    char t = tch(trans);
    if (layout == GbxRowMajor) {
        t = flip_t(t);
        int tmp = m; m = n; n = tmp;
    }
    dgemv_(&t, &m, &n, &alpha, a, &lda, x, &incx, &beta, y, &incy);
}

/* row-major: A^T += alpha y x^T */
void cblas_dger(int layout, int m, int n, double alpha, const double *x, int incx, const double *y, int incy,
                double *a, int lda)
{
    if (bad_layout(layout, "DGER  ")) return;
    if (layout == GbxColMajor) dger_(&m, &n, &alpha, x, &incx, y, &incy, a, &lda);
    else dger_(&n, &m, &alpha, y, &incy, x, &incx, a, &lda);
}

/* row-major: the stored triangle flips (A^T = A) */
void cblas_dsymv(int layout, int uplo, int n, double alpha, const double *a, int lda, const double *x, int incx,
                 double beta, double *y, int incy)
{
    if (bad_layout(layout, "DSYMV ")) return;
    char u = uch(uplo);
    if (layout == GbxRowMajor) u = flip_u(u);
    dsymv_(&u, &n, &alpha, a, &lda, x, &incx, &beta, y, &incy);
}

/* row-major: op(A) on A^T: the triangle flips and N <-> T */
void cblas_dtrsv(int layout, int uplo, int trans, int diag, int n, const double *a, int lda, double *x, int incx)
{
    if (bad_layout(layout, "DTRSV ")) return;
    char u = uch(uplo), t = tch(trans), d = dch(diag);
    if (layout == GbxRowMajor) { u = flip_u(u); t = flip_t(t); }
    dtrsv_(&u, &t, &d, &n, a, &lda, x, &incx);
}

void cblas_daxpy(int n, double alpha, const double *x, int incx, double *y, int incy)
{
    daxpy_(&n, &alpha, x, &incx, y, &incy);
}

double cblas_ddot(int n, const double *x, int incx, const double *y, int incy)
{
    return ddot_(&n, x, &incx, y, &incy);
}

double cblas_dnrm2(int n, const double *x, int incx) { return dnrm2_(&n, x, &incx); }

int cblas_idamax(int n, const double *x, int incx)
{
    int i = idamax_(&n, x, &incx);
    return i ? i - 1 : 0;
}

int cblas_idamin(int n, const double *x, int incx)
{
    int i = idamin_(&n, x, &incx);
    return i ? i - 1 : 0;
}
