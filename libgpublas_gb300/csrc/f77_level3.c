/*
 * f77_level3.c — Fortran-ABI and CBLAS entry points of the Level-3 routines
 * beyond the D/Z set of f77.c: xGEMM for S and C, xSYMM, xHEMM, xSYRK (S, C,
 * Z), xHERK, xSYR2K, xHER2K, xTRMM (S, C, Z) and xTRSM (S, C, Z).  These are
 * the symbols the reference exports from blas_level3/<routine>.cc (F77_gemm,
 * F77_symm, ... prototypes at blas.h:202-314); the reference hands each to
 * cuBLAS after its argument check.
 *
 * Every routine has the shape of f77.c's: netlib argument check (xerbla_
 * with the netlib position) -> netlib quick return -> placement of the
 * operands (device/managed memory used in place, host memory staged) ->
 * the gbx_* device routine -> copy-back -> synchronize.  Complex scalars are
 * pointers to (re, im) pairs.
 *
 * CBLAS: the standard C interface (complex scalars by pointer, real scalars
 * of the Hermitian routines by value).  Row-major calls are mapped onto the
 * column-major routines by transposing the problem; parameter errors report
 * the Fortran routine's numbering, an invalid layout position 1.
 */
#include "gbx_internal.h"
#include "../../include/gbxblas_f77.h"

#include <stddef.h>

#define NOTE(fun, p)                                    \
    do {                                                \
        if (gbx_tracker_note) gbx_tracker_note(fun, p); \
    } while (0)

/* ---- shared staging path ------------------------------------------------ */
typedef struct {
    const void *p;   /* caller's pointer (NULL: operand absent) */
    int rows, cols, ld;
} l3_mat;

typedef gbx_status (*l3_fn)(gbx_ctx *ctx, const gbx_operand *a, const gbx_operand *b, gbx_operand *c,
                            const void *args);

/* Places a and b (when the call has work), places the output c (copied in
 * when its old contents are read), runs fn, copies c back, synchronizes. */
static void l3_run(const char *name, size_t esz, int work, l3_mat a, l3_mat b, l3_mat c, int c_in, l3_fn fn,
                   const void *args)
{
    gbx_ctx *ctx = gbx_f77_ctx(name);
    if (!ctx) return;
    gbx_status st;
    /* operands left unplaced on quick paths keep the caller's (valid) ld */
    gbx_operand oa = {.ld = a.ld}, ob = {.ld = b.ld}, oc = {0};
    if (work && a.p &&
        (st = gbx_place_in(ctx, GBX_WS_STAGE_A, a.p, a.rows, a.cols, a.ld, esz, 1, &oa)) != GBX_OK)
        goto fail;
    if (work && b.p &&
        (st = gbx_place_in(ctx, GBX_WS_STAGE_B, b.p, b.rows, b.cols, b.ld, esz, 1, &ob)) != GBX_OK)
        goto fail;
    if ((st = gbx_place_in(ctx, GBX_WS_STAGE_C, c.p, c.rows, c.cols, c.ld, esz, c_in, &oc)) != GBX_OK) goto fail;
    if ((st = fn(ctx, &oa, &ob, &oc, args)) != GBX_OK) goto fail;
    if ((st = gbx_place_out(ctx, &oc, c.rows, c.cols, esz)) != GBX_OK) goto fail;
    if ((st = gbx_ctx_sync(ctx)) != GBX_OK) goto fail;
    return;
fail:
    gbx_f77_report(name, ctx, st);
}

static int z2(const float *a) { return a[0] == 0.0f && a[1] == 0.0f; }
static int o2(const float *a) { return a[0] == 1.0f && a[1] == 0.0f; }
static int zz(const double *a) { return a[0] == 0.0 && a[1] == 0.0; }
static int oz(const double *a) { return a[0] == 1.0 && a[1] == 0.0; }

/* ---------------------------------------------------------------- xGEMM */
struct gemm_args {
    char ta, tb;
    int m, n, k;
    const void *alpha, *beta;
};

static gbx_status run_sgemm(gbx_ctx *ctx, const gbx_operand *a, const gbx_operand *b, gbx_operand *c,
                            const void *v)
{
    const struct gemm_args *g = v;
    return gbx_sgemm(ctx, g->ta, g->tb, g->m, g->n, g->k, *(const float *)g->alpha, a->dev, a->ld, b->dev, b->ld,
                     *(const float *)g->beta, c->dev, c->ld);
}

static gbx_status run_cgemm(gbx_ctx *ctx, const gbx_operand *a, const gbx_operand *b, gbx_operand *c,
                            const void *v)
{
    const struct gemm_args *g = v;
    return gbx_cgemm(ctx, g->ta, g->tb, g->m, g->n, g->k, g->alpha, a->dev, a->ld, b->dev, b->ld, g->beta, c->dev,
                     c->ld);
}

#define GEMM_BODY(LABEL, NAME, SYM, ESZ, RUN, ALPHA0, BETA0, BETA1)                                                  \
    int info = gbx_check_gemm_args(*transa, *transb, *m, *n, *k, *lda, *ldb, *ldc);                             \
    if (info) { xerbla_(LABEL, &info, 6); return; }                                                             \
    NOTE(NAME, a); NOTE(NAME, b); NOTE(NAME, c);                                                                \
    GBX_FORWARD(SYM, (transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc));                           \
    if (*m == 0 || *n == 0 || (((ALPHA0) || *k == 0) && (BETA1))) return;                                       \
    const int nota = gbx_lsame(*transa, 'N'), notb = gbx_lsame(*transb, 'N');                                  \
    struct gemm_args g = {*transa, *transb, *m, *n, *k, alpha, beta};                                           \
    l3_run(LABEL, ESZ, !((ALPHA0) || *k == 0), (l3_mat){a, nota ? *m : *k, nota ? *k : *m, *lda},              \
           (l3_mat){b, notb ? *k : *n, notb ? *n : *k, *ldb}, (l3_mat){c, *m, *n, *ldc}, !(BETA0), RUN, &g);

void sgemm_(const char *transa, const char *transb, const int *m, const int *n, const int *k, const float *alpha,
            const float *a, const int *lda, const float *b, const int *ldb, const float *beta, float *c,
            const int *ldc)
{
    GEMM_BODY("SGEMM ", "sgemm_", sgemm_, 4, run_sgemm, *alpha == 0.0f, *beta == 0.0f, *beta == 1.0f)
}

void cgemm_(const char *transa, const char *transb, const int *m, const int *n, const int *k, const float *alpha,
            const float *a, const int *lda, const float *b, const int *ldb, const float *beta, float *c,
            const int *ldc)
{
    GEMM_BODY("CGEMM ", "cgemm_", cgemm_, 8, run_cgemm, z2(alpha), z2(beta), o2(beta))
}

/* -------------------------------------------------------- xSYMM / xHEMM */
struct symm_args {
    char side, uplo;
    int m, n;
    const void *alpha, *beta;
};

#define RUN_SYMM_REAL(FN, T)                                                                                    \
    static gbx_status run_##FN(gbx_ctx *ctx, const gbx_operand *a, const gbx_operand *b, gbx_operand *c,       \
                               const void *v)                                                                   \
    {                                                                                                           \
        const struct symm_args *s = v;                                                                          \
        return gbx_##FN(ctx, s->side, s->uplo, s->m, s->n, *(const T *)s->alpha, a->dev, a->ld, b->dev, b->ld, \
                        *(const T *)s->beta, c->dev, c->ld);                                                    \
    }
#define RUN_SYMM_CPLX(FN)                                                                                       \
    static gbx_status run_##FN(gbx_ctx *ctx, const gbx_operand *a, const gbx_operand *b, gbx_operand *c,       \
                               const void *v)                                                                   \
    {                                                                                                           \
        const struct symm_args *s = v;                                                                          \
        return gbx_##FN(ctx, s->side, s->uplo, s->m, s->n, s->alpha, a->dev, a->ld, b->dev, b->ld, s->beta,    \
                        c->dev, c->ld);                                                                         \
    }
RUN_SYMM_REAL(ssymm, float)
RUN_SYMM_REAL(dsymm, double)
RUN_SYMM_CPLX(csymm)
RUN_SYMM_CPLX(zsymm)
RUN_SYMM_CPLX(chemm)
RUN_SYMM_CPLX(zhemm)

#define SYMM_BODY(LABEL, NAME, SYM, ESZ, RUN, ALPHA0, BETA0, BETA1)                                                  \
    int info = gbx_check_symm_args(*side, *uplo, *m, *n, *lda, *ldb, *ldc);                                     \
    if (info) { xerbla_(LABEL, &info, 6); return; }                                                             \
    NOTE(NAME, a); NOTE(NAME, b); NOTE(NAME, c);                                                                \
    GBX_FORWARD(SYM, (side, uplo, m, n, alpha, a, lda, b, ldb, beta, c, ldc));                                  \
    if (*m == 0 || *n == 0 || ((ALPHA0) && (BETA1))) return;                                                    \
    const int na = gbx_lsame(*side, 'L') ? *m : *n;                                                             \
    struct symm_args s = {*side, *uplo, *m, *n, alpha, beta};                                                   \
    l3_run(LABEL, ESZ, !(ALPHA0), (l3_mat){a, na, na, *lda}, (l3_mat){b, *m, *n, *ldb},                        \
           (l3_mat){c, *m, *n, *ldc}, !(BETA0), RUN, &s);

#define SYMM_PROTO(FN, T)                                                                                       \
    void FN##_(const char *side, const char *uplo, const int *m, const int *n, const T *alpha, const T *a,      \
               const int *lda, const T *b, const int *ldb, const T *beta, T *c, const int *ldc)

SYMM_PROTO(ssymm, float) { SYMM_BODY("SSYMM ", "ssymm_", ssymm_, 4, run_ssymm, *alpha == 0.0f, *beta == 0.0f, *beta == 1.0f) }
SYMM_PROTO(dsymm, double) { SYMM_BODY("DSYMM ", "dsymm_", dsymm_, 8, run_dsymm, *alpha == 0.0, *beta == 0.0, *beta == 1.0) }
SYMM_PROTO(csymm, float) { SYMM_BODY("CSYMM ", "csymm_", csymm_, 8, run_csymm, z2(alpha), z2(beta), o2(beta)) }
SYMM_PROTO(zsymm, double) { SYMM_BODY("ZSYMM ", "zsymm_", zsymm_, 16, run_zsymm, zz(alpha), zz(beta), oz(beta)) }
SYMM_PROTO(chemm, float) { SYMM_BODY("CHEMM ", "chemm_", chemm_, 8, run_chemm, z2(alpha), z2(beta), o2(beta)) }
SYMM_PROTO(zhemm, double) { SYMM_BODY("ZHEMM ", "zhemm_", zhemm_, 16, run_zhemm, zz(alpha), zz(beta), oz(beta)) }

/* -------------------------------------------------------- xSYRK / xHERK */
struct rk_args {
    char uplo, trans;
    int n, k;
    const void *alpha, *beta;
    const void *b;   /* rank-2k second operand (device pointer set at run) */
};

#define RUN_SYRK_SCALAR(FN, T)                                                                                  \
    static gbx_status run_##FN(gbx_ctx *ctx, const gbx_operand *a, const gbx_operand *b, gbx_operand *c,       \
                               const void *v)                                                                   \
    {                                                                                                           \
        const struct rk_args *r = v;                                                                            \
        (void)b;                                                                                                \
        return gbx_##FN(ctx, r->uplo, r->trans, r->n, r->k, *(const T *)r->alpha, a->dev, a->ld,               \
                        *(const T *)r->beta, c->dev, c->ld);                                                    \
    }
#define RUN_SYRK_CPLX(FN)                                                                                       \
    static gbx_status run_##FN(gbx_ctx *ctx, const gbx_operand *a, const gbx_operand *b, gbx_operand *c,       \
                               const void *v)                                                                   \
    {                                                                                                           \
        const struct rk_args *r = v;                                                                            \
        (void)b;                                                                                                \
        return gbx_##FN(ctx, r->uplo, r->trans, r->n, r->k, r->alpha, a->dev, a->ld, r->beta, c->dev, c->ld); \
    }
RUN_SYRK_SCALAR(ssyrk, float)
RUN_SYRK_CPLX(csyrk)
RUN_SYRK_CPLX(zsyrk)
RUN_SYRK_SCALAR(cherk, float)
RUN_SYRK_SCALAR(zherk, double)

#define RK_BODY(LABEL, NAME, SYM, ESZ, RUN, ALLOWED, ALPHA0, BETA1)                                                  \
    int info = gbx_check_rank_k_args(*uplo, *trans, ALLOWED, *n, *k, *lda, *ldc);                               \
    if (info) { xerbla_(LABEL, &info, 6); return; }                                                             \
    NOTE(NAME, a); NOTE(NAME, c);                                                                               \
    GBX_FORWARD(SYM, (uplo, trans, n, k, alpha, a, lda, beta, c, ldc));                                         \
    if (*n == 0 || (((ALPHA0) || *k == 0) && (BETA1))) return;                                                  \
    const int notr = gbx_lsame(*trans, 'N');                                                                    \
    struct rk_args r = {*uplo, *trans, *n, *k, alpha, beta, NULL};                                              \
    /* the other triangle of C must survive the round trip: always copy in */                                   \
    l3_run(LABEL, ESZ, !((ALPHA0) || *k == 0), (l3_mat){a, notr ? *n : *k, notr ? *k : *n, *lda},              \
           (l3_mat){NULL, 0, 0, 1}, (l3_mat){c, *n, *n, *ldc}, 1, RUN, &r);

#define RK_PROTO(FN, T, S)                                                                                      \
    void FN##_(const char *uplo, const char *trans, const int *n, const int *k, const S *alpha, const T *a,     \
               const int *lda, const S *beta, T *c, const int *ldc)

RK_PROTO(ssyrk, float, float)
{
    RK_BODY("SSYRK ", "ssyrk_", ssyrk_, 4, run_ssyrk, GBX_TR_N | GBX_TR_T | GBX_TR_C, *alpha == 0.0f, *beta == 1.0f)
}
RK_PROTO(csyrk, float, float) { RK_BODY("CSYRK ", "csyrk_", csyrk_, 8, run_csyrk, GBX_TR_N | GBX_TR_T, z2(alpha), o2(beta)) }
RK_PROTO(zsyrk, double, double) { RK_BODY("ZSYRK ", "zsyrk_", zsyrk_, 16, run_zsyrk, GBX_TR_N | GBX_TR_T, zz(alpha), oz(beta)) }
RK_PROTO(cherk, float, float)
{
    RK_BODY("CHERK ", "cherk_", cherk_, 8, run_cherk, GBX_TR_N | GBX_TR_C, *alpha == 0.0f, *beta == 1.0f)
}
RK_PROTO(zherk, double, double)
{
    RK_BODY("ZHERK ", "zherk_", zherk_, 16, run_zherk, GBX_TR_N | GBX_TR_C, *alpha == 0.0, *beta == 1.0)
}

/* ------------------------------------------------------ xSYR2K / xHER2K */
#define RUN_R2K_REAL(FN, T)                                                                                     \
    static gbx_status run_##FN(gbx_ctx *ctx, const gbx_operand *a, const gbx_operand *b, gbx_operand *c,       \
                               const void *v)                                                                   \
    {                                                                                                           \
        const struct rk_args *r = v;                                                                            \
        return gbx_##FN(ctx, r->uplo, r->trans, r->n, r->k, *(const T *)r->alpha, a->dev, a->ld, b->dev, b->ld, \
                        *(const T *)r->beta, c->dev, c->ld);                                                    \
    }
#define RUN_R2K_CPLX(FN)                                                                                        \
    static gbx_status run_##FN(gbx_ctx *ctx, const gbx_operand *a, const gbx_operand *b, gbx_operand *c,       \
                               const void *v)                                                                   \
    {                                                                                                           \
        const struct rk_args *r = v;                                                                            \
        return gbx_##FN(ctx, r->uplo, r->trans, r->n, r->k, r->alpha, a->dev, a->ld, b->dev, b->ld, r->beta,   \
                        c->dev, c->ld);                                                                         \
    }
#define RUN_R2K_HERM(FN, T)                                                                                     \
    static gbx_status run_##FN(gbx_ctx *ctx, const gbx_operand *a, const gbx_operand *b, gbx_operand *c,       \
                               const void *v)                                                                   \
    {                                                                                                           \
        const struct rk_args *r = v;                                                                            \
        return gbx_##FN(ctx, r->uplo, r->trans, r->n, r->k, r->alpha, a->dev, a->ld, b->dev, b->ld,            \
                        *(const T *)r->beta, c->dev, c->ld);                                                    \
    }
RUN_R2K_REAL(ssyr2k, float)
RUN_R2K_REAL(dsyr2k, double)
RUN_R2K_CPLX(csyr2k)
RUN_R2K_CPLX(zsyr2k)
RUN_R2K_HERM(cher2k, float)
RUN_R2K_HERM(zher2k, double)

#define R2K_BODY(LABEL, NAME, SYM, ESZ, RUN, ALLOWED, ALPHA0, BETA1)                                                 \
    int info = gbx_check_rank_2k_args(*uplo, *trans, ALLOWED, *n, *k, *lda, *ldb, *ldc);                        \
    if (info) { xerbla_(LABEL, &info, 6); return; }                                                             \
    NOTE(NAME, a); NOTE(NAME, b); NOTE(NAME, c);                                                                \
    GBX_FORWARD(SYM, (uplo, trans, n, k, alpha, a, lda, b, ldb, beta, c, ldc));                                 \
    if (*n == 0 || (((ALPHA0) || *k == 0) && (BETA1))) return;                                                  \
    const int notr = gbx_lsame(*trans, 'N');                                                                    \
    struct rk_args r = {*uplo, *trans, *n, *k, alpha, beta, NULL};                                              \
    l3_run(LABEL, ESZ, !((ALPHA0) || *k == 0), (l3_mat){a, notr ? *n : *k, notr ? *k : *n, *lda},              \
           (l3_mat){b, notr ? *n : *k, notr ? *k : *n, *ldb}, (l3_mat){c, *n, *n, *ldc}, 1, RUN, &r);

#define R2K_PROTO(FN, T, S)                                                                                     \
    void FN##_(const char *uplo, const char *trans, const int *n, const int *k, const T *alpha, const T *a,     \
               const int *lda, const T *b, const int *ldb, const S *beta, T *c, const int *ldc)

R2K_PROTO(ssyr2k, float, float)
{
    R2K_BODY("SSYR2K", "ssyr2k_", ssyr2k_, 4, run_ssyr2k, GBX_TR_N | GBX_TR_T | GBX_TR_C, *alpha == 0.0f, *beta == 1.0f)
}
R2K_PROTO(dsyr2k, double, double)
{
    R2K_BODY("DSYR2K", "dsyr2k_", dsyr2k_, 8, run_dsyr2k, GBX_TR_N | GBX_TR_T | GBX_TR_C, *alpha == 0.0, *beta == 1.0)
}
R2K_PROTO(csyr2k, float, float)
{
    R2K_BODY("CSYR2K", "csyr2k_", csyr2k_, 8, run_csyr2k, GBX_TR_N | GBX_TR_T, z2(alpha), o2(beta))
}
R2K_PROTO(zsyr2k, double, double)
{
    R2K_BODY("ZSYR2K", "zsyr2k_", zsyr2k_, 16, run_zsyr2k, GBX_TR_N | GBX_TR_T, zz(alpha), oz(beta))
}
R2K_PROTO(cher2k, float, float)
{
    R2K_BODY("CHER2K", "cher2k_", cher2k_, 8, run_cher2k, GBX_TR_N | GBX_TR_C, z2(alpha), *beta == 1.0f)
}
R2K_PROTO(zher2k, double, double)
{
    R2K_BODY("ZHER2K", "zher2k_", zher2k_, 16, run_zher2k, GBX_TR_N | GBX_TR_C, zz(alpha), *beta == 1.0)
}

/* -------------------------------------------------------- xTRMM / xTRSM */
struct tr_args {
    char side, uplo, ta, diag;
    int m, n;
    const void *alpha;
};

#define RUN_TR_REAL(FN, T)                                                                                      \
    static gbx_status run_##FN(gbx_ctx *ctx, const gbx_operand *a, const gbx_operand *b, gbx_operand *c,       \
                               const void *v)                                                                   \
    {                                                                                                           \
        const struct tr_args *t = v;                                                                            \
        (void)b;                                                                                                \
        return gbx_##FN(ctx, t->side, t->uplo, t->ta, t->diag, t->m, t->n, *(const T *)t->alpha, a->dev,       \
                        a->ld, c->dev, c->ld);                                                                  \
    }
#define RUN_TR_CPLX(FN)                                                                                         \
    static gbx_status run_##FN(gbx_ctx *ctx, const gbx_operand *a, const gbx_operand *b, gbx_operand *c,       \
                               const void *v)                                                                   \
    {                                                                                                           \
        const struct tr_args *t = v;                                                                            \
        (void)b;                                                                                                \
        return gbx_##FN(ctx, t->side, t->uplo, t->ta, t->diag, t->m, t->n, t->alpha, a->dev, a->ld, c->dev,    \
                        c->ld);                                                                                 \
    }
RUN_TR_REAL(strmm, float)
RUN_TR_CPLX(ctrmm)
RUN_TR_CPLX(ztrmm)
RUN_TR_REAL(strsm, float)
RUN_TR_CPLX(ctrsm)
RUN_TR_CPLX(ztrsm)

#define TR_BODY(LABEL, NAME, SYM, ESZ, RUN, ALPHA0)                                                                  \
    int info = gbx_check_trxm_args(*side, *uplo, *transa, *diag, *m, *n, *lda, *ldb);                           \
    if (info) { xerbla_(LABEL, &info, 6); return; }                                                             \
    NOTE(NAME, a); NOTE(NAME, b);                                                                               \
    GBX_FORWARD(SYM, (side, uplo, transa, diag, m, n, alpha, a, lda, b, ldb));                                  \
    if (*m == 0 || *n == 0) return;                                                                             \
    const int na = gbx_lsame(*side, 'L') ? *m : *n;                                                             \
    struct tr_args t = {*side, *uplo, *transa, *diag, *m, *n, alpha};                                           \
    l3_run(LABEL, ESZ, !(ALPHA0), (l3_mat){a, na, na, *lda}, (l3_mat){NULL, 0, 0, 1},                          \
           (l3_mat){b, *m, *n, *ldb}, !(ALPHA0), RUN, &t);

#define TR_PROTO(FN, T)                                                                                         \
    void FN##_(const char *side, const char *uplo, const char *transa, const char *diag, const int *m,          \
               const int *n, const T *alpha, const T *a, const int *lda, T *b, const int *ldb)

TR_PROTO(strmm, float) { TR_BODY("STRMM ", "strmm_", strmm_, 4, run_strmm, *alpha == 0.0f) }
TR_PROTO(ctrmm, float) { TR_BODY("CTRMM ", "ctrmm_", ctrmm_, 8, run_ctrmm, z2(alpha)) }
TR_PROTO(ztrmm, double) { TR_BODY("ZTRMM ", "ztrmm_", ztrmm_, 16, run_ztrmm, zz(alpha)) }
TR_PROTO(strsm, float) { TR_BODY("STRSM ", "strsm_", strsm_, 4, run_strsm, *alpha == 0.0f) }
TR_PROTO(ctrsm, float) { TR_BODY("CTRSM ", "ctrsm_", ctrsm_, 8, run_ctrsm, z2(alpha)) }
TR_PROTO(ztrsm, double) { TR_BODY("ZTRSM ", "ztrsm_", ztrsm_, 16, run_ztrsm, zz(alpha)) }

/* ------------------------------------------------------------------ CBLAS */
static char tch(int t) { return t == GbxNoTrans ? 'N' : t == GbxTrans ? 'T' : t == GbxConjTrans ? 'C' : '?'; }
static char uch(int u) { return u == GbxUpper ? 'U' : u == GbxLower ? 'L' : '?'; }
static char dch(int d) { return d == GbxUnit ? 'U' : d == GbxNonUnit ? 'N' : '?'; }
static char sch(int s) { return s == GbxLeft ? 'L' : s == GbxRight ? 'R' : '?'; }
static char flip_u(char u) { return u == 'U' ? 'L' : u == 'L' ? 'U' : '?'; }
static char flip_s(char s) { return s == 'L' ? 'R' : s == 'R' ? 'L' : '?'; }
/* rank-k / rank-2k row-major: the transposition letter swaps between N and
 * the routine's other letter (T for symmetric, C for Hermitian) */
static char flip_rk(char t, char other) { return t == 'N' ? other : t == '?' ? '?' : 'N'; }

static int bad_layout(int layout, const char *name)
{
    if (layout == GbxRowMajor || layout == GbxColMajor) return 0;
    int info = 1;
    xerbla_(name, &info, 6);
    return 1;
}

/* C^T = op(B)^T op(A)^T */
#define CBLAS_GEMM(FN, T, S, LABEL, BYREF)                                                                       \
    void cblas_##FN(int layout, int transa, int transb, int m, int n, int k, S alpha, const void *a, int lda,   \
                    const void *b, int ldb, S beta, void *c, int ldc)                                            \
    {                                                                                                            \
        if (bad_layout(layout, LABEL)) return;                                                                   \
        char ta = tch(transa), tb = tch(transb);                                                                 \
        if (layout == GbxColMajor)                                                                               \
            FN##_(&ta, &tb, &m, &n, &k, BYREF(alpha), a, &lda, b, &ldb, BYREF(beta), c, &ldc);                  \
        else                                                                                                     \
            FN##_(&tb, &ta, &n, &m, &k, BYREF(alpha), b, &ldb, a, &lda, BYREF(beta), c, &ldc);                  \
    }
#define ADDR(x) (&(x))
#define PTR(x) ((const void *)(x))
CBLAS_GEMM(sgemm, float, float, "SGEMM ", ADDR)
CBLAS_GEMM(cgemm, float, const void *, "CGEMM ", PTR)

/* row-major: C^T = B^T A^T with A^T symmetric (Hermitian) stored in the
 * opposite triangle; side and uplo flip, m and n swap */
#define CBLAS_SYMM(FN, S, LABEL, BYREF)                                                                          \
    void cblas_##FN(int layout, int side, int uplo, int m, int n, S alpha, const void *a, int lda,              \
                    const void *b, int ldb, S beta, void *c, int ldc)                                            \
    {                                                                                                            \
        if (bad_layout(layout, LABEL)) return;                                                                   \
        char sd = sch(side), u = uch(uplo);                                                                      \
        if (layout == GbxRowMajor) {                                                                             \
            sd = flip_s(sd);                                                                                     \
            u = flip_u(u);                                                                                       \
            int tmp = m; m = n; n = tmp;                                                                         \
        }                                                                                                        \
        FN##_(&sd, &u, &m, &n, BYREF(alpha), a, &lda, b, &ldb, BYREF(beta), c, &ldc);                           \
    }
CBLAS_SYMM(ssymm, float, "SSYMM ", ADDR)
CBLAS_SYMM(dsymm, double, "DSYMM ", ADDR)
CBLAS_SYMM(csymm, const void *, "CSYMM ", PTR)
CBLAS_SYMM(zsymm, const void *, "ZSYMM ", PTR)
CBLAS_SYMM(chemm, const void *, "CHEMM ", PTR)
CBLAS_SYMM(zhemm, const void *, "ZHEMM ", PTR)

/* row-major: the stored triangle flips and N <-> T (C for Hermitian) */
#define CBLAS_RK(FN, S, LABEL, OTHER, BYREF)                                                                     \
    void cblas_##FN(int layout, int uplo, int trans, int n, int k, S alpha, const void *a, int lda, S beta,      \
                    void *c, int ldc)                                                                            \
    {                                                                                                            \
        if (bad_layout(layout, LABEL)) return;                                                                   \
        char u = uch(uplo), t = tch(trans);                                                                      \
        if (layout == GbxRowMajor) {                                                                             \
            u = flip_u(u);                                                                                       \
            t = flip_rk(t, OTHER);                                                                               \
        }                                                                                                        \
        FN##_(&u, &t, &n, &k, BYREF(alpha), a, &lda, BYREF(beta), c, &ldc);                                      \
    }
CBLAS_RK(ssyrk, float, "SSYRK ", 'T', ADDR)
CBLAS_RK(csyrk, const void *, "CSYRK ", 'T', PTR)
CBLAS_RK(zsyrk, const void *, "ZSYRK ", 'T', PTR)
CBLAS_RK(cherk, float, "CHERK ", 'C', ADDR)
CBLAS_RK(zherk, double, "ZHERK ", 'C', ADDR)

#define CBLAS_R2K(FN, S, SB, LABEL, OTHER, BYREF, BYREFB)                                                        \
    void cblas_##FN(int layout, int uplo, int trans, int n, int k, S alpha, const void *a, int lda,             \
                    const void *b, int ldb, SB beta, void *c, int ldc)                                           \
    {                                                                                                            \
        if (bad_layout(layout, LABEL)) return;                                                                   \
        char u = uch(uplo), t = tch(trans);                                                                      \
        if (layout == GbxRowMajor) {                                                                             \
            u = flip_u(u);                                                                                       \
            t = flip_rk(t, OTHER);                                                                               \
        }                                                                                                        \
        FN##_(&u, &t, &n, &k, BYREF(alpha), a, &lda, b, &ldb, BYREFB(beta), c, &ldc);                           \
    }
CBLAS_R2K(ssyr2k, float, float, "SSYR2K", 'T', ADDR, ADDR)
CBLAS_R2K(dsyr2k, double, double, "DSYR2K", 'T', ADDR, ADDR)
CBLAS_R2K(csyr2k, const void *, const void *, "CSYR2K", 'T', PTR, PTR)
CBLAS_R2K(zsyr2k, const void *, const void *, "ZSYR2K", 'T', PTR, PTR)

/* Hermitian rank-2k, row-major: conj(C) = conj(alpha) A'^H B' + alpha B'^H A'
 * with A' = A^T, B' = B^T, so the column-major call takes conj(alpha) */
#define CBLAS_HER2K(FN, R, LABEL)                                                                                \
    void cblas_##FN(int layout, int uplo, int trans, int n, int k, const void *alpha, const void *a, int lda,   \
                    const void *b, int ldb, R beta, void *c, int ldc)                                            \
    {                                                                                                            \
        if (bad_layout(layout, LABEL)) return;                                                                   \
        char u = uch(uplo), t = tch(trans);                                                                      \
        const R *al = (const R *)alpha;                                                                          \
        R alc[2] = {al[0], al[1]};                                                                               \
        if (layout == GbxRowMajor) {                                                                             \
            u = flip_u(u);                                                                                       \
            t = flip_rk(t, 'C');                                                                                 \
            alc[1] = -alc[1];                                                                                    \
        }                                                                                                        \
        FN##_(&u, &t, &n, &k, alc, a, &lda, b, &ldb, &beta, c, &ldc);                                           \
    }
CBLAS_HER2K(cher2k, float, "CHER2K")
CBLAS_HER2K(zher2k, double, "ZHER2K")

/* row-major: B^T = alpha B^T op(A)^T; side and uplo flip, m and n swap, the
 * transposition letter stays */
#define CBLAS_TR(FN, S, LABEL, BYREF)                                                                            \
    void cblas_##FN(int layout, int side, int uplo, int transa, int diag, int m, int n, S alpha, const void *a, \
                    int lda, void *b, int ldb)                                                                   \
    {                                                                                                            \
        if (bad_layout(layout, LABEL)) return;                                                                   \
        char sd = sch(side), u = uch(uplo), t = tch(transa), d = dch(diag);                                      \
        if (layout == GbxRowMajor) {                                                                             \
            sd = flip_s(sd);                                                                                     \
            u = flip_u(u);                                                                                       \
            int tmp = m; m = n; n = tmp;                                                                         \
        }                                                                                                        \
        FN##_(&sd, &u, &t, &d, &m, &n, BYREF(alpha), a, &lda, b, &ldb);                                         \
    }
CBLAS_TR(strmm, float, "STRMM ", ADDR)
CBLAS_TR(ctrmm, const void *, "CTRMM ", PTR)
CBLAS_TR(ztrmm, const void *, "ZTRMM ", PTR)
CBLAS_TR(strsm, float, "STRSM ", ADDR)
CBLAS_TR(ctrsm, const void *, "CTRSM ", PTR)
CBLAS_TR(ztrsm, const void *, "ZTRSM ", PTR)
