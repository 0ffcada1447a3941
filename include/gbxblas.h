/*
 * gbxblas.h — C ABI of the GB300 BLAS offload library (libgbxblas.so).
 *
 * Two layers are exported:
 *
 *  1. The drop-in layer: the Fortran-ABI BLAS symbols (dgemm_, dtrsm_, …) and
 *     the CBLAS symbols (cblas_dgemm, …) that the reference intercepts.  They
 *     take HOST (or managed / device) pointers, validate arguments with the
 *     netlib INFO numbering, stage operands, run on the GPU and return only
 *     after the result is visible to the caller.  See gbxblas_f77.h.
 *
 *  2. The device layer declared here: gbx_* functions over DEVICE pointers,
 *     asynchronous on the context's CUDA stream, returning a status code.
 *     This is the "thin C ABI" the host code calls; it never reads host
 *     operand memory and never synchronises unless the function says so.
 *
 * Everything is column-major, in the precision the routine's letter names
 * (s: float, d: double, c: float complex, z: double complex; complex values
 * are interleaved re/im pairs, leading dimensions counted in complex
 * elements).  Integer arguments are 32-bit, as in the LP64 Fortran ABI.
 */
#ifndef GBXBLAS_H
#define GBXBLAS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    GBX_OK = 0,
    GBX_ERR_ARG = 1,         /* invalid argument (info holds the netlib position) */
    GBX_ERR_CUDA = 2,        /* a CUDA runtime call failed                        */
    GBX_ERR_ALLOC = 3,       /* device or pinned allocation failed               */
    GBX_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up               */
    GBX_ERR_UNSUPPORTED = 5, /* combination not implemented                      */
    GBX_ERR_ADMISSION = 6    /* serving: request rejected by the memory budget   */
} gbx_status;

typedef struct gbx_ctx gbx_ctx;

/* ---- contexts ------------------------------------------------------------
 * A context owns one non-blocking CUDA stream and a growable device
 * workspace.  gbx_thread_ctx() returns the calling thread's context, created
 * on first use (the Fortran layer uses it; every host thread gets its own
 * stream).  Replaces the single global cuBLAS handle of the reference
 * (runtime-blas.c:14-23).                                                      */
gbx_status gbx_ctx_create(gbx_ctx **ctx, int device);
gbx_status gbx_ctx_destroy(gbx_ctx *ctx);
gbx_ctx   *gbx_thread_ctx(void);
/* Use a caller-provided stream (cudaStream_t passed as void*); NULL restores
 * the context's own stream. */
gbx_status gbx_ctx_set_stream(gbx_ctx *ctx, void *stream);
void      *gbx_ctx_get_stream(gbx_ctx *ctx);
gbx_status gbx_ctx_sync(gbx_ctx *ctx);
/* Pre-size the workspace so later calls do not allocate (bytes). */
gbx_status gbx_ctx_reserve(gbx_ctx *ctx, size_t bytes);
/* Number of kernels this library launched on the context since creation. */
uint64_t   gbx_ctx_launches(const gbx_ctx *ctx);
/* Device-time accounting: with timing on, the main kernel of each routine is
 * bracketed by CUDA events on the context's stream (up to 256 most recent
 * launches are kept).  gbx_ctx_kernel_time synchronises the stream and
 * returns the summed milliseconds and launch count for one tag.  The
 * reference has no equivalent (its statistics are hit/miss counts only,
 * blas2cuda.c:266-273). */
enum {
    GBX_TIMER_GEMM_FP64 = 1,   /* DFMA GEMM core (dgemm/zgemm/dsyrk/dtrmm/dtrsm) */
    GBX_TIMER_OZAKI_MMA = 2,   /* tensor-core slice products                     */
    GBX_TIMER_OZAKI_SPLIT = 3, /* slicing of the FP64 operands                   */
    GBX_TIMER_LEVEL1 = 4,      /* Level-1 streaming kernels                      */
    GBX_TIMER_GEMV = 5,        /* DGEMV streaming kernel                         */
    GBX_TIMER_BATCH = 6,       /* grouped / batched kernels                      */
    GBX_TIMER_H2D = 7,         /* staging copies of host operands into the GPU   */
    GBX_TIMER_D2H = 8          /* copies of staged results back to the host      */
};
gbx_status gbx_ctx_enable_timing(gbx_ctx *ctx, int on);
gbx_status gbx_ctx_kernel_time(gbx_ctx *ctx, int tag, double *ms, uint64_t *count);
/* Last status / CUDA error text recorded on the context. */
const char *gbx_ctx_last_error(const gbx_ctx *ctx);
const char *gbx_status_string(gbx_status s);

/* ---- Level 1 (device pointers) --------------------------------------------
 * Results of reductions are written to DEVICE memory (res) so the call stays
 * asynchronous and capturable.  Negative increments follow netlib (the
 * vector is walked from its far end).                                        */
/* y := alpha*x + y                   replaces cublasDaxpy, blas_level1/axpy.cc:49 */
gbx_status gbx_daxpy(gbx_ctx *ctx, int n, double alpha, const double *x, int incx,
                     double *y, int incy);
/* res := x^T y (deterministic)       replaces cublasDdot,  blas_level1/dot.cc:46  */
gbx_status gbx_ddot(gbx_ctx *ctx, int n, const double *x, int incx,
                    const double *y, int incy, double *res);
/* res := ||x||_2 (overflow-safe)     replaces cublasDnrm2, blas_level1/nrm2.cc:39 */
gbx_status gbx_dnrm2(gbx_ctx *ctx, int n, const double *x, int incx, double *res);
/* res := first 1-based i maximising |x_i|; 0 if n<1 or incx<=0
 *                                     replaces cublasIdamax, blas_level1/amax.cc:40 */
gbx_status gbx_idamax(gbx_ctx *ctx, int n, const double *x, int incx, int *res);
/* res := first 1-based i minimising |x_i|; 0 if n<1 or incx<=0
 *                                     replaces cublasIdamin, blas_level1/amin.cc:40 */
gbx_status gbx_idamin(gbx_ctx *ctx, int n, const double *x, int incx, int *res);
/* res := x^T y without allocating anything (no reference counterpart: it is
 * an addition of this library).  For callers that cannot allocate device
 * memory when they need the reduction: code running inside a malloc/free
 * interposer (which must not re-enter the CUDA allocator), code recording a
 * CUDA graph (cudaMalloc is not allowed during stream capture), or code under
 * a fixed memory budget.  It needs no context: it runs on 'stream'
 * (cudaStream_t as void*, NULL = default stream), and its partial sums live
 * in one 32 KiB device array shared by all calls; n is limited to 2^28
 * (4096 partials of 65536 elements) and larger n returns GBX_ERR_ARG.
 * Calls that overlap on the GPU race on that array.  The first call on a
 * device looks up the array's address; make it before any stream capture.
 * The looked-up address is kept for the life of the process: after a
 * cudaDeviceReset of that device it is stale, so do not call this entry
 * point on a device that was reset. 
 * Results agree with gbx_ddot within rounding (different partition). */
gbx_status gbx_ddot_noalloc(void *stream, int n, const double *x, int incx,
                            const double *y, int incy, double *res);
/* x := alpha*x (helper used by the Level-3 paths) */
gbx_status gbx_dscal(gbx_ctx *ctx, int n, double alpha, double *x, int incx);

/* ---- Level 2 ---------------------------------------------------------------
 * y := alpha*op(A)*x + beta*y         replaces cublasDgemv, blas_level2/gemv.cc:97 */
gbx_status gbx_dgemv(gbx_ctx *ctx, char trans, int m, int n, double alpha,
                     const double *A, int lda, const double *x, int incx,
                     double beta, double *y, int incy);

/* A := alpha*x*y^T + A                replaces cublasDger, blas_level2/ger.cc:86-94 */
gbx_status gbx_dger(gbx_ctx *ctx, int m, int n, double alpha, const double *x, int incx,
                    const double *y, int incy, double *A, int lda);
/* y := alpha*A*x + beta*y, A symmetric (one stored triangle)
 *                                     replaces cublasDsymv, blas_level2/symv.cc:88-96 */
gbx_status gbx_dsymv(gbx_ctx *ctx, char uplo, int n, double alpha, const double *A, int lda,
                     const double *x, int incx, double beta, double *y, int incy);
/* x := op(A)^-1 * x, A triangular     replaces cublasDtrsv, blas_level2/trsv.cc:81-87 */
gbx_status gbx_dtrsv(gbx_ctx *ctx, char uplo, char trans, char diag, int n, const double *A, int lda,
                     double *x, int incx);

/* ---- Level 3 ---------------------------------------------------------------
 * C := alpha*op(A)*op(B) + beta*C     replaces cublasDgemm, blas_level3/gemm.cc:62-82,174
 * beta == 0 sets C (NaN/Inf in C are not propagated), as netlib does.          */
gbx_status gbx_dgemm(gbx_ctx *ctx, char transa, char transb, int m, int n, int k,
                     double alpha, const double *A, int lda, const double *B, int ldb,
                     double beta, double *C, int ldc);
/* complex: alpha/beta point to HOST (re, im) pairs
 *                                     replaces cublasZgemm, blas_level3/gemm.cc:200-216 */
gbx_status gbx_zgemm(gbx_ctx *ctx, char transa, char transb, int m, int n, int k,
                     const double *alpha, const double *A, int lda, const double *B, int ldb,
                     const double *beta, double *C, int ldc);
/* C := alpha*A*A^T + beta*C (or A^T*A), one triangle
 *                                     replaces cublasDsyrk, blas_level3/syrk.cc:43-76,175 */
gbx_status gbx_dsyrk(gbx_ctx *ctx, char uplo, char trans, int n, int k, double alpha,
                     const double *A, int lda, double beta, double *C, int ldc);
/* B := alpha*op(A)^-1*B or alpha*B*op(A)^-1
 *                                     replaces cublasDtrsm, blas_level3/trsm.cc:40-73,167 */
gbx_status gbx_dtrsm(gbx_ctx *ctx, char side, char uplo, char transa, char diag,
                     int m, int n, double alpha, const double *A, int lda,
                     double *B, int ldb);
/* B := alpha*op(A)*B or alpha*B*op(A)
 *                                     replaces cublasDtrmm, blas_level3/trmm.cc:41-80,170 */
gbx_status gbx_dtrmm(gbx_ctx *ctx, char side, char uplo, char transa, char diag,
                     int m, int n, double alpha, const double *A, int lda,
                     double *B, int ldb);

/* The other precisions and the remaining Level-3 routines, same conventions
 * (device pointers, netlib semantics, beta == 0 sets C).  Complex scalars
 * point to HOST (re, im) pairs; complex matrices are interleaved (re, im).
 * Hermitian routines take real alpha/beta where netlib does and leave the
 * diagonal of C real.  Each replaces the cuBLAS call named, reached from the
 * reference's Fortran wrapper at the line given. */
/* cublasSgemm gemm.cc:143-160; cublasCgemm gemm.cc:181-198 */
gbx_status gbx_sgemm(gbx_ctx *ctx, char transa, char transb, int m, int n, int k,
                     float alpha, const float *A, int lda, const float *B, int ldb,
                     float beta, float *C, int ldc);
gbx_status gbx_cgemm(gbx_ctx *ctx, char transa, char transb, int m, int n, int k,
                     const float *alpha, const float *A, int lda, const float *B, int ldb,
                     const float *beta, float *C, int ldc);
/* C := alpha*A*B + beta*C (side L) or alpha*B*A + beta*C (side R), A symmetric
 * with one stored triangle: cublas[SDCZ]symm symm.cc:124-200 */
gbx_status gbx_ssymm(gbx_ctx *ctx, char side, char uplo, int m, int n, float alpha,
                     const float *A, int lda, const float *B, int ldb, float beta, float *C, int ldc);
gbx_status gbx_dsymm(gbx_ctx *ctx, char side, char uplo, int m, int n, double alpha,
                     const double *A, int lda, const double *B, int ldb, double beta, double *C, int ldc);
gbx_status gbx_csymm(gbx_ctx *ctx, char side, char uplo, int m, int n, const float *alpha,
                     const float *A, int lda, const float *B, int ldb, const float *beta, float *C, int ldc);
gbx_status gbx_zsymm(gbx_ctx *ctx, char side, char uplo, int m, int n, const double *alpha,
                     const double *A, int lda, const double *B, int ldb, const double *beta, double *C,
                     int ldc);
/* A Hermitian (diagonal taken as real): cublas[CZ]hemm hemm.cc:120-154 */
gbx_status gbx_chemm(gbx_ctx *ctx, char side, char uplo, int m, int n, const float *alpha,
                     const float *A, int lda, const float *B, int ldb, const float *beta, float *C, int ldc);
gbx_status gbx_zhemm(gbx_ctx *ctx, char side, char uplo, int m, int n, const double *alpha,
                     const double *A, int lda, const double *B, int ldb, const double *beta, double *C,
                     int ldc);
/* C := alpha*op(A)*op(A)^T + beta*C, one triangle (complex: trans N or T):
 * cublas[SCZ]syrk syrk.cc:148-216 */
gbx_status gbx_ssyrk(gbx_ctx *ctx, char uplo, char trans, int n, int k, float alpha,
                     const float *A, int lda, float beta, float *C, int ldc);
gbx_status gbx_csyrk(gbx_ctx *ctx, char uplo, char trans, int n, int k, const float *alpha,
                     const float *A, int lda, const float *beta, float *C, int ldc);
gbx_status gbx_zsyrk(gbx_ctx *ctx, char uplo, char trans, int n, int k, const double *alpha,
                     const double *A, int lda, const double *beta, double *C, int ldc);
/* C := alpha*op(A)*op(A)^H + beta*C, alpha and beta real (trans N or C):
 * cublas[CZ]herk herk.cc:131-163 */
gbx_status gbx_cherk(gbx_ctx *ctx, char uplo, char trans, int n, int k, float alpha,
                     const float *A, int lda, float beta, float *C, int ldc);
gbx_status gbx_zherk(gbx_ctx *ctx, char uplo, char trans, int n, int k, double alpha,
                     const double *A, int lda, double beta, double *C, int ldc);
/* C := alpha*op(A)*op(B)^T + alpha*op(B)*op(A)^T + beta*C, one triangle:
 * cublas[SDCZ]syr2k syr2k.cc:146-218 */
gbx_status gbx_ssyr2k(gbx_ctx *ctx, char uplo, char trans, int n, int k, float alpha,
                      const float *A, int lda, const float *B, int ldb, float beta, float *C, int ldc);
gbx_status gbx_dsyr2k(gbx_ctx *ctx, char uplo, char trans, int n, int k, double alpha,
                      const double *A, int lda, const double *B, int ldb, double beta, double *C, int ldc);
gbx_status gbx_csyr2k(gbx_ctx *ctx, char uplo, char trans, int n, int k, const float *alpha,
                      const float *A, int lda, const float *B, int ldb, const float *beta, float *C,
                      int ldc);
gbx_status gbx_zsyr2k(gbx_ctx *ctx, char uplo, char trans, int n, int k, const double *alpha,
                      const double *A, int lda, const double *B, int ldb, const double *beta, double *C,
                      int ldc);
/* C := alpha*op(A)*op(B)^H + conj(alpha)*op(B)*op(A)^H + beta*C, beta real:
 * cublas[CZ]her2k her2k.cc:141-183 */
gbx_status gbx_cher2k(gbx_ctx *ctx, char uplo, char trans, int n, int k, const float *alpha,
                      const float *A, int lda, const float *B, int ldb, float beta, float *C, int ldc);
gbx_status gbx_zher2k(gbx_ctx *ctx, char uplo, char trans, int n, int k, const double *alpha,
                      const double *A, int lda, const double *B, int ldb, double beta, double *C, int ldc);
/* cublas[SCZ]trmm trmm.cc:139-215 (the reference disables trmm.cc in its
 * build, meson.build:86-87) */
gbx_status gbx_strmm(gbx_ctx *ctx, char side, char uplo, char transa, char diag, int m, int n,
                     float alpha, const float *A, int lda, float *B, int ldb);
gbx_status gbx_ctrmm(gbx_ctx *ctx, char side, char uplo, char transa, char diag, int m, int n,
                     const float *alpha, const float *A, int lda, float *B, int ldb);
gbx_status gbx_ztrmm(gbx_ctx *ctx, char side, char uplo, char transa, char diag, int m, int n,
                     const double *alpha, const double *A, int lda, double *B, int ldb);
/* cublas[SCZ]trsm trsm.cc:134-215 */
gbx_status gbx_strsm(gbx_ctx *ctx, char side, char uplo, char transa, char diag, int m, int n,
                     float alpha, const float *A, int lda, float *B, int ldb);
gbx_status gbx_ctrsm(gbx_ctx *ctx, char side, char uplo, char transa, char diag, int m, int n,
                     const float *alpha, const float *A, int lda, float *B, int ldb);
gbx_status gbx_ztrsm(gbx_ctx *ctx, char side, char uplo, char transa, char diag, int m, int n,
                     const double *alpha, const double *A, int lda, double *B, int ldb);

/* Cholesky of one small diagonal block, lower, n <= 256, in place; *info (a
 * device int) is 0 or the 1-based column of a non-positive pivot.  Not a
 * BLAS routine (no reference counterpart): the diagonal step of the blocked
 * Cholesky that drives the serving trace. */
gbx_status gbx_dpotrf_small(gbx_ctx *ctx, char uplo, int n, double *A, int lda, int *info);

/* ---- Ozaki split-precision products (opt-in; no reference counterpart) ----
 * FP64 results from exact low-precision tensor-core products of integer
 * slices, recombined in FP64.  tol is the target relative Frobenius error
 * (<= 0 picks 1e-14); the slice count is chosen per call from the operands'
 * exponent range (slices > 0 forces a count).  *slices_used may be NULL.     */
gbx_status gbx_dgemm_ozaki(gbx_ctx *ctx, char transa, char transb, int m, int n, int k,
                           double alpha, const double *A, int lda, const double *B, int ldb,
                           double beta, double *C, int ldc, double tol, int slices,
                           int *slices_used);
gbx_status gbx_zgemm_ozaki(gbx_ctx *ctx, char transa, char transb, int m, int n, int k,
                           const double *alpha, const double *A, int lda,
                           const double *B, int ldb, const double *beta, double *C, int ldc,
                           double tol, int slices, int *slices_used);
gbx_status gbx_dsyrk_ozaki(gbx_ctx *ctx, char uplo, char trans, int n, int k, double alpha,
                           const double *A, int lda, double beta, double *C, int ldc,
                           double tol, int slices, int *slices_used);
/* B := alpha*op(A)^-1*B or alpha*B*op(A)^-1 for a triangle of order <= 1024:
 * op(A)^-1 is formed in FP64 (the triangular solve against I on the DFMA
 * path), then applied to B as one Ozaki product.  Larger orders run the FP64
 * DTRSM.  Same arguments as gbx_dtrsm. */
gbx_status gbx_dtrsm_ozaki(gbx_ctx *ctx, char side, char uplo, char transa, char diag, int m, int n,
                           double alpha, const double *A, int lda, double *B, int ldb, double tol,
                           int slices, int *slices_used);

/* ---- grouped execution of many small calls (no reference counterpart) ------
 * A plan turns a list of independent DGEMM / DTRSM operations (device
 * pointers) into one persistent grouped kernel: GEMMs are tiled (tile size
 * per size bucket chosen by an autotuner that times both variants the first
 * time a bucket is seen and caches the choice in GBX_AUTOTUNE_CACHE or
 * $HOME/.cache/gbxblas/autotune.json), TRSMs of order <= 256 are solved one
 * CTA per 16 right-hand sides, and all work items are scheduled dynamically.
 * gbx_plan_launch enqueues a counter reset and the kernel (capturable);
 * gbx_plan_graph_launch records that into a CUDA graph once and replays it.
 * The operations must not overlap in their outputs. */
enum {
    GBX_OP_GEMM = 1, /* grouped kernel and serving loop                        */
    GBX_OP_TRSM = 2, /* grouped kernel and serving loop                        */
    GBX_OP_SYRK = 3, /* serving loop: uplo, transa as trans, n, k, A, beta, C   */
    GBX_OP_DOT = 4,  /* serving loop: n, x = A (incx = lda), y = B (incy = ldb),
                        result in device memory at C                           */
    GBX_OP_NRM2 = 5, /* serving loop: n, x = A (incx = lda), result at C        */
    GBX_OP_POTRF = 6,      /* serving loop: lower Cholesky of the n x n block at
                              C (ldc), n <= 256; int info at (int *)B          */
    GBX_OP_GEMM_OZAKI = 7, /* serving loop: DGEMM through the Ozaki path       */
    GBX_OP_SYRK_OZAKI = 8, /* serving loop: DSYRK through the Ozaki path       */
    GBX_OP_TRSM_OZAKI = 9  /* serving loop: DTRSM through gbx_dtrsm_ozaki      */
};
typedef struct {
    int kind;                 /* GBX_OP_GEMM or GBX_OP_TRSM                     */
    char transa, transb;      /* GEMM: op(A), op(B); TRSM: transa = op(A)       */
    char side, uplo, diag;    /* TRSM                                            */
    int m, n, k;              /* GEMM: C is m x n, K = k; TRSM: B is m x n       */
    double alpha, beta;       /* TRSM: alpha only                                */
    const double *A; int lda;
    const double *B; int ldb; /* GEMM: B (TRSM: unused)                          */
    double *C; int ldc;       /* GEMM: C; TRSM: the right-hand sides B, in/out   */
} gbx_op;
typedef struct gbx_plan gbx_plan;
gbx_status gbx_plan_create(gbx_ctx *ctx, const gbx_op *ops, int count, gbx_plan **plan);
gbx_status gbx_plan_launch(gbx_ctx *ctx, gbx_plan *plan);
gbx_status gbx_plan_graph_launch(gbx_ctx *ctx, gbx_plan *plan);
gbx_status gbx_plan_destroy(gbx_plan *plan);
gbx_status gbx_plan_info(const gbx_plan *plan, int *work_items, double *flops);
/* The same operations issued one call each through the regular routines
 * (gbx_dgemm, gbx_dtrsm, ...) on the context's stream: the per-call
 * baseline the grouped kernel is measured against. */
gbx_status gbx_ops_run(gbx_ctx *ctx, const gbx_op *ops, int count);

/* ---- serving loop (no reference counterpart: the reference serves one call
 * at a time on one cuBLAS handle, runtime-blas.c:14-23) -------------------
 * Continuous batching of calls from many host threads on device-resident
 * operands.  gbx_server_call runs a request on the calling thread, on a free
 * slot's stream with the whole GPU, unless the slots are all busy or, for a
 * small request (DGEMM with m, n <= 512 and k <= 4096, DTRSM of order
 * <= 256), other small requests are already queued; queued requests (and
 * those of gbx_server_submit) go to worker threads that take every small
 * request queued at that moment as one grouped kernel and the others one by
 * one, each batch on the stream of a free slot, so new requests overlap with
 * work already on the GPU.  A small DGEMM computes the same bits on either
 * route and a small DTRSM always runs in the grouped kernel (a group of one
 * when run inline), so results are identical served alone or in a mix.
 * With GBX_SERVE_LOOP=1 at creation, the small FP64 requests (DGEMM and
 * DSYRK with m, n <= 512 and k <= 4096; DTRSM of order <= 256 with at most
 * 256 right-hand sides) go instead to a device-side request loop: a
 * resident kernel on a quarter of the SMs that takes them from a ring in
 * pinned host memory and shares its CTAs among them tile by tile, with no
 * launch or synchronisation per call.  gbx_server_admit / gbx_server_release
 * reserve staging memory against a budget (mem_budget, or 80% of the HBM free at
 * creation when 0) and block while it is exhausted. */
typedef struct gbx_server gbx_server;
gbx_status gbx_server_create(int device, int slots, size_t mem_budget, gbx_server **srv);
gbx_status gbx_server_submit(gbx_server *srv, const gbx_op *op, uint64_t *ticket);
gbx_status gbx_server_wait(gbx_server *srv, uint64_t ticket, double *latency_us);
gbx_status gbx_server_call(gbx_server *srv, const gbx_op *op, double *latency_us);
gbx_status gbx_server_admit(gbx_server *srv, size_t bytes);
gbx_status gbx_server_release(gbx_server *srv, size_t bytes);
gbx_status gbx_server_stats(gbx_server *srv, uint64_t *completed, uint64_t *batches,
                            uint64_t *grouped_calls, double *p50_us, double *p99_us,
                            uint64_t *admission_waits);
/* The device-side request loop behind gbx_server_call: whether the server
 * has one (GBX_SERVE_LOOP=1 at creation turns it on), the calls it ran and
 * how often its resident kernel was (re)started. */
gbx_status gbx_server_loop_stats(gbx_server *srv, int *enabled, uint64_t *calls, uint64_t *launches);
gbx_status gbx_server_reset_stats(gbx_server *srv);
gbx_status gbx_server_destroy(gbx_server *srv);

#ifdef __cplusplus
}
#endif
#endif
