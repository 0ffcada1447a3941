/*
 * gbx_internal.h — shared between the CUDA translation units and the C host
 * layer of libgbxblas.  Not installed.
 */
#ifndef GBX_INTERNAL_H
#define GBX_INTERNAL_H

#include "../../include/gbxblas.h"
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- host-side helpers implemented in gbx_runtime.cu ---------------------- */
int  gbx_lsame(char a, char b);
/* Record an error string on the context (printf-style) and return status. */
gbx_status gbx_fail(gbx_ctx *ctx, gbx_status st, const char *fmt, ...);
/* Device workspace owned by the context: returns a pointer to >= bytes,
 * 256-byte aligned.  Slot s (0..GBX_WS_SLOTS-1) is an independent buffer;
 * growing a slot synchronises the context's stream first. */
#define GBX_WS_SLOTS 16
/* slot assignment */
#define GBX_WS_TMP0     0   /* routine temporaries (dtrmm copy, ...)        */
#define GBX_WS_TMP1     1
#define GBX_WS_TMP2     2
#define GBX_WS_STAGE_A  3   /* staging of caller operands (Fortran layer)   */
#define GBX_WS_STAGE_B  4
#define GBX_WS_STAGE_C  5
#define GBX_WS_OZ0      6   /* Ozaki slices and scales                      */
#define GBX_WS_OZ1      7
#define GBX_WS_OZ2      8
#define GBX_WS_OZ3      9
#define GBX_WS_BATCH    10  /* grouped/batched descriptors                  */
#define GBX_WS_STAGE_D  11
#define GBX_WS_TRSM_X   12  /* dtrsm_ozaki: inverse of the triangle          */
#define GBX_WS_SPARE13  13  /* unused                                      */
#define GBX_WS_GEMV     14  /* gemv partial sums                            */
#define GBX_WS_RED      15  /* reduction partials                           */
gbx_status gbx_ws(gbx_ctx *ctx, int slot, size_t bytes, void **ptr);
/* Pinned host scratch owned by the context (for small results). */
gbx_status gbx_pinned(gbx_ctx *ctx, size_t bytes, void **ptr);
void gbx_count_launch(gbx_ctx *ctx, int n);
/* Event bracket around one launch (no-op unless timing is enabled). */
void gbx_timer_begin(gbx_ctx *ctx, int tag);
void gbx_timer_end(gbx_ctx *ctx);
/* The context's status words for kernels with bounded waits (64 bytes of
 * device memory, zero while nothing failed) and the device address of their
 * mapped host mirror, which such kernels set to the status when it is
 * nonzero as they finish.  gbx_ctx_sync reports a nonzero mirror (5: a
 * non-finite Ozaki operand, GBX_ERR_ARG; else GBX_ERR_TIMEOUT) and clears
 * both.  Word 0 is the status; word 12 is the DPOTRF step's last-CTA
 * counter, which its kernel resets. */
gbx_status gbx_ctx_status(gbx_ctx *ctx, int **dev_status, int **host_mirror);
/* Check cudaGetLastError after a launch, record and map it. */
gbx_status gbx_check_launch(gbx_ctx *ctx, const char *what);
int gbx_ctx_device(const gbx_ctx *ctx);
/* SM count of the context's device (cached). */
int gbx_ctx_sms(const gbx_ctx *ctx);

/* ---- placement of host operands (gbx_placement.cu) ------------------------
 * Classifies a caller pointer: device-resident and managed memory are used in
 * place (a "hit"), anything else is staged through a workspace slot (a
 * "miss").  Counters mirror the reference's b2c_hits / b2c_misses
 * (runtime-mem.hpp:9,83,112), made atomic. */
typedef struct {
    const void *host;    /* caller's pointer                                */
    void       *dev;     /* pointer the kernel uses                         */
    int         ld;      /* leading dimension of dev (elements)             */
    int         host_ld; /* leading dimension of host (elements)            */
    int         staged;  /* 1 if dev is a staging copy                      */
} gbx_operand;
/* rows×cols block with leading dimension ld (elements of elem bytes). */
gbx_status gbx_place_in(gbx_ctx *ctx, int slot, const void *host, int rows, int cols,
                        int ld, size_t elem, int copy_in, gbx_operand *op);
/* Copy a staged operand back into the caller's memory (no-op for hits). */
gbx_status gbx_place_out(gbx_ctx *ctx, const gbx_operand *op, int rows, int cols, size_t elem);
/* Vector operand of n elements with increment inc (any sign). Staged as a
 * compact copy covering 1+(n-1)*|inc| elements. */
gbx_status gbx_place_vec(gbx_ctx *ctx, int slot, const void *host, int n, int inc,
                         size_t elem, int copy_in, gbx_operand *op);
gbx_status gbx_place_vec_out(gbx_ctx *ctx, const gbx_operand *op, int n, int inc, size_t elem);
void gbx_placement_counters(uint64_t *hits, uint64_t *misses, uint64_t *bytes_h2d,
                            uint64_t *bytes_d2h);
/* DGEMM on host operands with the copies pipelined against block products
 * (gbx_runtime.cu): eligible when op(A), op(B) and C are all host memory and
 * C splits into blocks of two 128 x 128 tiles per SM; the call returns after
 * the result is back in C (the context's stream may still be finishing). */
int gbx_dgemm_pipeline_eligible(gbx_ctx *ctx, int m, int n, int k, const void *A, const void *B, const void *C);
gbx_status gbx_dgemm_host_pipelined(gbx_ctx *ctx, char ta, char tb, int m, int n, int k, double alpha,
                                    const double *A, int lda, const double *B, int ldb, double beta,
                                    double *C, int ldc);

/* ---- library configuration (gbx_config.c) ---------------------------------- */
typedef struct {
    int    precision_ozaki;  /* precision=ozaki                                */
    double ozaki_tol;        /* precision=ozaki:<tol>                           */
    int    prefetch;         /* prefetch=on: managed operands prefetched        */
    int    abort_on_error;   /* errors=abort                                     */
    int    trace;            /* trace=<file> set                                 */
    int    heuristic;        /* 0 false, 1 true, 2 random, 3 oracle             */
    size_t managed_min;      /* managed_min=<bytes>: smaller objects stay host  */
    char   oracle_file[1024];/* heuristic=oracle:<file>                          */
    char   stats_file[1024]; /* statistics[=<file>] written at exit              */
    int    serve;            /* serve=on: Fortran calls go through the server    */
    char   trace_file[1024]; /* trace=<file>: allocation/call trace (preload)    */
} gbx_config;

/* Trace hook (defined by libgbxblas_preload.so when trace=<file> is set):
 * records one "C" line naming the tracked object that contains ptr. */
void gbx_tracker_note(const char *fun, const void *ptr) __attribute__((weak));
const gbx_config *gbx_get_config(void);

/* Forwarding hook (defined by libgbxblas_preload.so when
 * OBJTRACKER_OPTIONS=blas_libs=... names CPU BLAS libraries): the function
 * the Fortran routine `sym` is forwarded to, or NULL to run it here.
 * GBX_FORWARD(sym, (args)) returns from the calling routine after the
 * forwarded call; GBX_FORWARD_RET does the same for routines with a result.
 * The target's type is the routine's own prototype (gbxblas_f77.h). */
void *gbx_tracker_forward(const char *sym) __attribute__((weak));
#define GBX_FORWARD(sym, args)                                                  \
    do {                                                                        \
        if (gbx_tracker_forward) {                                              \
            __typeof__(&sym) fwd_ = (__typeof__(&sym))gbx_tracker_forward(#sym); \
            if (fwd_) {                                                         \
                fwd_ args;                                                      \
                return;                                                         \
            }                                                                   \
        }                                                                       \
    } while (0)
#define GBX_FORWARD_RET(sym, args)                                              \
    do {                                                                        \
        if (gbx_tracker_forward) {                                              \
            __typeof__(&sym) fwd_ = (__typeof__(&sym))gbx_tracker_forward(#sym); \
            if (fwd_) return fwd_ args;                                         \
        }                                                                       \
    } while (0)

/* The serving layer's device-side request loop (serve_loop.cu): a resident
 * kernel fed through a ring in pinned host memory.  gbx_loop_accepts tells
 * whether an operation can run there (FP64 GEMM and SYRK with m, n <= 512
 * and k <= 4096, TRSM of order <= 256 with at most 256 right-hand sides,
 * each with work to do); gbx_loop_call submits it from the calling thread and
 * waits for its completion word. */
typedef struct gbx_loop gbx_loop;
gbx_status gbx_loop_create(int device, int ctas, gbx_loop **out);
int gbx_loop_accepts(const gbx_op *op);
gbx_status gbx_loop_call(gbx_loop *l, const gbx_op *op);
uint64_t gbx_loop_launches(const gbx_loop *l);
gbx_status gbx_loop_destroy(gbx_loop *l);

/* Fortran-layer helpers (f77.c): the calling thread's context (counting
 * the call; reports when no context can be made) and the failure report
 * (prints, and aborts under errors=abort). */
gbx_ctx *gbx_f77_ctx(const char *name);
void gbx_f77_report(const char *name, gbx_ctx *ctx, gbx_status st);

/* netlib argument checks (INFO numbering); 0 when the call is valid */
enum { GBX_TR_N = 1, GBX_TR_T = 2, GBX_TR_C = 4 };   /* transposition letters a routine takes */
int gbx_check_gemm_args(char ta, char tb, int m, int n, int k, int lda, int ldb, int ldc);
// FP64 GEMM core block tile (64, 32 or 16) for an m x n output (a triangle
// when triangular) on `sms` SMs
int gbx_dgemm_tile_choice(int m, int n, int triangular, int sms);
int gbx_check_syrk_args(char uplo, char trans, int n, int k, int lda, int ldc);
int gbx_check_trxm_args(char side, char uplo, char ta, char diag, int m, int n, int lda, int ldb);
int gbx_check_rank_k_args(char uplo, char trans, int allowed, int n, int k, int lda, int ldc);
int gbx_check_rank_2k_args(char uplo, char trans, int allowed, int n, int k, int lda, int ldb, int ldc);
int gbx_check_symm_args(char side, char uplo, int m, int n, int lda, int ldb, int ldc);
int gbx_trans_ok(char trans, int allowed);
int gbx_op_tri(char uplo, char transa, char diag);

#ifdef __cplusplus
}
#endif
#endif
