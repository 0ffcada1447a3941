/*
 * gbxdiag.h — diagnostics of libgbxblas, in a library of their own
 * (libgbxdiag.so, linked against libgbxblas.so).  They measure the device
 * and drive benchmark and failure-path workloads; an application linking the
 * BLAS library needs none of them.  None has a counterpart in the reference
 * (its statistics are hit/miss counts only, blas2cuda.c:266-273).
 */
#ifndef GBXDIAG_H
#define GBXDIAG_H

#include "gbxblas.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Measured FP64 FMA throughput of the device (TFLOP/s) from a ~50 ms DFMA
 * loop on the context's stream; the denominator of the FP64 roofline. */
gbx_status gbx_diag_fp64_peak(gbx_ctx *ctx, double *tflops);

/* Throughput of the arithmetic pipes (best over 1-8 CTAs of 256 threads per
 * SM, best of three launches on the context's stream): SIMT DFMA, FP64
 * mma.sync m8n8k4, s8 mma.sync m16n8k32 (TOP/s), bf16 m16n8k16 and E4M3
 * m16n8k32 mma.sync; the same kernel's warps on DFMA only, on the FP64
 * mma.sync only, and half and half (TFLOP/s); and dependent-chain latency
 * in clock64 cycles per operation for 1, 32 and 256 threads of one CTA:
 * FP64 FMA, FP32 FMA, FP64 multiply, shared load + FP64 FMA, shuffle + FP64
 * multiply. */
typedef struct {
    double dfma_tflops, dmma_tflops, imma_tops, hmma_bf16_tflops, qmma_e4m3_tflops;
    double mix_tflops[3];
    double latency_cycles[3][5];
} gbx_pipe_rates;
gbx_status gbx_diag_pipe_rates(gbx_ctx *ctx, gbx_pipe_rates *rates);

/* Issue and completion cost of tcgen05.mma kind::f8f6f4 (E4M3 x E4M3 ->
 * FP32, M = 128, K = 32, both operands in shared memory) for a given N: one
 * thread per CTA (grid CTAs, one per SM) issues count MMAs back to back into
 * accumulators that rotate every four, commits and waits (bounded, 2 s).
 * Best of three launches of the slowest CTA, in SM cycles per MMA. */
gbx_status gbx_diag_mma_issue(gbx_ctx *ctx, int n, int count, int grid, double *issue_cycles,
                              double *done_cycles);

/* Failure-path check of the bounded device waits: launches, on the context's
 * stream, one CTA that waits on an mbarrier nothing will ever arrive on,
 * through the same bounded wait the tensor-core kernels use (2 s limit).  The
 * wait gives up, records its code in the context's status word and mirror,
 * and the kernel returns; nothing is left in flight.  The next
 * gbx_ctx_sync returns GBX_ERR_TIMEOUT and clears the status, after which
 * the context is usable again.  Returns the launch status. */
gbx_status gbx_diag_expire_wait(gbx_ctx *ctx);

/* Native driver of the serving workload: nthreads host threads, thread t
 * running the calls of a blocked right-looking Cholesky of the n[t] x n[t]
 * matrix A[t] (leading dimension lda[t], block nb[t] <= 256, lower triangle,
 * info[t] its INFO) through server (or plain per-call dispatch on one
 * context per thread when server is NULL); ozaki selects the Ozaki forms of
 * dtrsm/dsyrk/dgemm.  The threads start together; per-call latency is taken
 * on the calling thread.  Op kinds index kind_calls / kind_sum_us. */
#define GBX_TRACE_MAX_THREADS 64
#define GBX_TRACE_KINDS 16
typedef struct {
    uint64_t calls;
    double wall_s;
    double p50_us, p99_us;
    uint64_t kind_calls[GBX_TRACE_KINDS];
    double kind_sum_us[GBX_TRACE_KINDS];
    double thread_finish_s[GBX_TRACE_MAX_THREADS];
    int first_error;   /* status of the first failed call (0: none) */
} gbx_trace_stats;
gbx_status gbx_diag_cholesky_trace(gbx_server *server, int device, int nthreads, const int *n, const int *nb,
                                   double *const *A, const int *lda, int *info, int ozaki,
                                   gbx_trace_stats *out);
/* The same driver on given operation lists: thread t issues ops[t][0 ..
 * count[t]) one call at a time, through server or plain per-call dispatch. */
gbx_status gbx_diag_ops_trace(gbx_server *server, int device, int nthreads, const gbx_op *const *ops,
                              const int *count, gbx_trace_stats *out);

#ifdef __cplusplus
}
#endif
#endif
