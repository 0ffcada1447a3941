// fp64_peak.cu — device capability measurement used as the FP64 roofline
// denominator: sustained DFMA throughput of the whole GPU.
//
// Each thread runs 8 independent FMA chains (enough to cover the DFMA
// latency), 8 blocks of 256 threads per SM; the result is written so the
// chains cannot be eliminated.
#include "gbx_internal.h"
#include "gbxdiag.h"

#include <cuda_runtime.h>

namespace {

__global__ void __launch_bounds__(256)
dfma_rate_kernel(double *out, int iters, double a, double b)
{
    double x[8];
#pragma unroll
    for (int j = 0; j < 8; j++) x[j] = threadIdx.x * 1e-3 + j;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 8; j++) x[j] = fma(x[j], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 8; j++) s += x[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" gbx_status gbx_diag_fp64_peak(gbx_ctx *ctx, double *tflops)
{
    if (!ctx || !tflops) return GBX_ERR_ARG;
    const int blocks = gbx_ctx_sms(ctx) * 8, threads = 256, iters = 8192;
    double *out;
    gbx_status st = gbx_ws(ctx, GBX_WS_TMP0, sizeof(double) * (size_t)blocks * threads, (void **)&out);
    if (st != GBX_OK) return st;
    cudaStream_t s = (cudaStream_t)gbx_ctx_get_stream(ctx);
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return gbx_fail(ctx, GBX_ERR_CUDA, "diag events");
    dfma_rate_kernel<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-7);  // warm-up
    float best = 1e30f;
    for (int r = 0; r < 3; r++) {
        cudaEventRecord(e0, s);
        dfma_rate_kernel<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-7);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    gbx_count_launch(ctx, 4);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    st = gbx_check_launch(ctx, "diag fp64");
    if (st != GBX_OK) return st;
    const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return GBX_OK;
}
