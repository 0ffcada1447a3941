// pipes.cu — throughput of the arithmetic pipes a BLAS library can use on
// this GPU, and the latency of dependent FP64 chains.  These measurements
// decide where the kernels run: SIMT DFMA against the FP64 mma.sync path for
// the FP64 GEMM core, the integer and FP8 tensor paths for the Ozaki
// slices, and what bounds serial FP64 work (pivots, substitutions).
//
// Each throughput probe keeps 4-8 independent accumulator chains per thread,
// runs 2-8 CTAs of 256 threads per SM, and reports the best of three timed
// launches on the context's stream; the mixed probe splits one kernel's
// warps between DFMA and the FP64 mma.sync, which would beat either alone
// if the two had separate pipes.  Latencies are clock64 cycles per dependent
// operation in one CTA.
#include "gbx_internal.h"
#include "gbxdiag.h"

#include <cuda_runtime.h>
#include <stdint.h>

namespace {

__global__ void dfma_probe(double *out, int iters, double a, double b)
{
    double x[8];
#pragma unroll
    for (int j = 0; j < 8; j++) x[j] = threadIdx.x * 1e-3 + j;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 8; j++) x[j] = fma(x[j], a, b);
    }
    double s = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) s += x[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void dmma_probe(double *out, int iters)
{
    const double a = threadIdx.x * 1e-3, b = 1.0 - threadIdx.x * 1e-4;
    double c[8][2];
#pragma unroll
    for (int j = 0; j < 8; j++) { c[j][0] = j; c[j][1] = j + 1; }
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 8; j++)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                         : "+d"(c[j][0]), "+d"(c[j][1]) : "d"(a), "d"(b));
    }
    double s = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) s += c[j][0] + c[j][1];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void imma_probe(int *out, int iters)
{
    const uint32_t a0 = threadIdx.x, a1 = a0 * 3, a2 = a0 * 5, a3 = a0 * 7, b0 = a0 * 11, b1 = a0 * 13;
    int c[4][4];
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) c[j][q] = j + q;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 4; j++)
            asm volatile("mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                         "{%0,%1,%2,%3};"
                         : "+r"(c[j][0]), "+r"(c[j][1]), "+r"(c[j][2]), "+r"(c[j][3])
                         : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
    }
    int s = 0;
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) s += c[j][q];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// bf16 (type 0) or E4M3 (type 1) mma.sync with FP32 accumulation
template <int TYPE>
__global__ void fmma_probe(float *out, int iters)
{
    const uint32_t av = TYPE == 0 ? 0x3f803f80u : 0x38383838u, bv = TYPE == 0 ? 0x3c003c00u : 0x38383838u;
    float c[4][4];
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) c[j][q] = j + q;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if (TYPE == 0)
                asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
                             "{%8,%9}, {%0,%1,%2,%3};"
                             : "+f"(c[j][0]), "+f"(c[j][1]), "+f"(c[j][2]), "+f"(c[j][3])
                             : "r"(av), "r"(av), "r"(av), "r"(av), "r"(bv), "r"(bv));
            else
                asm volatile("mma.sync.aligned.m16n8k32.row.col.f32.e4m3.e4m3.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
                             "{%8,%9}, {%0,%1,%2,%3};"
                             : "+f"(c[j][0]), "+f"(c[j][1]), "+f"(c[j][2]), "+f"(c[j][3])
                             : "r"(av), "r"(av), "r"(av), "r"(av), "r"(bv), "r"(bv));
        }
    }
    float s = 0;
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) s += c[j][q];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// warps of one kernel on DFMA (mode 0), on the FP64 mma.sync (mode 1), or
// half and half (mode 2)
__global__ void mix_probe(double *out, int iters, int mode)
{
    const int warp = threadIdx.x >> 5;
    const bool use_mma = (mode == 1) || (mode == 2 && (warp & 1));
    double r = 0;
    if (!use_mma) {
        double x[8];
#pragma unroll
        for (int j = 0; j < 8; j++) x[j] = threadIdx.x * 1e-3 + j;
        for (int i = 0; i < iters; i++) {
#pragma unroll
            for (int j = 0; j < 8; j++) x[j] = fma(x[j], 0.999999, 1e-7);
        }
#pragma unroll
        for (int j = 0; j < 8; j++) r += x[j];
    } else {
        const double a = threadIdx.x * 1e-3, b = 1.0 - threadIdx.x * 1e-4;
        double c[8][2];
#pragma unroll
        for (int j = 0; j < 8; j++) { c[j][0] = j; c[j][1] = j + 1; }
        for (int i = 0; i < iters / 8; i++) {
#pragma unroll
            for (int j = 0; j < 8; j++)
                asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                             : "+d"(c[j][0]), "+d"(c[j][1]) : "d"(a), "d"(b));
        }
#pragma unroll
        for (int j = 0; j < 8; j++) r += c[j][0] + c[j][1];
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = r;
}

// dependent-chain latency, clock64 cycles per operation: FP64 FMA, FP32 FMA,
// FP64 multiply, shared load feeding an FP64 FMA, shuffle feeding an FP64
// multiply
__global__ void lat_probe(double *out, long long *cyc, double a, double b, int n, float af, float bf)
{
    double x = threadIdx.x * 1e-3 + 1.0;
    const long long t0 = clock64();
    for (int i = 0; i < n; i++) x = fma(x, a, b);
    const long long t1 = clock64();
    float y = threadIdx.x * 1e-3f + 1.0f;
    for (int i = 0; i < n; i++) y = fmaf(y, af, bf);
    const long long t2 = clock64();
    double z = x;
    for (int i = 0; i < n; i++) z = z * a;
    const long long t3 = clock64();
    __shared__ double sh[64];
    sh[threadIdx.x & 63] = z;
    __syncwarp();
    double w = z;
    for (int i = 0; i < n; i++) w = fma(sh[(i + threadIdx.x) & 63], w, b);
    const long long t4 = clock64();
    double v = w;
    for (int i = 0; i < n; i++) v = __shfl_sync(0xffffffffu, v, i & 31) * a;
    const long long t5 = clock64();
    out[threadIdx.x] = x + y + z + w + v;
    if (threadIdx.x == 0) {
        cyc[0] = t1 - t0; cyc[1] = t2 - t1; cyc[2] = t3 - t2; cyc[3] = t4 - t3; cyc[4] = t5 - t4;
    }
}

}  // namespace

extern "C" gbx_status gbx_diag_pipe_rates(gbx_ctx *ctx, gbx_pipe_rates *r)
{
    if (!ctx || !r) return GBX_ERR_ARG;
    const int sms = gbx_ctx_sms(ctx);
    cudaStream_t s = (cudaStream_t)gbx_ctx_get_stream(ctx);
    void *buf;
    gbx_status st = gbx_ws(ctx, GBX_WS_TMP0, sizeof(double) * (size_t)sms * 8 * 256 + 256, &buf);
    if (st != GBX_OK) return st;
    double *out = (double *)buf;
    long long *cyc = (long long *)((char *)buf + sizeof(double) * (size_t)sms * 8 * 256);
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return gbx_fail(ctx, GBX_ERR_CUDA, "pipe probe events");
    // best of three timed launches (after one untimed), in milliseconds
    auto best_ms = [&](auto launch) {
        launch();
        float best = 1e30f;
        for (int rep = 0; rep < 3; rep++) {
            cudaEventRecord(e0, s);
            launch();
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            best = ms < best ? ms : best;
        }
        return (double)best;
    };
    const int threads = 256, warps = 8;
    r->dfma_tflops = r->dmma_tflops = r->imma_tops = r->hmma_bf16_tflops = r->qmma_e4m3_tflops = 0.0;
    for (int bpsm : {2, 4, 8}) {
        const int blocks = sms * bpsm, iters = 4096;
        const double ms = best_ms([&] { dfma_probe<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-7); });
        const double tf = 2.0 * 8 * iters * (double)blocks * threads / ms / 1e9;
        if (tf > r->dfma_tflops) r->dfma_tflops = tf;
    }
    for (int bpsm : {1, 2, 4}) {
        const int blocks = sms * bpsm, iters = 2048;
        const double ms = best_ms([&] { dmma_probe<<<blocks, threads, 0, s>>>(out, iters); });
        const double tf = 512.0 * 8 * iters * (double)blocks * warps / ms / 1e9;
        if (tf > r->dmma_tflops) r->dmma_tflops = tf;
        const double ms2 = best_ms([&] { imma_probe<<<blocks, threads, 0, s>>>((int *)out, 4096); });
        const double t2 = 8192.0 * 4 * 4096 * (double)blocks * warps / ms2 / 1e9;
        if (t2 > r->imma_tops) r->imma_tops = t2;
        const double ms3 = best_ms([&] { fmma_probe<0><<<blocks, threads, 0, s>>>((float *)out, 4096); });
        const double t3 = 4096.0 * 4 * 4096 * (double)blocks * warps / ms3 / 1e9;
        if (t3 > r->hmma_bf16_tflops) r->hmma_bf16_tflops = t3;
        const double ms4 = best_ms([&] { fmma_probe<1><<<blocks, threads, 0, s>>>((float *)out, 4096); });
        const double t4 = 8192.0 * 4 * 4096 * (double)blocks * warps / ms4 / 1e9;
        if (t4 > r->qmma_e4m3_tflops) r->qmma_e4m3_tflops = t4;
    }
    for (int mode = 0; mode < 3; mode++) {
        const int blocks = sms * 4, iters = 8192;
        const double ms = best_ms([&] { mix_probe<<<blocks, threads, 0, s>>>(out, iters, mode); });
        const double nw = (double)blocks * warps;
        const double fma_fl = 8.0 * iters * 64.0, mma_fl = 8.0 * (iters / 8) * 512.0;   // per warp
        const double fl = mode == 0 ? nw * fma_fl : mode == 1 ? nw * mma_fl : nw / 2 * (fma_fl + mma_fl);
        r->mix_tflops[mode] = fl / ms / 1e9;
    }
    const int lat_threads[3] = {1, 32, 256};
    for (int i = 0; i < 3; i++) {
        lat_probe<<<1, lat_threads[i], 0, s>>>(out, cyc, 1.0000001, 1e-9, 4096, 1.0000001f, 1e-9f);
        long long h[5] = {0, 0, 0, 0, 0};
        if (cudaMemcpyAsync(h, cyc, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            break;
        for (int k = 0; k < 5; k++) r->latency_cycles[i][k] = h[k] / 4096.0;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    gbx_count_launch(ctx, 1);
    return gbx_check_launch(ctx, "pipe probes");
}
