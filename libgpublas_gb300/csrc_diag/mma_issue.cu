// mma_issue.cu — issue and completion cost of one tcgen05.mma (kind::f8f6f4,
// E4M3 x E4M3 -> FP32, M = 128, K = 32, both operands in shared memory) as a
// function of N, for the tile shapes the Ozaki kernels use.  One CTA per SM
// (120 KB of dynamic shared memory keeps a second one off); one thread
// issues `count` MMAs back to back into accumulators that rotate every four
// MMAs (the k steps of one 128-byte k block, as in the Ozaki kernels), then
// commits to an mbarrier and waits for it through the bounded wait of the
// product kernels.  Per MMA, in SM cycles (clock64): the issue cost (the
// issuing thread's time per instruction) and the completion cost (first
// issue to last completion, divided by count).  The operand bytes are
// whatever shared memory holds: the values do not matter for timing.
#include "gbx_internal.h"
#include "gbxdiag.h"
#include "tc_ptx.cuh"

#include <cuda_runtime.h>
#include <stdint.h>

using namespace gbx_tc;

namespace {

constexpr int ISSUE_SMEM = 120 * 1024;

__global__ void __launch_bounds__(128, 1) mma_issue_kernel(int N, int count, long long *out, int *status)
{
    extern __shared__ uint8_t raw[];
    uint8_t *sm = (uint8_t *)(((uintptr_t)raw + 1023) & ~(uintptr_t)1023);
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    if (warp == 0) {
        tmem_alloc(&tslot, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tslot;
    if (threadIdx.x == 0) {
        const uint32_t idesc = idesc_e4m3_f32(128, N);
        const uint32_t a = smem_u32(sm), b = smem_u32(sm + 16384);   // A 128 x 128 B, B N x 128 B
        const int nacc = 512 / N;
        const long long t0 = clock64();
        for (int i = 0; i < count; i++) {
            const int kk = i & 3;
            const uint32_t d = tbase + (uint32_t)(((i >> 2) % nacc) * N);
            mma_f8f6f4(d, smem_desc_k128(a + kk * 32), smem_desc_k128(b + kk * 32), idesc, kk ? 1u : 0u);
        }
        const long long t1 = clock64();
        mma_commit(&bar);
        const bool ok = mbar_wait(&bar, 0, status, TC_TIMEOUT_FULL);
        const long long t2 = clock64();
        out[2 * blockIdx.x] = ok ? t1 - t0 : -1;
        out[2 * blockIdx.x + 1] = ok ? t2 - t0 : -1;
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tbase, 512);
    }
}

}  // namespace

extern "C" gbx_status gbx_diag_mma_issue(gbx_ctx *ctx, int n, int count, int grid, double *issue_cycles,
                                         double *done_cycles)
{
    if (!ctx || !issue_cycles || !done_cycles) return GBX_ERR_ARG;
    if (n < 16 || n > 256 || n % 16 || count < 1 || count > (1 << 20) || grid < 1 || grid > gbx_ctx_sms(ctx))
        return gbx_fail(ctx, GBX_ERR_ARG, "mma issue probe: n in 16..256 (multiple of 16), grid <= SMs");
    cudaStream_t s = (cudaStream_t)gbx_ctx_get_stream(ctx);
    void *buf;
    gbx_status st = gbx_ws(ctx, GBX_WS_TMP0, sizeof(long long) * 2 * (size_t)grid + 256, &buf);
    if (st != GBX_OK) return st;
    long long *out = (long long *)buf;
    int *status;
    int *mirror;
    if ((st = gbx_ctx_status(ctx, &status, &mirror)) != GBX_OK) return st;
    if (cudaFuncSetAttribute(mma_issue_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, ISSUE_SMEM) !=
        cudaSuccess)
        return gbx_fail(ctx, GBX_ERR_CUDA, "mma issue probe: shared memory attribute");
    long long *h = new long long[2 * (size_t)grid];
    long long best_i = 1LL << 62, best_d = 1LL << 62;
    for (int rep = 0; rep < 3 && st == GBX_OK; rep++) {
        mma_issue_kernel<<<grid, 128, ISSUE_SMEM, s>>>(n, count, out, status);
        gbx_count_launch(ctx, 1);
        if ((st = gbx_check_launch(ctx, "mma issue probe")) != GBX_OK) break;
        if (cudaMemcpyAsync(h, out, sizeof(long long) * 2 * grid, cudaMemcpyDeviceToHost, s) != cudaSuccess) {
            st = gbx_fail(ctx, GBX_ERR_CUDA, "mma issue probe: copy");
            break;
        }
        if ((st = gbx_ctx_sync(ctx)) != GBX_OK) break;   // a wait that gave up: GBX_ERR_TIMEOUT
        long long wi = 0, wd = 0;
        for (int c = 0; c < grid; c++) {
            wi = h[2 * c] > wi ? h[2 * c] : wi;
            wd = h[2 * c + 1] > wd ? h[2 * c + 1] : wd;
        }
        best_i = wi < best_i ? wi : best_i;
        best_d = wd < best_d ? wd : best_d;
    }
    delete[] h;
    if (st != GBX_OK) return st;
    *issue_cycles = (double)best_i / count;
    *done_cycles = (double)best_d / count;
    return GBX_OK;
}
