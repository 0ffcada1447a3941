// utc_probe.cu — issue and completion cost of one tcgen05.mma (kind::f8f6f4,
// E4M3 x E4M3 -> FP32, M = 128, K = 32, both operands in shared memory) as a
// function of N, for the tile shapes the Ozaki kernels use.  One CTA per SM
// (120 KB of dynamic shared memory keeps a second one off), one thread issues
// COUNT MMAs back to back into accumulators that rotate every four MMAs (the
// k steps of one 128-wide k block, as in the Ozaki kernels), then commits to
// an mbarrier and waits for it (bounded: 2 s).  Reported per MMA, in SM
// cycles (clock64): the issue cost (the issuing thread's time per
// instruction) and the completion cost (issue of the first to completion of
// the last, divided by COUNT).  Operand bytes are whatever shared memory
// holds: timing only.  Standalone diagnostic, not part of the library:
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o utc_probe \
//        libgpublas_gb300/diag/utc_probe.cu && ./utc_probe
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>

#include "../csrc/tc_ptx.cuh"

using namespace gbx_tc;

#define CK(x)                                                                                   \
    do {                                                                                        \
        cudaError_t e = (x);                                                                    \
        if (e != cudaSuccess) {                                                                 \
            printf("ERR %s line %d: %s\n", #x, __LINE__, cudaGetErrorString(e));                \
            return 1;                                                                           \
        }                                                                                       \
    } while (0)

constexpr int SMEM = 120 * 1024;

__global__ void __launch_bounds__(128, 1) utc_probe(int N, int count, long long *out, int *status)
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
        const bool ok = mbar_wait(&bar, 0, status, 1);
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

int main()
{
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
    CK(cudaFuncSetAttribute(utc_probe, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM));
    long long *d_out;
    int *d_status;
    CK(cudaMalloc(&d_out, sizeof(long long) * 2 * sms));
    CK(cudaMalloc(&d_status, sizeof(int)));
    CK(cudaMemset(d_status, 0, sizeof(int)));
    long long *h = new long long[2 * sms];
    printf("%6s %6s %6s %14s %14s %18s\n", "N", "count", "CTAs", "issue cyc/MMA", "done cyc/MMA", "FP8 TFLOP/s/SM@clk");
    const int Ns[] = {16, 32, 64, 128, 256};
    const int counts[] = {4, 64, 1024};
    int clk_khz = 0;
    CK(cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, 0));
    for (int N : Ns)
        for (int count : counts)
            for (int grid : {1, sms}) {
                long long best_i = 1LL << 62, best_d = 1LL << 62;
                for (int rep = 0; rep < 3; rep++) {
                    utc_probe<<<grid, 128, SMEM>>>(N, count, d_out, d_status);
                    CK(cudaGetLastError());
                    CK(cudaDeviceSynchronize());
                    CK(cudaMemcpy(h, d_out, sizeof(long long) * 2 * grid, cudaMemcpyDeviceToHost));
                    long long wi = 0, wd = 0;
                    for (int c = 0; c < grid; c++) {
                        if (h[2 * c] < 0) { printf("wait timed out\n"); return 1; }
                        wi = h[2 * c] > wi ? h[2 * c] : wi;
                        wd = h[2 * c + 1] > wd ? h[2 * c + 1] : wd;
                    }
                    best_i = wi < best_i ? wi : best_i;
                    best_d = wd < best_d ? wd : best_d;
                }
                const double per = (double)best_d / count;
                const double tf = 2.0 * 128 * N * 32 / per * (clk_khz * 1e3) / 1e12;
                printf("%6d %6d %6d %14.1f %14.1f %18.3f\n", N, count, grid, (double)best_i / count, per, tf);
            }
    int st = 0;
    CK(cudaMemcpy(&st, d_status, sizeof(int), cudaMemcpyDeviceToHost));
    printf("status %d\n", st);
    return st;
}
