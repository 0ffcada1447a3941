// pipes_probe.cu — throughput of the arithmetic pipes a BLAS library can use
// on this GPU: SIMT DFMA, FP64 mma.sync (m8n8k4), s8 IMMA (m16n8k32), bf16
// HMMA (m16n8k16) and E4M3 mma.sync (m16n8k32), whether DFMA and DMMA
// overlap, and the latency of dependent FP64 and FP32 chains.  Each probe keeps 4–8
// independent accumulator chains per thread over 1–8 CTAs per SM and reports
// the best of three timed launches.  It decides which pipe the FP64 GEMM core
// runs on (DFMA or DMMA) and sizes the Ozaki tensor-core path against the
// FP64 one.  Standalone diagnostic, not part of the library:
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o pipes_probe \
//        libgpublas_gb300/diag/pipes_probe.cu && ./pipes_probe
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>
#define CK(x) do{cudaError_t e=(x); if(e!=cudaSuccess){printf("ERR %s line %d: %s\n",#x,__LINE__,cudaGetErrorString(e)); return 1;}}while(0)

__global__ void dfma_probe(double* out, int iters, double a, double b) {
  double x[8];
  for (int j=0;j<8;j++) x[j] = threadIdx.x*1e-3 + j;
  for (int i=0;i<iters;i++) {
#pragma unroll
    for (int j=0;j<8;j++) x[j] = fma(x[j], a, b);
  }
  double s=0; for (int j=0;j<8;j++) s+=x[j];
  out[blockIdx.x*blockDim.x+threadIdx.x] = s;
}

__global__ void dmma_probe(double* out, int iters) {
  double a = threadIdx.x*1e-3, b = 1.0 - threadIdx.x*1e-4;
  double c[8][2];
  for (int j=0;j<8;j++){c[j][0]=j;c[j][1]=j+1;}
  for (int i=0;i<iters;i++) {
#pragma unroll
    for (int j=0;j<8;j++)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
        : "+d"(c[j][0]), "+d"(c[j][1]) : "d"(a), "d"(b));
  }
  double s=0; for (int j=0;j<8;j++) s+=c[j][0]+c[j][1];
  out[blockIdx.x*blockDim.x+threadIdx.x] = s;
}

__global__ void imma_probe(int* out, int iters) {
  uint32_t a0=threadIdx.x, a1=a0*3, a2=a0*5, a3=a0*7, b0=a0*11, b1=a0*13;
  int c[4][4];
  for (int j=0;j<4;j++) for(int q=0;q<4;q++) c[j][q]=j+q;
  for (int i=0;i<iters;i++) {
#pragma unroll
    for (int j=0;j<4;j++)
      asm volatile("mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
        : "+r"(c[j][0]), "+r"(c[j][1]), "+r"(c[j][2]), "+r"(c[j][3]) : "r"(a0),"r"(a1),"r"(a2),"r"(a3),"r"(b0),"r"(b1));
  }
  int s=0; for (int j=0;j<4;j++) for(int q=0;q<4;q++) s+=c[j][q];
  out[blockIdx.x*blockDim.x+threadIdx.x] = s;
}

__global__ void hmma_probe(float* out, int iters) {
  uint32_t a0=0x3f803f80u, a1=a0, a2=a0, a3=a0, b0=0x3c003c00u, b1=b0;
  float c[4][4];
  for (int j=0;j<4;j++) for(int q=0;q<4;q++) c[j][q]=j+q;
  for (int i=0;i<iters;i++) {
#pragma unroll
    for (int j=0;j<4;j++)
      asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[j][0]), "+f"(c[j][1]), "+f"(c[j][2]), "+f"(c[j][3]) : "r"(a0),"r"(a1),"r"(a2),"r"(a3),"r"(b0),"r"(b1));
  }
  float s=0; for (int j=0;j<4;j++) for(int q=0;q<4;q++) s+=c[j][q];
  out[blockIdx.x*blockDim.x+threadIdx.x] = s;
}

__global__ void qmma_probe(float* out, int iters) {
  uint32_t a0=0x38383838u, a1=a0, a2=a0, a3=a0, b0=a0, b1=a0;
  float c[4][4];
  for (int j=0;j<4;j++) for(int q=0;q<4;q++) c[j][q]=j+q;
  for (int i=0;i<iters;i++) {
#pragma unroll
    for (int j=0;j<4;j++)
      asm volatile("mma.sync.aligned.m16n8k32.row.col.f32.e4m3.e4m3.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[j][0]), "+f"(c[j][1]), "+f"(c[j][2]), "+f"(c[j][3]) : "r"(a0),"r"(a1),"r"(a2),"r"(a3),"r"(b0),"r"(b1));
  }
  float s=0; for (int j=0;j<4;j++) for(int q=0;q<4;q++) s+=c[j][q];
  out[blockIdx.x*blockDim.x+threadIdx.x] = s;
}

// Warps of one kernel split between SIMT DFMA and DMMA (mode 2): if the two
// ran on separate pipes the split would beat either alone.
__global__ void mix_probe(double* out, int iters, int mode) {
  const int warp = threadIdx.x >> 5;
  bool use_mma = (mode == 1) || (mode == 2 && (warp & 1));
  double r = 0;
  if (!use_mma) {
    double x[8]; for (int j=0;j<8;j++) x[j] = threadIdx.x*1e-3 + j;
    for (int i=0;i<iters;i++) {
#pragma unroll
      for (int j=0;j<8;j++) x[j] = fma(x[j], 0.999999, 1e-7);
    }
    for (int j=0;j<8;j++) r += x[j];
  } else {
    double a = threadIdx.x*1e-3, b = 1.0 - threadIdx.x*1e-4;
    double c[8][2]; for (int j=0;j<8;j++){c[j][0]=j;c[j][1]=j+1;}
    // 8 MMAs (512 flop each per warp) vs 8 FMAs (2 flop x 32 lanes = 64 per warp): scale iters
    for (int i=0;i<iters/8;i++) {
#pragma unroll
      for (int j=0;j<8;j++)
        asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
          : "+d"(c[j][0]), "+d"(c[j][1]) : "d"(a), "d"(b));
    }
    for (int j=0;j<8;j++) r += c[j][0]+c[j][1];
  }
  out[blockIdx.x*blockDim.x+threadIdx.x] = r;
}
template <typename F>
float timeit(F f) {
  cudaEvent_t e0,e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  f(); cudaDeviceSynchronize();
  float best=1e30f;
  for (int r=0;r<3;r++){
    cudaEventRecord(e0); f(); cudaEventRecord(e1); cudaEventSynchronize(e1);
    float ms; cudaEventElapsedTime(&ms,e0,e1); if(ms<best)best=ms;
  }
  return best;
}

// Latency of dependent chains (clock64 cycles per operation, one CTA): FP64
// FMA and multiply, FP32 FMA, and the shared-memory and shuffle hops of a
// substitution step, with 1, 32 and 256 threads (8 warps share the SM's FP64
// pipe).  Serial FP64 work -- pivots, substitutions -- is bound by these.
__global__ void lat_probe(double* out, long long* cyc, double a, double b, int n, float af, float bf) {
  double x = threadIdx.x * 1e-3 + 1.0;
  long long t0 = clock64();
  for (int i = 0; i < n; i++) x = fma(x, a, b);
  long long t1 = clock64();
  float y = threadIdx.x * 1e-3f + 1.0f;
  for (int i = 0; i < n; i++) y = fmaf(y, af, bf);
  long long t2 = clock64();
  double z = x;
  for (int i = 0; i < n; i++) z = z * a;
  long long t3 = clock64();
  __shared__ double sh[64];
  sh[threadIdx.x & 63] = z;
  __syncwarp();
  double w = z;
  for (int i = 0; i < n; i++) w = fma(sh[(i + threadIdx.x) & 63], w, b);
  long long t4 = clock64();
  double v = w;
  for (int i = 0; i < n; i++) v = __shfl_sync(0xffffffffu, v, i & 31) * a;
  long long t5 = clock64();
  out[threadIdx.x] = x + y + z + w + v;
  if (threadIdx.x == 0) { cyc[0] = t1 - t0; cyc[1] = t2 - t1; cyc[2] = t3 - t2; cyc[3] = t4 - t3; cyc[4] = t5 - t4; }
}

int main() {
  cudaDeviceProp p; CK(cudaGetDeviceProperties(&p,0));
  printf("device %s sms %d cc %d.%d\n", p.name, p.multiProcessorCount, p.major, p.minor);
  int sms = p.multiProcessorCount;
  size_t maxthreads = (size_t)sms*32*1024;
  double* dout; CK(cudaMalloc(&dout, maxthreads*8));
  for (int bpsm : {2, 4, 8}) {
    int blocks = sms*bpsm, threads=256, iters=4096;
    float ms = timeit([&]{ dfma_probe<<<blocks,threads>>>(dout, iters, 0.999999, 1e-7); });
    CK(cudaGetLastError());
    double fl = 2.0*8*iters*(double)blocks*threads;
    printf("DFMA   bpsm=%d: %.3f ms  %.3f TFLOP/s\n", bpsm, ms, fl/ms/1e9);
  }
  for (int bpsm : {1, 2, 4}) {
    int blocks = sms*bpsm, threads=256, iters=2048;
    float ms = timeit([&]{ dmma_probe<<<blocks,threads>>>(dout, iters); });
    CK(cudaGetLastError());
    double fl = 512.0*8*iters*(double)blocks*(threads/32);
    printf("DMMA   bpsm=%d: %.3f ms  %.3f TFLOP/s\n", bpsm, ms, fl/ms/1e9);
  }
  for (int bpsm : {1, 2, 4}) {
    int blocks = sms*bpsm, threads=256, iters=4096;
    float ms = timeit([&]{ imma_probe<<<blocks,threads>>>((int*)dout, iters); });
    CK(cudaGetLastError());
    double fl = 8192.0*4*iters*(double)blocks*(threads/32);
    printf("IMMA   bpsm=%d: %.3f ms  %.3f TOP/s\n", bpsm, ms, fl/ms/1e9);
  }
  for (int bpsm : {1, 2, 4}) {
    int blocks = sms*bpsm, threads=256, iters=4096;
    float ms = timeit([&]{ hmma_probe<<<blocks,threads>>>((float*)dout, iters); });
    CK(cudaGetLastError());
    double fl = 4096.0*4*iters*(double)blocks*(threads/32);
    printf("HMMAbf16 bpsm=%d: %.3f ms  %.3f TFLOP/s\n", bpsm, ms, fl/ms/1e9);
  }
  for (int bpsm : {1, 2, 4}) {
    int blocks = sms*bpsm, threads=256, iters=4096;
    float ms = timeit([&]{ qmma_probe<<<blocks,threads>>>((float*)dout, iters); });
    CK(cudaGetLastError());
    double fl = 8192.0*4*iters*(double)blocks*(threads/32);
    printf("QMMAe4m3 bpsm=%d: %.3f ms  %.3f TFLOP/s\n", bpsm, ms, fl/ms/1e9);
  }
  for (int mode = 0; mode < 3; mode++) {
    const int blocks = sms * 4, threads = 256, iters = 8192;
    float ms = timeit([&]{ mix_probe<<<blocks,threads>>>(dout, iters, mode); });
    CK(cudaGetLastError());
    const double warps = blocks * threads / 32.0;
    const double fma_fl = 8.0 * iters * 64.0, mma_fl = 8.0 * (iters / 8) * 512.0;   // per warp
    const double fl = mode == 0 ? warps * fma_fl : mode == 1 ? warps * mma_fl : warps / 2 * (fma_fl + mma_fl);
    printf("mix %d (%s): %.3f ms  %.3f TFLOP/s\n", mode, mode == 0 ? "DFMA" : mode == 1 ? "DMMA" : "half/half", ms,
           fl / ms / 1e9);
  }
  {
    long long* dcyc; CK(cudaMalloc(&dcyc, 64));
    for (int threads : {1, 32, 256}) {
      lat_probe<<<1, threads>>>(dout, dcyc, 1.0000001, 1e-9, 4096, 1.0000001f, 1e-9f);
      CK(cudaGetLastError());
      CK(cudaDeviceSynchronize());
      long long h[5]; CK(cudaMemcpy(h, dcyc, sizeof(h), cudaMemcpyDeviceToHost));
      printf("latency threads=%d: DFMA %.1f  FFMA %.1f  DMUL %.1f  LDS+DFMA %.1f  SHFL+DMUL %.1f cycles\n", threads,
             h[0] / 4096.0, h[1] / 4096.0, h[2] / 4096.0, h[3] / 4096.0, h[4] / 4096.0);
    }
    CK(cudaFree(dcyc));
  }
  CK(cudaDeviceSynchronize());
  return 0;
}
