// l1_noalloc.cu — gbx_ddot_noalloc: a dot product that allocates nothing.
//
// Some callers cannot allocate device memory at the moment they need a
// reduction: the allocation interposer of this library runs inside the
// application's malloc/free and must not re-enter the CUDA allocator; code
// that records work into a CUDA graph may not call cudaMalloc while the
// stream is being captured; a serving loop may run under a fixed memory
// budget where a surprise allocation can fail.  gbx_ddot takes its partial
// sums from the context workspace, which is allocated (and grown) on first
// use.  This variant keeps them in one fixed array in device memory instead:
//
//   * scratch: GBX_NOALLOC_PARTIALS (4096) doubles = 32 KiB, a file-scope
//     __device__ array; every GPU that loads the library holds it until the
//     process exits;
//   * partition: one partial per fixed chunk of 65536 elements, so the
//     largest accepted n is 4096 * 65536 = 2^28; larger n is rejected with
//     GBX_ERR_ARG before anything is launched;
//   * every call shares the array.  Each partial a call reads is written
//     earlier by the same call, so nothing needs clearing, but two calls
//     that overlap on the GPU (different streams, no ordering) race on the
//     array and may return wrong sums;
//   * set-up: the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current and caches it; make
//     that first call before any stream capture.  The cached address does
//     not survive a cudaDeviceReset of that device: after a reset, this entry
//     point must not be called on it.
// It calls no cudaMalloc, cudaFree or allocating library routine.
#include "gbx_internal.h"
#include "l1_kernels.cuh"

#include <cuda_runtime.h>
#include <mutex>

using namespace gbx_l1;

#define GBX_NOALLOC_PARTIALS 4096
#define GBX_NOALLOC_CHUNK 65536
#define GBX_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double g_noalloc_partials[GBX_NOALLOC_PARTIALS];

namespace {

// Host code only sees a host-side stand-in for g_noalloc_partials; the
// address a kernel may use comes from cudaGetSymbolAddress, per device.
double *g_partials_addr[GBX_NOALLOC_MAX_DEVICES];
std::mutex g_setup_mutex;

cudaError_t partials_for_current_device(double **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= GBX_NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_partials_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess) return e;
        g_partials_addr[dev] = (double *)p;
    }
    *out = g_partials_addr[dev];
    return cudaSuccess;
}

// Block b reduces elements [b*CHUNK, min(n, (b+1)*CHUNK)) of x.*y (x, y at
// element 0 of the logical vectors) into part[b].
__global__ void __launch_bounds__(L1_THREADS)
dot_chunk_partial(int n, const double *__restrict__ x, int incx, const double *__restrict__ y, int incy,
                  double *__restrict__ part)
{
    const long long c0 = (long long)blockIdx.x * GBX_NOALLOC_CHUNK;
    const long long c1 = min((long long)n, c0 + GBX_NOALLOC_CHUNK);
    double s0 = 0.0, s1 = 0.0;
    long long i = c0 + threadIdx.x;
    for (; i + L1_THREADS < c1; i += 2 * L1_THREADS) {
        s0 = fma(x[i * incx], y[i * incy], s0);
        s1 = fma(x[(i + L1_THREADS) * incx], y[(i + L1_THREADS) * incy], s1);
    }
    if (i < c1) s0 = fma(x[i * incx], y[i * incy], s0);
    const double b = block_sum(s0 + s1);
    if (threadIdx.x == 0) part[blockIdx.x] = b;
}

}  // namespace

extern "C" gbx_status gbx_ddot_noalloc(void *stream, int n, const double *x, int incx, const double *y,
                                       int incy, double *res)
{
    if (!res) return GBX_ERR_ARG;
    if ((long long)n > (long long)GBX_NOALLOC_PARTIALS * GBX_NOALLOC_CHUNK) return GBX_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    double *part = nullptr;
    if (partials_for_current_device(&part) != cudaSuccess) {
        cudaGetLastError();
        return GBX_ERR_CUDA;
    }
    if (n <= 0) {
        zero_result<<<1, 1, 0, s>>>(res);
    } else {
        const int g = (int)(((long long)n + GBX_NOALLOC_CHUNK - 1) / GBX_NOALLOC_CHUNK);
        const double *xb = incx >= 0 ? x : x + (long long)(n - 1) * (-incx);
        const double *yb = incy >= 0 ? y : y + (long long)(n - 1) * (-incy);
        dot_chunk_partial<<<g, L1_THREADS, 0, s>>>(n, xb, incx, yb, incy, part);
        sum_partials<<<1, L1_THREADS, 0, s>>>(part, g, res);
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GBX_OK : GBX_ERR_CUDA;
}
