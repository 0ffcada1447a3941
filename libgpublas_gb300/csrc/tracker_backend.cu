// tracker_backend.cu — CUDA side of the allocation interposer: managed slabs.
//
// The interposer (tracker.c, linked only into libgbxblas_preload.so) serves
// chosen malloc/calloc/realloc requests from CUDA managed memory, as the
// reference does with one cudaMallocManaged per request plus an inline
// 8-byte size header (blas2cuda.c:127-148, runtime.c:251-260).  Here the
// managed memory comes in large slabs that the interposer sub-allocates, and
// each slab is advised to prefer the GPU and to be accessed by the host, so
// BLAS operands placed there are resident when a call arrives.
//
// GBX_TRACKER_FAKE_MANAGED=1 replaces managed memory by 256-byte aligned host
// memory: a test mode for hosts without a GPU (the interposer's logic is
// exercised, no CUDA call is made).
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>

extern "C" int gbx_tracker_fake_managed(void)
{
    static int v = -1;
    if (v < 0) {
        const char *s = getenv("GBX_TRACKER_FAKE_MANAGED");
        v = (s && s[0] == '1') ? 1 : 0;
    }
    return v;
}

// Allocate 'bytes' of managed memory (256-byte aligned); NULL on failure.
// 'host_alloc' is the interposer's pointer to the real aligned allocator,
// used in fake mode.
extern "C" void *gbx_tracker_slab_alloc(size_t bytes, int (*host_alloc)(void **, size_t, size_t))
{
    if (gbx_tracker_fake_managed()) {
        void *p = nullptr;
        return host_alloc(&p, 256, bytes) == 0 ? p : nullptr;
    }
    void *p = nullptr;
    if (cudaMallocManaged(&p, bytes, cudaMemAttachGlobal) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess) {
        cudaMemLocation gpu;
        gpu.type = cudaMemLocationTypeDevice;
        gpu.id = dev;
        cudaMemLocation host;
        host.type = cudaMemLocationTypeHost;
        host.id = 0;
        // hints only; failures are ignored
        if (cudaMemAdvise(p, bytes, cudaMemAdviseSetPreferredLocation, gpu) != cudaSuccess) cudaGetLastError();
        if (cudaMemAdvise(p, bytes, cudaMemAdviseSetAccessedBy, host) != cudaSuccess) cudaGetLastError();
    }
    return p;
}

extern "C" void gbx_tracker_slab_free(void *p, void (*host_free)(void *))
{
    if (!p) return;
    if (gbx_tracker_fake_managed()) {
        host_free(p);
        return;
    }
    if (cudaFree(p) != cudaSuccess) cudaGetLastError();
}
