// wait_probe.cu — failure-path check of the bounded device waits.
//
// The tensor-core kernels never spin without a limit: every mbarrier wait
// polls %globaltimer, gives up after 2 s, records a code in the context's
// status word (first error wins) and the kernel returns; the CTA copies a
// nonzero status into the context's mapped host mirror as it finishes, and
// gbx_ctx_sync reports it (GBX_ERR_TIMEOUT) and clears it.  A test cannot
// make a real pipeline stall without breaking the kernel, so this launch
// waits, through the same gbx_tc::mbar_wait, on an mbarrier that nothing
// arrives on: no copy or MMA is in flight when the wait gives up, and the
// context must come back usable.  This replaces the reference's abort() on
// any runtime failure (runtime.c:208-213) with a status the caller reads.
#include "gbx_internal.h"
#include "gbxdiag.h"
#include "tc_ptx.cuh"

#include <cuda_runtime.h>

namespace {

__global__ void __launch_bounds__(32) expire_wait_kernel(int *status, int *status_host)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        gbx_tc::mbar_init(&bar, 1);
        gbx_tc::fence_barrier_init();
    }
    __syncwarp();
    if (threadIdx.x == 0) {
        // expected arrivals: one; arrivals made: none -- phase 0 never completes
        gbx_tc::mbar_wait(&bar, 0u, status, gbx_tc::TC_TIMEOUT_FULL);
        const int st = *(volatile int *)status;
        if (st) *(volatile int *)status_host = st;
    }
}

}  // namespace

extern "C" gbx_status gbx_diag_expire_wait(gbx_ctx *ctx)
{
    if (!ctx) return GBX_ERR_ARG;
    int *status, *mirror;
    gbx_status st = gbx_ctx_status(ctx, &status, &mirror);
    if (st != GBX_OK) return st;
    expire_wait_kernel<<<1, 32, 0, (cudaStream_t)gbx_ctx_get_stream(ctx)>>>(status, mirror);
    gbx_count_launch(ctx, 1);
    return gbx_check_launch(ctx, "expire_wait");
}
