// gbx_runtime.cu — contexts, per-thread streams, workspaces, error records and
// placement of caller operands.
//
// Replaces the reference's device runtime and staging layer:
//   * one global cuBLAS handle on the legacy stream (runtime-blas.c:14-23)
//     -> one context per host thread with its own non-blocking stream;
//   * gpuptr<T> (runtime-mem.hpp:37-165): a hit in managed memory is used in
//     place, a miss is cudaMalloc + blocking memcpy + cudaFree per call
//     -> hits are used in place (optionally prefetched), misses are staged in
//        context-owned workspace slots that persist across calls;
//   * abort() on every runtime failure (runtime.c:208-213)
//     -> a status code plus a text record on the context.
#include "gbx_internal.h"

#include <cuda_runtime.h>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

// Kernel timing: when enabled, the main kernel of each routine is bracketed by
// a pair of CUDA events on the context's stream; gbx_ctx_kernel_time() sums
// the elapsed times per tag after a synchronisation.
#define GBX_TIMER_PAIRS 256
struct gbx_timer_rec {
    cudaEvent_t start, stop;
    int tag;
    int used;
};

struct gbx_ctx {
    int device;
    int sms;
    cudaStream_t own_stream;
    cudaStream_t stream;
    void  *ws[GBX_WS_SLOTS];
    size_t ws_bytes[GBX_WS_SLOTS];
    void  *pinned;
    size_t pinned_bytes;
    uint64_t launches;
    int *status_dev;     // device status words of kernels with bounded waits ([0]; [12] a counter)
    int *status_host;    // mapped pinned mirror of status_dev[0], written by the kernels on failure
    int *status_mirror;  // the mirror's device address
    int status_armed;    // a kernel that reports through the mirror ran since the last sync
    int timing;
    int timer_next;
    int timer_open;
    gbx_timer_rec timers[GBX_TIMER_PAIRS];
    char err[512];
};

extern "C" gbx_status gbx_ctx_enable_timing(gbx_ctx *c, int on)
{
    if (!c) return GBX_ERR_ARG;
    if (on && !c->timers[0].start) {
        for (int i = 0; i < GBX_TIMER_PAIRS; i++) {
            if (cudaEventCreate(&c->timers[i].start) != cudaSuccess ||
                cudaEventCreate(&c->timers[i].stop) != cudaSuccess)
                return gbx_fail(c, GBX_ERR_CUDA, "timer events");
        }
    }
    c->timing = on;
    c->timer_next = 0;
    for (int i = 0; i < GBX_TIMER_PAIRS; i++) c->timers[i].used = 0;
    return GBX_OK;
}

extern "C" void gbx_timer_begin(gbx_ctx *c, int tag)
{
    if (!c || !c->timing) return;
    gbx_timer_rec *r = &c->timers[c->timer_next % GBX_TIMER_PAIRS];
    r->tag = tag;
    r->used = 1;
    c->timer_open = c->timer_next % GBX_TIMER_PAIRS;
    cudaEventRecord(r->start, c->stream);
}

extern "C" void gbx_timer_end(gbx_ctx *c)
{
    if (!c || !c->timing) return;
    cudaEventRecord(c->timers[c->timer_open].stop, c->stream);
    c->timer_next++;
}

extern "C" gbx_status gbx_ctx_kernel_time(gbx_ctx *c, int tag, double *ms, uint64_t *count)
{
    if (!c || !ms) return GBX_ERR_ARG;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return gbx_fail(c, GBX_ERR_CUDA, "timer sync: %s", cudaGetErrorString(e));
    double total = 0.0;
    uint64_t n = 0;
    for (int i = 0; i < GBX_TIMER_PAIRS; i++) {
        gbx_timer_rec *r = &c->timers[i];
        if (!r->used || r->tag != tag) continue;
        float t = 0.f;
        if (cudaEventElapsedTime(&t, r->start, r->stop) == cudaSuccess) {
            total += t;
            n++;
        }
    }
    *ms = total;
    if (count) *count = n;
    return GBX_OK;
}

extern "C" int gbx_lsame(char a, char b)
{
    if (a >= 'a' && a <= 'z') a = (char)(a - 32);
    if (b >= 'a' && b <= 'z') b = (char)(b - 32);
    return a == b;
}

extern "C" const char *gbx_status_string(gbx_status s)
{
    switch (s) {
    case GBX_OK: return "ok";
    case GBX_ERR_ARG: return "invalid argument";
    case GBX_ERR_CUDA: return "CUDA error";
    case GBX_ERR_ALLOC: return "allocation failed";
    case GBX_ERR_TIMEOUT: return "device wait timed out";
    case GBX_ERR_UNSUPPORTED: return "unsupported";
    case GBX_ERR_ADMISSION: return "admission rejected";
    }
    return "unknown status";
}

extern "C" gbx_status gbx_fail(gbx_ctx *ctx, gbx_status st, const char *fmt, ...)
{
    if (ctx) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(ctx->err, sizeof ctx->err, fmt, ap);
        va_end(ap);
    }
    return st;
}

// Defined only in libgbxblas_preload.so (the allocation interposer): rescans
// the mapped CUDA libraries, which are loaded when the first context is made.
extern "C" void gbx_tracker_refresh(void) __attribute__((weak));

extern "C" gbx_status gbx_ctx_create(gbx_ctx **out, int device)
{
    if (!out) return GBX_ERR_ARG;
    *out = nullptr;
    gbx_ctx *c = (gbx_ctx *)calloc(1, sizeof(gbx_ctx));
    if (!c) return GBX_ERR_ALLOC;
    c->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        free(c);
        return GBX_ERR_CUDA;
    }
    c->stream = c->own_stream;
    *out = c;
    if (gbx_tracker_refresh) gbx_tracker_refresh();
    return GBX_OK;
}

extern "C" gbx_status gbx_ctx_destroy(gbx_ctx *c)
{
    if (!c) return GBX_OK;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (int i = 0; i < GBX_WS_SLOTS; i++)
        if (c->ws[i]) cudaFree(c->ws[i]);
    if (c->pinned) cudaFreeHost(c->pinned);
    if (c->status_dev) cudaFree(c->status_dev);
    if (c->status_host) cudaFreeHost(c->status_host);
    for (int i = 0; i < GBX_TIMER_PAIRS; i++) {
        if (c->timers[i].start) cudaEventDestroy(c->timers[i].start);
        if (c->timers[i].stop) cudaEventDestroy(c->timers[i].stop);
    }
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    free(c);
    return GBX_OK;
}

namespace {
// Destroys the calling thread's context when the thread exits.  At process
// exit the CUDA runtime may already be shut down; the calls then fail
// harmlessly, so they are not checked.
struct ThreadCtx {
    gbx_ctx *ctx = nullptr;
    ~ThreadCtx() { if (ctx) gbx_ctx_destroy(ctx); }
};
thread_local ThreadCtx t_ctx;
}

extern "C" gbx_ctx *gbx_thread_ctx(void)
{
    if (!t_ctx.ctx) {
        int dev = 0;
        const char *d = getenv("GBX_DEVICE");
        if (d) dev = atoi(d);
        if (gbx_ctx_create(&t_ctx.ctx, dev) != GBX_OK) t_ctx.ctx = nullptr;
    } else {
        cudaSetDevice(t_ctx.ctx->device);
    }
    return t_ctx.ctx;
}

extern "C" gbx_status gbx_ctx_set_stream(gbx_ctx *c, void *stream)
{
    if (!c) return GBX_ERR_ARG;
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    return GBX_OK;
}

extern "C" void *gbx_ctx_get_stream(gbx_ctx *c) { return c ? (void *)c->stream : nullptr; }

// Kernels with bounded device-side waits share one status word per context
// (zero while nothing failed; first error wins) and copy it, when it is
// nonzero, into a mapped pinned mirror as they finish.  A sync reads the
// mirror: no copy or reset is queued per call, only after a failure.
extern "C" gbx_status gbx_ctx_status(gbx_ctx *c, int **dev_status, int **host_mirror)
{
    if (!c) return GBX_ERR_ARG;
    if (!c->status_dev) {
        if (cudaMalloc((void **)&c->status_dev, 64) != cudaSuccess)
            return gbx_fail(c, GBX_ERR_ALLOC, "status word");
        if (cudaMemset(c->status_dev, 0, 64) != cudaSuccess ||
            cudaHostAlloc((void **)&c->status_host, sizeof(int), cudaHostAllocMapped) != cudaSuccess ||
            cudaHostGetDevicePointer((void **)&c->status_mirror, c->status_host, 0) != cudaSuccess) {
            cudaGetLastError();
            if (c->status_host) cudaFreeHost(c->status_host);
            cudaFree(c->status_dev);
            c->status_dev = nullptr;
            c->status_host = nullptr;
            return gbx_fail(c, GBX_ERR_ALLOC, "status mirror");
        }
        *(volatile int *)c->status_host = 0;
    }
    c->status_armed = 1;
    *dev_status = c->status_dev;
    *host_mirror = c->status_mirror;
    return GBX_OK;
}

extern "C" gbx_status gbx_ctx_sync(gbx_ctx *c)
{
    if (!c) return GBX_ERR_ARG;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return gbx_fail(c, GBX_ERR_CUDA, "stream sync: %s", cudaGetErrorString(e));
    if (!c->status_armed) return GBX_OK;
    c->status_armed = 0;
    const int bad = *(volatile int *)c->status_host;
    if (!bad) return GBX_OK;
    // clear the words for the next call (the DPOTRF counter at [12] is reset
    // by the kernel that uses it, but a failed call may have left it behind)
    cudaMemsetAsync(c->status_dev, 0, 64, c->stream);
    e = cudaStreamSynchronize(c->stream);
    *(volatile int *)c->status_host = 0;
    if (e != cudaSuccess) return gbx_fail(c, GBX_ERR_CUDA, "status reset: %s", cudaGetErrorString(e));
    if (bad == 5) return gbx_fail(c, GBX_ERR_ARG, "non-finite operand: the Ozaki path needs finite inputs");
    return gbx_fail(c, GBX_ERR_TIMEOUT, "a bounded device wait gave up (code %d)", bad);
}

extern "C" uint64_t gbx_ctx_launches(const gbx_ctx *c) { return c ? c->launches : 0; }
extern "C" const char *gbx_ctx_last_error(const gbx_ctx *c) { return c ? c->err : "no context"; }
extern "C" void gbx_count_launch(gbx_ctx *c, int n) { if (c) c->launches += (uint64_t)n; }
extern "C" int gbx_ctx_device(const gbx_ctx *c) { return c ? c->device : 0; }
extern "C" int gbx_ctx_sms(const gbx_ctx *c) { return c && c->sms > 0 ? c->sms : 152; }

extern "C" gbx_status gbx_check_launch(gbx_ctx *c, const char *what)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return gbx_fail(c, GBX_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return GBX_OK;
}

// Allocation fault injection for host-side tests: GBX_FAULT_ALLOC=<n> makes
// the n-th workspace allocation (1-based) of the process report failure
// without touching the device.
static std::atomic<long> g_alloc_count{0};
static bool inject_alloc_failure()
{
    static long target = [] {
        const char *s = getenv("GBX_FAULT_ALLOC");
        return s ? atol(s) : 0L;
    }();
    if (target <= 0) return false;
    return ++g_alloc_count == target;
}

extern "C" gbx_status gbx_ws(gbx_ctx *c, int slot, size_t bytes, void **ptr)
{
    if (!c || slot < 0 || slot >= GBX_WS_SLOTS) return GBX_ERR_ARG;
    if (bytes == 0) bytes = 256;
    if (c->ws_bytes[slot] < bytes) {
        // grow geometrically so a sweep of sizes does not reallocate each call
        size_t want = bytes + bytes / 4;
        want = (want + 4095) & ~(size_t)4095;
        if (inject_alloc_failure())
            return gbx_fail(c, GBX_ERR_ALLOC, "workspace slot %d: injected allocation failure", slot);
        cudaError_t e = cudaStreamSynchronize(c->stream);
        if (c->ws[slot]) cudaFree(c->ws[slot]);
        c->ws[slot] = nullptr;
        c->ws_bytes[slot] = 0;
        if (e == cudaSuccess) e = cudaMalloc(&c->ws[slot], want);
        if (e != cudaSuccess) {
            c->ws[slot] = nullptr;
            cudaGetLastError();
            return gbx_fail(c, GBX_ERR_ALLOC, "workspace slot %d: %zu bytes: %s", slot, want,
                            cudaGetErrorString(e));
        }
        c->ws_bytes[slot] = want;
    }
    *ptr = c->ws[slot];
    return GBX_OK;
}

extern "C" gbx_status gbx_ctx_reserve(gbx_ctx *c, size_t bytes)
{
    void *p;
    return gbx_ws(c, 0, bytes, &p);
}

extern "C" gbx_status gbx_pinned(gbx_ctx *c, size_t bytes, void **ptr)
{
    if (!c) return GBX_ERR_ARG;
    if (c->pinned_bytes < bytes) {
        cudaStreamSynchronize(c->stream);
        if (c->pinned) cudaFreeHost(c->pinned);
        c->pinned = nullptr;
        c->pinned_bytes = 0;
        size_t want = bytes < 4096 ? 4096 : bytes;
        cudaError_t e = cudaMallocHost(&c->pinned, want);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return gbx_fail(c, GBX_ERR_ALLOC, "pinned %zu bytes: %s", want, cudaGetErrorString(e));
        }
        c->pinned_bytes = want;
    }
    *ptr = c->pinned;
    return GBX_OK;
}

// --------------------------------------------------------------------------
// placement
// --------------------------------------------------------------------------
static std::atomic<uint64_t> g_hits{0}, g_misses{0}, g_h2d{0}, g_d2h{0};

extern "C" void gbx_placement_counters(uint64_t *hits, uint64_t *misses, uint64_t *h2d,
                                       uint64_t *d2h)
{
    if (hits) *hits = g_hits.load();
    if (misses) *misses = g_misses.load();
    if (h2d) *h2d = g_h2d.load();
    if (d2h) *d2h = g_d2h.load();
}

// 1 = device memory of any kind the kernels can address directly without a
// copy (device or managed); 0 = host memory to be staged.
static int resident_kind(gbx_ctx *c, const void *p, int *managed)
{
    *managed = 0;
    cudaPointerAttributes a;
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) { cudaGetLastError(); return 0; }
    if (a.type == cudaMemoryTypeDevice) return 1;
    if (a.type == cudaMemoryTypeManaged) { *managed = 1; return 1; }
    (void)c;
    return 0;
}

static gbx_status prefetch_managed(gbx_ctx *c, const void *p, size_t bytes)
{
    const gbx_config *cfg = gbx_get_config();
    if (!cfg->prefetch || bytes == 0) return GBX_OK;
    cudaMemLocation loc;
    loc.type = cudaMemLocationTypeDevice;
    loc.id = c->device;
    cudaError_t e = cudaMemPrefetchAsync(p, bytes, loc, 0, c->stream);
    if (e != cudaSuccess) cudaGetLastError();  // a hint only
    return GBX_OK;
}

static int round_ld(int rows) { return rows < 1 ? 1 : ((rows + 3) & ~3); }

extern "C" gbx_status gbx_place_in(gbx_ctx *c, int slot, const void *host, int rows, int cols,
                                   int ld, size_t elem, int copy_in, gbx_operand *op)
{
    op->host = host;
    op->host_ld = ld;
    op->staged = 0;
    int managed;
    if (host && resident_kind(c, host, &managed)) {
        op->dev = (void *)host;
        op->ld = ld;
        g_hits++;
        if (managed && cols > 0) prefetch_managed(c, host, ((size_t)(cols - 1) * ld + rows) * elem);
        return GBX_OK;
    }
    g_misses++;
    int dld = round_ld(rows);
    void *d;
    gbx_status st = gbx_ws(c, slot, (size_t)dld * (cols > 0 ? cols : 1) * elem, &d);
    if (st != GBX_OK) return st;
    op->dev = d;
    op->ld = dld;
    op->staged = 1;
    if (copy_in && rows > 0 && cols > 0) {
        // one linear copy when the columns are contiguous on both sides (a
        // pitched copy of many short rows runs well below the link rate)
        gbx_timer_begin(c, GBX_TIMER_H2D);
        cudaError_t e = (dld == ld && dld == rows)
                            ? cudaMemcpyAsync(d, host, (size_t)rows * cols * elem, cudaMemcpyHostToDevice, c->stream)
                            : cudaMemcpy2DAsync(d, (size_t)dld * elem, host, (size_t)ld * elem, (size_t)rows * elem,
                                                (size_t)cols, cudaMemcpyHostToDevice, c->stream);
        gbx_timer_end(c);
        if (e != cudaSuccess)
            return gbx_fail(c, GBX_ERR_CUDA, "stage in: %s", cudaGetErrorString(e));
        g_h2d += (uint64_t)rows * cols * elem;
    }
    return GBX_OK;
}

extern "C" gbx_status gbx_place_out(gbx_ctx *c, const gbx_operand *op, int rows, int cols,
                                    size_t elem)
{
    if (!op->staged || rows <= 0 || cols <= 0) return GBX_OK;
    gbx_timer_begin(c, GBX_TIMER_D2H);
    cudaError_t e = (op->ld == op->host_ld && op->ld == rows)
                        ? cudaMemcpyAsync((void *)op->host, op->dev, (size_t)rows * cols * elem,
                                          cudaMemcpyDeviceToHost, c->stream)
                        : cudaMemcpy2DAsync((void *)op->host, (size_t)op->host_ld * elem, op->dev,
                                            (size_t)op->ld * elem, (size_t)rows * elem, (size_t)cols,
                                            cudaMemcpyDeviceToHost, c->stream);
    gbx_timer_end(c);
    if (e != cudaSuccess) return gbx_fail(c, GBX_ERR_CUDA, "stage out: %s", cudaGetErrorString(e));
    g_d2h += (uint64_t)rows * cols * elem;
    return GBX_OK;
}

static size_t vec_span(int n, int inc) { return n <= 0 ? 0 : 1 + (size_t)(n - 1) * (size_t)(inc < 0 ? -inc : inc); }

extern "C" gbx_status gbx_place_vec(gbx_ctx *c, int slot, const void *host, int n, int inc,
                                    size_t elem, int copy_in, gbx_operand *op)
{
    size_t span = vec_span(n, inc);
    op->host = host;
    op->staged = 0;
    op->ld = op->host_ld = 1;
    int managed;
    if (host && resident_kind(c, host, &managed)) {
        op->dev = (void *)host;
        g_hits++;
        if (managed) prefetch_managed(c, host, span * elem);
        return GBX_OK;
    }
    g_misses++;
    void *d;
    gbx_status st = gbx_ws(c, slot, (span ? span : 1) * elem, &d);
    if (st != GBX_OK) return st;
    op->dev = d;
    op->staged = 1;
    if (copy_in && span) {
        cudaError_t e = cudaMemcpyAsync(d, host, span * elem, cudaMemcpyHostToDevice, c->stream);
        if (e != cudaSuccess) return gbx_fail(c, GBX_ERR_CUDA, "stage vec in: %s", cudaGetErrorString(e));
        g_h2d += span * elem;
    }
    return GBX_OK;
}

extern "C" gbx_status gbx_place_vec_out(gbx_ctx *c, const gbx_operand *op, int n, int inc,
                                        size_t elem)
{
    size_t span = vec_span(n, inc);
    if (!op->staged || !span) return GBX_OK;
    cudaError_t e = cudaMemcpyAsync((void *)op->host, op->dev, span * elem, cudaMemcpyDeviceToHost,
                                    c->stream);
    if (e != cudaSuccess) return gbx_fail(c, GBX_ERR_CUDA, "stage vec out: %s", cudaGetErrorString(e));
    g_d2h += span * elem;
    return GBX_OK;
}
