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
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

// Kernel timing: when enabled, the main kernel of each routine is bracketed by
// a pair of CUDA events on the context's stream; gbx_ctx_kernel_time() sums
// the elapsed times per tag after a synchronisation.
#define GBX_TIMER_PAIRS 1024
#define GBX_AUX_EVENTS 160
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
    cudaStream_t aux[3];           // copy-in, copy-out and second compute stream of the pipelined DGEMM (lazy)
    cudaEvent_t aux_ev[GBX_AUX_EVENTS];
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

// The same bracket on another stream of the context (the pipelined copies).
static void timer_begin_on(gbx_ctx *c, int tag, cudaStream_t s)
{
    if (!c || !c->timing) return;
    gbx_timer_rec *r = &c->timers[c->timer_next % GBX_TIMER_PAIRS];
    r->tag = tag;
    r->used = 1;
    c->timer_open = c->timer_next % GBX_TIMER_PAIRS;
    cudaEventRecord(r->start, s);
}

static void timer_end_on(gbx_ctx *c, cudaStream_t s)
{
    if (!c || !c->timing) return;
    cudaEventRecord(c->timers[c->timer_open].stop, s);
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
    for (int i = 0; i < 3; i++)
        if (c->aux[i]) cudaStreamDestroy(c->aux[i]);
    for (int i = 0; i < GBX_AUX_EVENTS; i++)
        if (c->aux_ev[i]) cudaEventDestroy(c->aux_ev[i]);
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

// --------------------------------------------------------------------------
// DGEMM on host operands with the copies pipelined against the products
// --------------------------------------------------------------------------
// The reference stages every operand with blocking copies before cuBLAS runs
// (gemm.cc:46-83, runtime-mem.hpp:84-155), so a large call pays all of its
// host transfers on top of the product.  Here, when op(A), op(B) and C all
// live in host memory and C is large, C is cut into R x P blocks, each still
// at least two 128 x 128 tiles per SM: the copy-in stream brings row block r
// of op(A), column panel c of op(B) and block C(r, c) (when beta != 0), the
// context's stream and a second compute stream take the blocks in turn, each
// as soon as its operands are in (two streams, so that the last wave of one
// block's tiles overlaps the next block instead of leaving SMs idle), and
// the copy-out stream returns each finished block.  Only the first block's
// operands and the last block's result are exposed.  Every output element
// is one FMA chain over K in the same order as in the undivided product, so
// the result is bit-identical to it.
static gbx_status aux_ready(gbx_ctx *c)
{
    for (int i = 0; i < 3; i++)
        if (!c->aux[i] && cudaStreamCreateWithFlags(&c->aux[i], cudaStreamNonBlocking) != cudaSuccess) {
            c->aux[i] = nullptr;
            cudaGetLastError();
            return gbx_fail(c, GBX_ERR_CUDA, "copy streams");
        }
    for (int i = 0; i < GBX_AUX_EVENTS; i++)
        if (!c->aux_ev[i] && cudaEventCreateWithFlags(&c->aux_ev[i], cudaEventDisableTiming) != cudaSuccess) {
            c->aux_ev[i] = nullptr;
            cudaGetLastError();
            return gbx_fail(c, GBX_ERR_CUDA, "copy events");
        }
    return GBX_OK;
}

// Block grid for an m x n product: row blocks of op(A) of >= 2048 rows (at
// most 8) and column panels of >= 1024 columns (at most 8), reduced until
// every block holds at least 128 * 128^2 outputs (512 of the 64 x 64 FP64
// tiles, more than two per SM).  Small first blocks keep
// the exposed copy-in short (the host link runs at a few tens of GB/s on
// some boxes); the two compute streams keep the SMs busy across blocks.
// Returns 0 when the call is too small to split.
static int pipeline_plan(int m, int n, int sms, int *rb, int *cb)
{
    (void)sms;
    int R = std::max(1, std::min(8, m / 2048)), P = std::max(1, std::min(8, n / 1024));
    while (R * P > 1) {
        const int r = ((m + R - 1) / R + 127) / 128 * 128, q = ((n + P - 1) / P + 127) / 128 * 128;
        if ((long long)(r / 128) * (q / 128) >= 128) {
            *rb = r;
            *cb = q;
            return 1;
        }
        if (P >= R) P--;
        else R--;
    }
    return 0;
}

extern "C" int gbx_dgemm_pipeline_eligible(gbx_ctx *c, int m, int n, int k, const void *A, const void *B,
                                           const void *C)
{
    int managed, rb, cb;
    if (!c || m <= 0 || n <= 0 || k <= 0) return 0;
    if (!pipeline_plan(m, n, gbx_ctx_sms(c), &rb, &cb)) return 0;
    return !resident_kind(c, A, &managed) && !resident_kind(c, B, &managed) && !resident_kind(c, C, &managed);
}

static cudaError_t copy2d(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, size_t height,
                          cudaMemcpyKind kind, cudaStream_t s)
{
    if (width == 0 || height == 0) return cudaSuccess;
    return cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, height, kind, s);
}

extern "C" gbx_status gbx_dgemm_host_pipelined(gbx_ctx *c, char ta, char tb, int m, int n, int k, double alpha,
                                               const double *A, int lda, const double *B, int ldb, double beta,
                                               double *C, int ldc)
{
    int rb, cb;
    if (!pipeline_plan(m, n, gbx_ctx_sms(c), &rb, &cb)) return GBX_ERR_UNSUPPORTED;
    gbx_status st = aux_ready(c);
    if (st != GBX_OK) return st;
    const bool nota = gbx_lsame(ta, 'N'), notb = gbx_lsame(tb, 'N');
    const bool cin = beta != 0.0;
    // staged copies keep the stored shape: A is (nota ? m x k : k x m), B is (notb ? k x n : n x k)
    const int ar = nota ? m : k, ac = nota ? k : m, br = notb ? k : n, bc = notb ? n : k;
    const int dla = round_ld(ar), dlb = round_ld(br), dlc = round_ld(m);
    double *dA, *dB, *dC;
    if ((st = gbx_ws(c, GBX_WS_STAGE_A, sizeof(double) * (size_t)dla * ac, (void **)&dA)) != GBX_OK) return st;
    if ((st = gbx_ws(c, GBX_WS_STAGE_B, sizeof(double) * (size_t)dlb * bc, (void **)&dB)) != GBX_OK) return st;
    if ((st = gbx_ws(c, GBX_WS_STAGE_C, sizeof(double) * (size_t)dlc * n, (void **)&dC)) != GBX_OK) return st;
    const int R = (m + rb - 1) / rb, P = (n + cb - 1) / cb;
    if (R + P + 2 * R * P + 1 > GBX_AUX_EVENTS) return GBX_ERR_UNSUPPORTED;
    cudaEvent_t *evA = c->aux_ev, *evB = evA + R, *evC = evB + P, *evK = evC + R * P, evJoin = evK[R * P];
    cudaStream_t cin_s = c->aux[0], cout_s = c->aux[1], ks0 = c->stream, ks1 = c->aux[2];
    const size_t e8 = sizeof(double);
    cudaError_t e = cudaSuccess;
    uint64_t h2d = 0, d2h = 0;
    g_misses += 3;
    // the copy-in stream must not start before earlier work on the context's
    // stream (which may still read these staging buffers) is done
    e = cudaEventRecord(evK[0], ks0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(cin_s, evK[0], 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(cout_s, evK[0], 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ks1, evK[0], 0);
    for (int r = 0; r < R && e == cudaSuccess; r++) {
        const int r0 = r * rb, rn = std::min(rb, m - r0);
        // row block r of op(A): rows r0.. of A (nota) or columns r0.. of A
        timer_begin_on(c, GBX_TIMER_H2D, cin_s);
        if (nota)
            e = copy2d(dA + r0, dla * e8, A + r0, (size_t)lda * e8, rn * e8, (size_t)k, cudaMemcpyHostToDevice, cin_s);
        else
            e = copy2d(dA + (size_t)r0 * dla, dla * e8, A + (size_t)r0 * lda, (size_t)lda * e8, (size_t)k * e8,
                       (size_t)rn, cudaMemcpyHostToDevice, cin_s);
        timer_end_on(c, cin_s);
        h2d += (uint64_t)rn * k * e8;
        if (e == cudaSuccess) e = cudaEventRecord(evA[r], cin_s);
        for (int q = 0; q < P && e == cudaSuccess; q++) {
            const int c0 = q * cb, cn = std::min(cb, n - c0);
            if (r == 0) {
                // column panel q of op(B): columns c0.. of B (notb) or rows c0.. of B
                timer_begin_on(c, GBX_TIMER_H2D, cin_s);
                if (notb)
                    e = copy2d(dB + (size_t)c0 * dlb, dlb * e8, B + (size_t)c0 * ldb, (size_t)ldb * e8, (size_t)k * e8,
                               (size_t)cn, cudaMemcpyHostToDevice, cin_s);
                else
                    e = copy2d(dB + c0, dlb * e8, B + c0, (size_t)ldb * e8, cn * e8, (size_t)k, cudaMemcpyHostToDevice,
                               cin_s);
                timer_end_on(c, cin_s);
                h2d += (uint64_t)cn * k * e8;
                if (e == cudaSuccess) e = cudaEventRecord(evB[q], cin_s);
            }
            if (cin && e == cudaSuccess) {
                timer_begin_on(c, GBX_TIMER_H2D, cin_s);
                e = copy2d(dC + (size_t)c0 * dlc + r0, dlc * e8, C + (size_t)c0 * ldc + r0, (size_t)ldc * e8, rn * e8,
                           (size_t)cn, cudaMemcpyHostToDevice, cin_s);
                timer_end_on(c, cin_s);
                h2d += (uint64_t)rn * cn * e8;
                if (e == cudaSuccess) e = cudaEventRecord(evC[r * P + q], cin_s);
            }
            if (e != cudaSuccess) break;
            // the block's product on one of the two compute streams, once its operands are in
            const cudaStream_t ks = ((r * P + q) & 1) ? ks1 : ks0;
            e = cudaStreamWaitEvent(ks, evA[r], 0);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(ks, evB[q], 0);
            if (e == cudaSuccess && cin) e = cudaStreamWaitEvent(ks, evC[r * P + q], 0);
            if (e != cudaSuccess) break;
            const double *ab = nota ? dA + r0 : dA + (size_t)r0 * dla;
            const double *bb = notb ? dB + (size_t)c0 * dlb : dB + c0;
            c->stream = ks;
            st = gbx_dgemm(c, ta, tb, rn, cn, k, alpha, ab, dla, bb, dlb, beta, dC + (size_t)c0 * dlc + r0, dlc);
            c->stream = ks0;
            if (st != GBX_OK) return st;
            e = cudaEventRecord(evK[r * P + q], ks);
        }
    }
    // results back, block by block, as each product finishes
    for (int r = 0; r < R && e == cudaSuccess; r++)
        for (int q = 0; q < P && e == cudaSuccess; q++) {
            const int r0 = r * rb, rn = std::min(rb, m - r0), c0 = q * cb, cn = std::min(cb, n - c0);
            e = cudaStreamWaitEvent(cout_s, evK[r * P + q], 0);
            timer_begin_on(c, GBX_TIMER_D2H, cout_s);
            if (e == cudaSuccess)
                e = copy2d(C + (size_t)c0 * ldc + r0, (size_t)ldc * e8, dC + (size_t)c0 * dlc + r0, dlc * e8, rn * e8,
                           (size_t)cn, cudaMemcpyDeviceToHost, cout_s);
            timer_end_on(c, cout_s);
            d2h += (uint64_t)rn * cn * e8;
        }
    // the context's stream orders after the second compute stream's blocks
    if (e == cudaSuccess) e = cudaEventRecord(evJoin, ks1);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ks0, evJoin, 0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cout_s);
    g_h2d += h2d;
    g_d2h += d2h;
    if (e != cudaSuccess) {
        cudaStreamSynchronize(cin_s);
        cudaStreamSynchronize(ks1);
        cudaStreamSynchronize(ks0);
        return gbx_fail(c, GBX_ERR_CUDA, "pipelined dgemm: %s", cudaGetErrorString(e));
    }
    return GBX_OK;
}
