// batched.cu — grouped execution of many small, uneven DGEMM / DTRSM calls in
// one persistent kernel (no reference counterpart: the reference issues one
// cuBLAS call at a time on one handle, runtime-blas.c:14-23).
//
// A plan is built once from a list of operations:
//   * every DGEMM is cut into C tiles of 32x32 or 64x64 computed by the GEMM
//     core of the stream path (so a grouped DGEMM gives the bits of
//     gbx_dgemm; the variant is chosen per size bucket by the autotuner
//     below); every DTRSM (order <= 256) is one work item solved by one CTA;
//   * work items are ordered by decreasing cost (longest first) and handed
//     out dynamically: each CTA of a persistent grid (2 CTAs per SM) takes
//     the next item with one atomicAdd on a counter that the launch resets;
//   * the launch is a memset + one kernel, so it can be recorded in a CUDA
//     graph; gbx_plan_graph_launch records it on first use and replays it.
// Autotuner: for each bucket of GEMMs (by max(M,N)), both tile variants are
// timed on the plan's own operands (results written to scratch, beta = 0)
// the first time the bucket is seen; the choice is kept per device in
// memory and in a JSON cache file (GBX_AUTOTUNE_CACHE, default
// $HOME/.cache/gbxblas/autotune.json), so later plans skip the timing.
#include "gbx_internal.h"
#include "gemm_host.h"
#include "gemm_simt.cuh"
#include "grouped_dev.cuh"

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <algorithm>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

namespace {

using gbx_grouped::DevOp;
using gbx_grouped::trsm_item;

constexpr int BT_THREADS = 256;
constexpr int TRSM_MAX_ORDER = 256;
constexpr int TRSM_SYS = 16;      // right-hand sides solved together
constexpr int NBUCKET = 6;        // max(M,N) <= 32, 64, 128, 256, 512, larger

struct Item {
    int op;
    int variant;                  // GEMM: 0 = 32x32 tile, 1 = 64x64; TRSM: systems chunk
    int tm, tn;
};

// One tile of a DGEMM on the GEMM core (double-buffered shared-memory
// stages with register prefetch), the arithmetic of gbx_dgemm element for
// element.
__device__ __forceinline__ void core_tile(const DevOp &o, const Item &w)
{
    gbx_gemm::GemmArgs<double> g{};
    g.m = o.m; g.n = o.n; g.k = o.k;
    g.A = o.A; g.lda = o.lda; g.ta = o.ta;
    g.B = o.B; g.ldb = o.ldb; g.tb = o.tb;
    g.alpha = o.alpha; g.beta = o.beta;
    g.C = o.C; g.ldc = o.ldc;
    g.c_part = gbx_gemm::C_FULL;
    const int ts = w.variant ? 64 : 32;
    g.tiles_m = (o.m + ts - 1) / ts;
    g.tiles_n = (o.n + ts - 1) / ts;
    if (w.variant) gbx_gemm::gemm_simt_tile<double, 4, 4, 8>(g, w.tm + w.tn * g.tiles_m);
    else gbx_gemm::gemm_simt_tile<double, 2, 2, 8>(g, w.tm + w.tn * g.tiles_m);
}

__global__ void __launch_bounds__(BT_THREADS, 2)
grouped_kernel(const DevOp *__restrict__ ops, const Item *__restrict__ items, int nitems, int *counter)
{
    __shared__ __align__(16) double smem[TRSM_MAX_ORDER * TRSM_SYS];
    __shared__ int s_item;
    while (true) {
        if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= nitems) break;
        const Item w = items[it];
        const DevOp o = ops[w.op];
        if (o.kind == GBX_OP_TRSM) trsm_item<TRSM_SYS, BT_THREADS>(o, w.variant * TRSM_SYS, smem);
        else core_tile(o, w);
        __syncthreads();
    }
}

// ---------------------------------------------------------------- autotune
int bucket_of(int m, int n)
{
    const int s = std::max(m, n);
    int b = 0;
    for (int lim = 32; b < NBUCKET - 1 && s > lim; lim *= 2) b++;
    return b;
}

std::mutex g_tune_mu;
int g_tune[64][NBUCKET];          // per device: -1 unknown, else variant
bool g_tune_loaded = false;

std::string tune_path()
{
    const char *p = getenv("GBX_AUTOTUNE_CACHE");
    if (p) return p;
    const char *h = getenv("HOME");
    return std::string(h ? h : "/tmp") + "/.cache/gbxblas/autotune.json";
}

// The cache file is a small JSON object {"<device name> core tiles": [v0,
// ..., v5]} (the key names the tile code, so choices timed on an earlier one
// are timed again); it is written by this library only, so a fixed-format
// parser suffices.
void tune_load_locked(int dev, const char *devname)
{
    for (int d = 0; d < 64; d++)
        for (int b = 0; b < NBUCKET; b++) g_tune[d][b] = -1;
    g_tune_loaded = true;
    FILE *f = fopen(tune_path().c_str(), "r");
    if (!f) return;
    char buf[4096];
    size_t len = fread(buf, 1, sizeof buf - 1, f);
    fclose(f);
    buf[len] = '\0';
    std::string key = std::string("\"") + devname + " core tiles\": [";
    const char *p = strstr(buf, key.c_str());
    if (!p) return;
    p += key.size();
    for (int b = 0; b < NBUCKET; b++) {
        int v = -1;
        if (sscanf(p, "%d", &v) == 1 && (v == 0 || v == 1)) g_tune[dev][b] = v;
        p = strchr(p, b + 1 < NBUCKET ? ',' : ']');
        if (!p) break;
        p++;
    }
}

void tune_save_locked(int dev, const char *devname)
{
    std::string path = tune_path();
    std::string dir = path.substr(0, path.find_last_of('/'));
    if (!dir.empty()) {
        // create the directory chain (best effort)
        for (size_t i = 1; i <= dir.size(); i++)
            if (i == dir.size() || dir[i] == '/') {
                std::string sub = dir.substr(0, i);
                if (!sub.empty()) (void)mkdir(sub.c_str(), 0755);
            }
    }
    FILE *f = fopen(path.c_str(), "w");
    if (!f) return;
    fprintf(f, "{\"%s core tiles\": [", devname);
    for (int b = 0; b < NBUCKET; b++) fprintf(f, "%d%s", g_tune[dev][b] < 0 ? 1 : g_tune[dev][b], b + 1 < NBUCKET ? ", " : "");
    fprintf(f, "]}\n");
    fclose(f);
}

}  // namespace

struct gbx_plan {
    int device;
    DevOp *d_ops;
    Item *d_items;
    int *d_counter;
    int nitems, nops;
    double flops;
    int grid;
    cudaGraphExec_t gexec;
};

namespace {

void tile_items(const DevOp &o, int opi, int variant, std::vector<Item> &items, std::vector<double> &cost)
{
    if (o.kind == GBX_OP_TRSM) {
        const int nsys = o.left ? o.n : o.m;
        const int order = o.left ? o.m : o.n;
        for (int s = 0; s * TRSM_SYS < nsys; s++) {
            items.push_back({opi, s, 0, 0});
            cost.push_back((double)order * order * TRSM_SYS * 4.0);   // serial substitution
        }
        return;
    }
    const int ts = variant ? 64 : 32;
    const int tmn = (o.m + ts - 1) / ts, tnn = (o.n + ts - 1) / ts;
    for (int j = 0; j < tnn; j++)
        for (int i = 0; i < tmn; i++) {
            items.push_back({opi, variant, i, j});
            cost.push_back((double)ts * ts * std::max(o.k, 1));
        }
}

gbx_status upload(gbx_ctx *ctx, const std::vector<DevOp> &ops, const std::vector<int> &variant, gbx_plan *p)
{
    std::vector<Item> items;
    std::vector<double> cost;
    for (size_t i = 0; i < ops.size(); i++) tile_items(ops[i], (int)i, variant[i], items, cost);
    std::vector<int> order(items.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    std::vector<Item> sorted(items.size());
    for (size_t i = 0; i < order.size(); i++) sorted[i] = items[order[i]];
    p->nitems = (int)sorted.size();
    p->nops = (int)ops.size();
    cudaError_t e = cudaMalloc(&p->d_ops, sizeof(DevOp) * std::max<size_t>(1, ops.size()));
    if (e == cudaSuccess) e = cudaMalloc(&p->d_items, sizeof(Item) * std::max<size_t>(1, sorted.size()));
    if (e == cudaSuccess) e = cudaMalloc(&p->d_counter, sizeof(int));
    if (e != cudaSuccess) return gbx_fail(ctx, GBX_ERR_ALLOC, "plan: %s", cudaGetErrorString(e));
    cudaStream_t s = (cudaStream_t)gbx_ctx_get_stream(ctx);
    if (!ops.empty()) cudaMemcpyAsync(p->d_ops, ops.data(), sizeof(DevOp) * ops.size(), cudaMemcpyHostToDevice, s);
    if (!sorted.empty())
        cudaMemcpyAsync(p->d_items, sorted.data(), sizeof(Item) * sorted.size(), cudaMemcpyHostToDevice, s);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return gbx_fail(ctx, GBX_ERR_CUDA, "plan upload: %s", cudaGetErrorString(e));
    p->grid = gbx_ctx_sms(ctx) * 2;
    return GBX_OK;
}

gbx_status launch(gbx_ctx *ctx, gbx_plan *p)
{
    cudaStream_t s = (cudaStream_t)gbx_ctx_get_stream(ctx);
    if (p->nitems == 0) return GBX_OK;
    cudaError_t e = cudaMemsetAsync(p->d_counter, 0, sizeof(int), s);
    if (e != cudaSuccess) return gbx_fail(ctx, GBX_ERR_CUDA, "plan counter: %s", cudaGetErrorString(e));
    gbx_timer_begin(ctx, GBX_TIMER_BATCH);
    grouped_kernel<<<std::min(p->grid, p->nitems), BT_THREADS, 0, s>>>(p->d_ops, p->d_items, p->nitems,
                                                                       p->d_counter);
    gbx_timer_end(ctx);
    gbx_count_launch(ctx, 1);
    return gbx_check_launch(ctx, "grouped kernel");
}

void plan_free(gbx_plan *p)
{
    if (!p) return;
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    if (p->d_ops) cudaFree(p->d_ops);
    if (p->d_items) cudaFree(p->d_items);
    if (p->d_counter) cudaFree(p->d_counter);
    free(p);
}

// time one plan variant (median of 3 launches), ms
float time_variant(gbx_ctx *ctx, const std::vector<DevOp> &ops, int variant)
{
    gbx_plan *p = (gbx_plan *)calloc(1, sizeof(gbx_plan));
    std::vector<int> v(ops.size(), variant);
    float best = 1e30f;
    if (p && upload(ctx, ops, v, p) == GBX_OK) {
        cudaStream_t s = (cudaStream_t)gbx_ctx_get_stream(ctx);
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        launch(ctx, p);
        for (int r = 0; r < 3; r++) {
            cudaEventRecord(e0, s);
            launch(ctx, p);
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            best = std::min(best, ms);
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    plan_free(p);
    return best;
}

}  // namespace

// Validates one operation and converts it to its device form.  Returns 0 and
// sets *skip for operations with no work.  The flops of the operation are
// added to *flops.
static gbx_status to_devop(gbx_ctx *ctx, const gbx_op &o, int i, DevOp &d, bool &skip, double &flops)
{
    d = DevOp{};
    skip = false;
    d.kind = o.kind;
    d.m = o.m; d.n = o.n; d.k = o.k;
    d.alpha = o.alpha; d.beta = o.beta;
    d.A = o.A; d.lda = o.lda; d.B = o.B; d.ldb = o.ldb; d.C = o.C; d.ldc = o.ldc;
    if (o.kind == GBX_OP_GEMM) {
        int info = gbx_check_gemm_args(o.transa, o.transb, o.m, o.n, o.k, o.lda, o.ldb, o.ldc);
        if (info) return gbx_fail(ctx, GBX_ERR_ARG, "op %d: DGEMM parameter %d", i, info);
        d.ta = !gbx_lsame(o.transa, 'N');
        d.tb = !gbx_lsame(o.transb, 'N');
        if (o.m == 0 || o.n == 0) { skip = true; return GBX_OK; }
        if (o.k == 0 || o.alpha == 0.0) d.k = 0;   // tiles then scale C by beta
        flops += 2.0 * o.m * o.n * o.k;
        return GBX_OK;
    }
    if (o.kind == GBX_OP_TRSM) {
        int info = gbx_check_trxm_args(o.side, o.uplo, o.transa, o.diag, o.m, o.n, o.lda, o.ldc);
        if (info) return gbx_fail(ctx, GBX_ERR_ARG, "op %d: DTRSM parameter %d", i, info);
        d.left = gbx_lsame(o.side, 'L');
        const int order = d.left ? o.m : o.n;
        if (order > TRSM_MAX_ORDER)
            return gbx_fail(ctx, GBX_ERR_UNSUPPORTED, "op %d: triangle order %d > %d", i, order, TRSM_MAX_ORDER);
        d.ta = !gbx_lsame(o.transa, 'N');
        // effective triangle of the matrix T solved against (op(A) for side
        // L, op(A)^T for side R)
        const bool op_lower = (gbx_op_tri(o.uplo, o.transa, o.diag) & 1) != 0;
        d.lower = d.left ? op_lower : !op_lower;
        d.unit = gbx_lsame(o.diag, 'U');
        if (o.m == 0 || o.n == 0) { skip = true; return GBX_OK; }
        flops += (double)order * order * (d.left ? o.n : o.m);
        return GBX_OK;
    }
    return gbx_fail(ctx, GBX_ERR_ARG, "op %d: kind %d is not a grouped operation", i, o.kind);
}

// Grouped launch without a plan: descriptors are packed into the context's
// pinned buffer and copied to its workspace on its stream, then the counter
// is reset and the kernel launched; nothing synchronises.  Used by the
// serving loop.  The pinned buffer is reused by the next call on the same
// context, which must therefore come after this one completed (the serving
// loop hands a context out again only after its work finished).
extern "C" gbx_status gbx_grouped_launch_inline(gbx_ctx *ctx, const gbx_op *ops, int count)
{
    std::vector<DevOp> dops;
    dops.reserve(count);
    double flops = 0.0;
    for (int i = 0; i < count; i++) {
        DevOp d;
        bool skip;
        gbx_status st = to_devop(ctx, ops[i], i, d, skip, flops);
        if (st != GBX_OK) return st;
        if (!skip) dops.push_back(d);
    }
    if (dops.empty()) return GBX_OK;
    const int dev = gbx_ctx_device(ctx);
    std::vector<Item> items;
    std::vector<double> cost;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        for (size_t i = 0; i < dops.size(); i++) {
            int v = 1;
            if (dops[i].kind == GBX_OP_GEMM && g_tune_loaded && dev < 64) {
                const int t = g_tune[dev][bucket_of(dops[i].m, dops[i].n)];
                v = t < 0 ? 1 : t;
            }
            tile_items(dops[i], (int)i, v, items, cost);
        }
    }
    std::vector<int> order(items.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
    const size_t ops_bytes = sizeof(DevOp) * dops.size();
    const size_t items_off = (ops_bytes + 255) & ~(size_t)255;
    const size_t items_bytes = sizeof(Item) * items.size();
    const size_t ctr_off = (items_off + items_bytes + 255) & ~(size_t)255;
    const size_t total = ctr_off + 256;
    void *h, *d;
    gbx_status st;
    if ((st = gbx_pinned(ctx, total, &h)) != GBX_OK) return st;
    if ((st = gbx_ws(ctx, GBX_WS_BATCH, total, &d)) != GBX_OK) return st;
    memcpy(h, dops.data(), ops_bytes);
    Item *hi = (Item *)((char *)h + items_off);
    for (size_t i = 0; i < order.size(); i++) hi[i] = items[order[i]];
    memset((char *)h + ctr_off, 0, 256);
    cudaStream_t s = (cudaStream_t)gbx_ctx_get_stream(ctx);
    cudaError_t e = cudaMemcpyAsync(d, h, total, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return gbx_fail(ctx, GBX_ERR_CUDA, "grouped upload: %s", cudaGetErrorString(e));
    const int nitems = (int)items.size();
    gbx_timer_begin(ctx, GBX_TIMER_BATCH);
    grouped_kernel<<<std::min(gbx_ctx_sms(ctx) * 2, nitems), BT_THREADS, 0, s>>>(
        (const DevOp *)d, (const Item *)((char *)d + items_off), nitems, (int *)((char *)d + ctr_off));
    gbx_timer_end(ctx);
    gbx_count_launch(ctx, 1);
    return gbx_check_launch(ctx, "grouped kernel");
}

extern "C" gbx_status gbx_plan_create(gbx_ctx *ctx, const gbx_op *ops, int count, gbx_plan **out)
{
    if (!ctx || !out || count < 0 || (count > 0 && !ops)) return GBX_ERR_ARG;
    *out = nullptr;
    std::vector<DevOp> dops;
    dops.reserve(count);
    double flops = 0.0;
    for (int i = 0; i < count; i++) {
        DevOp d;
        bool skip;
        gbx_status st = to_devop(ctx, ops[i], i, d, skip, flops);
        if (st != GBX_OK) return st;
        if (!skip) dops.push_back(d);
    }

    // autotune the GEMM tile variant per bucket
    int dev = gbx_ctx_device(ctx);
    cudaDeviceProp prop;
    char devname[256] = "gpu";
    if (cudaGetDeviceProperties(&prop, dev) == cudaSuccess) snprintf(devname, sizeof devname, "%s", prop.name);
    std::vector<int> variant(dops.size(), 1);
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        if (!g_tune_loaded) tune_load_locked(dev, devname);
        bool changed = false;
        for (int b = 0; b < NBUCKET; b++) {
            std::vector<DevOp> sub;
            for (auto &d : dops)
                if (d.kind == GBX_OP_GEMM && bucket_of(d.m, d.n) == b) sub.push_back(d);
            if (sub.empty() || (dev < 64 && g_tune[dev][b] >= 0)) continue;
            // time on scratch output: same shapes and operands, beta = 0
            double *scratch = nullptr;
            size_t need = 0;
            for (auto &d : sub) need = std::max(need, (size_t)d.ldc * d.n);
            if (cudaMalloc(&scratch, sizeof(double) * std::max<size_t>(need, 1)) != cudaSuccess) {
                cudaGetLastError();
                continue;
            }
            for (auto &d : sub) { d.C = scratch; d.beta = 0.0; }
            const float t32 = time_variant(ctx, sub, 0), t64 = time_variant(ctx, sub, 1);
            cudaFree(scratch);
            if (dev < 64) g_tune[dev][b] = t32 < t64 ? 0 : 1;
            changed = true;
        }
        if (changed && dev < 64) tune_save_locked(dev, devname);
        for (size_t i = 0; i < dops.size(); i++)
            if (dops[i].kind == GBX_OP_GEMM && dev < 64) {
                const int v = g_tune[dev][bucket_of(dops[i].m, dops[i].n)];
                variant[i] = v < 0 ? 1 : v;
            }
    }

    gbx_plan *p = (gbx_plan *)calloc(1, sizeof(gbx_plan));
    if (!p) return GBX_ERR_ALLOC;
    p->device = dev;
    p->flops = flops;
    gbx_status st = upload(ctx, dops, variant, p);
    if (st != GBX_OK) {
        plan_free(p);
        return st;
    }
    *out = p;
    return GBX_OK;
}

extern "C" gbx_status gbx_plan_launch(gbx_ctx *ctx, gbx_plan *p)
{
    if (!ctx || !p) return GBX_ERR_ARG;
    return launch(ctx, p);
}

extern "C" gbx_status gbx_plan_graph_launch(gbx_ctx *ctx, gbx_plan *p)
{
    if (!ctx || !p) return GBX_ERR_ARG;
    cudaStream_t s = (cudaStream_t)gbx_ctx_get_stream(ctx);
    if (!p->gexec) {
        cudaGraph_t g;
        cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return gbx_fail(ctx, GBX_ERR_CUDA, "capture: %s", cudaGetErrorString(e));
        gbx_status st = launch(ctx, p);
        e = cudaStreamEndCapture(s, &g);
        if (st != GBX_OK) return st;
        if (e != cudaSuccess) return gbx_fail(ctx, GBX_ERR_CUDA, "capture end: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&p->gexec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return gbx_fail(ctx, GBX_ERR_CUDA, "instantiate: %s", cudaGetErrorString(e));
    }
    gbx_count_launch(ctx, 1);
    cudaError_t e = cudaGraphLaunch(p->gexec, s);
    return e == cudaSuccess ? GBX_OK : gbx_fail(ctx, GBX_ERR_CUDA, "graph launch: %s", cudaGetErrorString(e));
}

extern "C" gbx_status gbx_plan_destroy(gbx_plan *p)
{
    plan_free(p);
    return GBX_OK;
}

extern "C" gbx_status gbx_plan_info(const gbx_plan *p, int *items, double *flops)
{
    if (!p) return GBX_ERR_ARG;
    if (items) *items = p->nitems;
    if (flops) *flops = p->flops;
    return GBX_OK;
}
