// serve.cu — continuous-batching serving loop for BLAS calls from many host
// threads (no reference counterpart: the reference runs one call at a time
// on one cuBLAS handle and the legacy stream, runtime-blas.c:14-23).
//
// Host threads submit operations on device-resident operands and wait on a
// ticket.  Each slot (one context: stream and workspace) has a worker
// thread.  A free worker takes the next queued work -- every small
// DGEMM/DTRSM request queued at that moment, grouped into one kernel
// launch, or the next large request -- launches it on its own stream,
// waits for it, completes the tickets and records per-call latency (submit
// to completion) for p50/p99.  Work that arrives while other work is on the
// GPU is admitted as slots free up and overlaps with it; the host-side cost
// of enqueueing (argument checks, tensor-map encoding, launches) is spread
// over the workers instead of one dispatcher thread.

// A result is bit-identical whether the call was served alone or in a mix:
// a small DGEMM (m, n <= 512, k <= 4096) runs inline on a free slot when
// nothing is queued to group it with, else grouped, and both routes compute
// each element with the same FMA chain and epilogue; a small DTRSM (order
// <= 256) always runs in the grouped kernel, inline as a group of one or
// with others; everything else runs alone.
// Critical-path requests (DPOTRF of a diagonal block, DTRSM of a panel) run
// on a high-priority stream of their slot.
//
// Small FP64 DGEMM, DSYRK and DTRSM requests (m, n <= 512, k <= 4096;
// triangle order <= 256, at most 256 right-hand sides) made through
// gbx_server_call can run on the device-side request loop (serve_loop.cu): a
// resident kernel fed through a ring in pinned host memory, so such a call
// costs no launch, stream synchronisation or worker-thread hand-off.  The
// loop holds a quarter of the SMs while it is resident (it leaves the GPU
// after 20 ms without work), which pays off for latency-bound callers and
// loses on FP64-bound traces, so it is opt-in: GBX_SERVE_LOOP=1 at server
// creation.
//
// Admission by memory: callers that stage host operands reserve their bytes
// with gbx_server_admit (blocks while the reserved total would exceed the
// budget: a fraction of the free HBM when the server started, or an explicit
// cap) and give them back with gbx_server_release.
#include "gbx_internal.h"

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

extern "C" gbx_status gbx_grouped_launch_inline(gbx_ctx *ctx, const gbx_op *ops, int count);

namespace {

using clk = std::chrono::steady_clock;

struct Request {
    gbx_op op;
    uint64_t ticket;
    clk::time_point t_submit, t_done;
    gbx_status status;
    bool done;
};

struct Slot {
    gbx_ctx *ctx = nullptr;
    cudaStream_t hi = nullptr;   // high-priority stream for critical-path requests
    bool busy = false;   // taken by its worker or by a calling thread (under the server mutex)
};

bool is_small(const gbx_op &o)
{
    if (o.kind == GBX_OP_GEMM) return o.m <= 512 && o.n <= 512 && o.k <= 4096;
    if (o.kind == GBX_OP_TRSM) return (gbx_lsame(o.side, 'L') ? o.m : o.n) <= 256;
    return false;
}

}  // namespace

struct gbx_server {
    int device;
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done, cv_mem;
    std::deque<Request *> queue;
    std::vector<Request *> finished;   // completed, not yet waited for
    uint64_t next_ticket = 1;
    bool stop = false;
    std::vector<std::thread> workers;
    // latency record (microseconds), ring of the last 1M calls
    std::vector<float> lat;
    size_t lat_next = 0, completed = 0, batches = 0, grouped_calls = 0;
    // memory admission
    size_t budget = 0, reserved = 0;
    uint64_t admission_waits = 0;
    // device-side request loop (null when disabled)
    gbx_loop *loop = nullptr;
    std::atomic<uint64_t> loop_calls{0};
};

namespace {

gbx_status run_request(gbx_ctx *ctx, const gbx_op &o)
{
    switch (o.kind) {
    case GBX_OP_GEMM:
        return gbx_dgemm(ctx, o.transa, o.transb, o.m, o.n, o.k, o.alpha, o.A, o.lda, o.B, o.ldb, o.beta, o.C,
                         o.ldc);
    case GBX_OP_TRSM:
        return gbx_dtrsm(ctx, o.side, o.uplo, o.transa, o.diag, o.m, o.n, o.alpha, o.A, o.lda, o.C, o.ldc);
    case GBX_OP_SYRK:
        return gbx_dsyrk(ctx, o.uplo, o.transa, o.n, o.k, o.alpha, o.A, o.lda, o.beta, o.C, o.ldc);
    case GBX_OP_DOT:
        return gbx_ddot(ctx, o.n, o.A, o.lda, o.B, o.ldb, o.C);
    case GBX_OP_NRM2:
        return gbx_dnrm2(ctx, o.n, o.A, o.lda, o.C);
    case GBX_OP_POTRF:
        return gbx_dpotrf_small(ctx, o.uplo, o.n, o.C, o.ldc, (int *)o.B);
    case GBX_OP_GEMM_OZAKI:
        return gbx_dgemm_ozaki(ctx, o.transa, o.transb, o.m, o.n, o.k, o.alpha, o.A, o.lda, o.B, o.ldb,
                               o.beta, o.C, o.ldc, 0.0, 0, nullptr);
    case GBX_OP_TRSM_OZAKI:
        return gbx_dtrsm_ozaki(ctx, o.side, o.uplo, o.transa, o.diag, o.m, o.n, o.alpha, o.A, o.lda, o.C, o.ldc,
                               0.0, 0, nullptr);
    case GBX_OP_SYRK_OZAKI:
        return gbx_dsyrk_ozaki(ctx, o.uplo, o.transa, o.n, o.k, o.alpha, o.A, o.lda, o.beta, o.C, o.ldc, 0.0, 0,
                               nullptr);
    default:
        return GBX_ERR_ARG;
    }
}

// The sequential steps of blocked factorizations (the diagonal-block
// Cholesky and the panel solves) gate every later call of their chain, while
// the trailing updates they release are many and independent: they run on
// the slot's high-priority stream, so their CTAs are scheduled ahead of
// queued trailing-update CTAs as SMs free up.
bool is_critical(const gbx_op &o)
{
    return o.kind == GBX_OP_POTRF || o.kind == GBX_OP_TRSM || o.kind == GBX_OP_TRSM_OZAKI;
}

// One request on a slot, synchronised (the slot's stream, or its
// high-priority stream for a critical-path request).
gbx_status run_on_slot(Slot *sl, const gbx_op &o)
{
    const bool hi = sl->hi && is_critical(o);
    if (hi) gbx_ctx_set_stream(sl->ctx, sl->hi);
    gbx_status st = run_request(sl->ctx, o);
    const gbx_status sync = gbx_ctx_sync(sl->ctx);   // also collects bounded-wait status words
    if (hi) gbx_ctx_set_stream(sl->ctx, nullptr);
    return st == GBX_OK ? sync : st;
}

// A small DTRSM run inline by its caller: the grouped kernel on its own, so
// that its bits are those of the grouped route it takes under load.
gbx_status run_grouped_on_slot(Slot *sl, const gbx_op &o)
{
    const bool hi = sl->hi && is_critical(o);
    if (hi) gbx_ctx_set_stream(sl->ctx, sl->hi);
    gbx_status st = gbx_grouped_launch_inline(sl->ctx, &o, 1);
    const gbx_status sync = gbx_ctx_sync(sl->ctx);
    if (hi) gbx_ctx_set_stream(sl->ctx, nullptr);
    return st == GBX_OK ? sync : st;
}

}  // namespace

extern "C" gbx_status gbx_ops_run(gbx_ctx *ctx, const gbx_op *ops, int count)
{
    if (!ctx || count < 0 || (count > 0 && !ops)) return GBX_ERR_ARG;
    for (int i = 0; i < count; i++) {
        gbx_status st = run_request(ctx, ops[i]);
        if (st != GBX_OK) return st;
    }
    return GBX_OK;
}

namespace {

void record(gbx_server *s, clk::time_point t0, clk::time_point t1)
{
    const float us = (float)std::chrono::duration<double, std::micro>(t1 - t0).count();
    if (s->lat.size() < (1u << 20)) s->lat.push_back(us);
    else s->lat[s->lat_next++ % s->lat.size()] = us;
    s->completed++;
}

void complete(gbx_server *s, const std::vector<Request *> &reqs, gbx_status st)
{
    const auto now = clk::now();
    for (auto *r : reqs) {
        if (r->status == GBX_OK) r->status = st;
        r->t_done = now;
        r->done = true;
        record(s, r->t_submit, r->t_done);
        s->finished.push_back(r);
    }
}

void worker_loop(gbx_server *s, Slot *sl)
{
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        s->cv_work.wait(lk, [&] { return s->stop || (!s->queue.empty() && !sl->busy); });
        if (s->queue.empty()) {
            if (s->stop) break;
            continue;
        }
        sl->busy = true;
        // take the front request; if it is small, every small request queued
        // now goes with it into one grouped launch
        std::vector<Request *> mine;
        const bool small = is_small(s->queue.front()->op);
        if (small) {
            for (auto it = s->queue.begin(); it != s->queue.end();) {
                if (is_small((*it)->op)) {
                    mine.push_back(*it);
                    it = s->queue.erase(it);
                } else {
                    ++it;
                }
            }
        } else {
            mine.push_back(s->queue.front());
            s->queue.pop_front();
        }
        if (!s->queue.empty()) s->cv_work.notify_one();   // more work for another worker
        lk.unlock();
        gbx_status st;
        if (small) {
            std::vector<gbx_op> ops;
            ops.reserve(mine.size());
            for (auto *r : mine) ops.push_back(r->op);
            st = gbx_grouped_launch_inline(sl->ctx, ops.data(), (int)ops.size());
            const gbx_status sync = gbx_ctx_sync(sl->ctx);   // also collects bounded-wait status words
            if (st == GBX_OK) st = sync;
        } else {
            st = run_on_slot(sl, mine[0]->op);
        }
        lk.lock();
        sl->busy = false;
        s->batches++;
        if (small) s->grouped_calls += mine.size();
        complete(s, mine, st);
        s->cv_done.notify_all();
        if (!s->queue.empty()) s->cv_work.notify_all();
    }
}

}  // namespace

extern "C" gbx_status gbx_server_create(int device, int nslots, size_t mem_budget, gbx_server **out)
{
    if (!out || nslots < 1 || nslots > 64) return GBX_ERR_ARG;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return GBX_ERR_CUDA;
    gbx_server *s = new gbx_server();
    s->device = device;
    s->slots.resize(nslots);
    int prio_low = 0, prio_high = 0;
    cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    for (auto &sl : s->slots) {
        if (gbx_ctx_create(&sl.ctx, device) != GBX_OK ||
            cudaStreamCreateWithPriority(&sl.hi, cudaStreamNonBlocking, prio_high) != cudaSuccess) {
            cudaGetLastError();
            for (auto &q : s->slots) {
                if (q.ctx) gbx_ctx_destroy(q.ctx);
                if (q.hi) cudaStreamDestroy(q.hi);
            }
            delete s;
            return GBX_ERR_CUDA;
        }
    }
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const size_t auto_budget = free_b / 10 * 8;   // 80% of what is free now
    s->budget = mem_budget ? std::min(mem_budget, auto_budget) : auto_budget;
    const char *lp = getenv("GBX_SERVE_LOOP");
    if (lp && atoi(lp) != 0) {
        // a quarter of the SMs: the loop takes the small requests, and the SMs it
        // leaves free run the large ones and the factorisation steps on the slot streams
        int sms = 152;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        int ctas = std::max(8, sms / 4);
        // GBX_SERVE_LOOP_CTAS: another size (at most one CTA per SM), e.g. every
        // SM for callers whose requests are all small
        if (const char *lc = getenv("GBX_SERVE_LOOP_CTAS"))
            if (atoi(lc) > 0) ctas = std::min(atoi(lc), sms);
        if (gbx_loop_create(device, ctas, &s->loop) != GBX_OK) s->loop = nullptr;
    }
    for (auto &sl : s->slots) s->workers.emplace_back(worker_loop, s, &sl);
    *out = s;
    return GBX_OK;
}

extern "C" gbx_status gbx_server_submit(gbx_server *s, const gbx_op *op, uint64_t *ticket)
{
    if (!s || !op || !ticket) return GBX_ERR_ARG;
    Request *r = new Request();
    r->op = *op;
    r->status = GBX_OK;
    r->done = false;
    r->t_submit = clk::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) {
            delete r;
            return GBX_ERR_ARG;
        }
        r->ticket = s->next_ticket++;
        s->queue.push_back(r);
        *ticket = r->ticket;
    }
    s->cv_work.notify_one();
    return GBX_OK;
}

extern "C" gbx_status gbx_server_wait(gbx_server *s, uint64_t ticket, double *latency_us)
{
    if (!s) return GBX_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    Request *found = nullptr;
    s->cv_done.wait(lk, [&] {
        for (size_t i = 0; i < s->finished.size(); i++)
            if (s->finished[i]->ticket == ticket) {
                found = s->finished[i];
                s->finished[i] = s->finished.back();
                s->finished.pop_back();
                return true;
            }
        return false;
    });
    const gbx_status st = found->status;
    if (latency_us)
        *latency_us = std::chrono::duration<double, std::micro>(found->t_done - found->t_submit).count();
    delete found;
    return st;
}

// A large request whose caller would only wait for it runs on the calling
// thread, on a free slot's stream: the slot pool still bounds how much work
// is on the GPU, and no hand-off to and back from a worker thread is added
// to a latency that sits on the caller's critical path.  Small requests (and
// large ones that find every slot busy) go through the queue and are grouped.
extern "C" gbx_status gbx_server_call(gbx_server *s, const gbx_op *op, double *latency_us)
{
    if (!s || !op) return GBX_ERR_ARG;
    if (s->loop && gbx_loop_accepts(op)) {
        const auto t0 = clk::now();
        const gbx_status st = gbx_loop_call(s->loop, op);
        const auto t1 = clk::now();
        {
            std::lock_guard<std::mutex> lk(s->mu);
            record(s, t0, t1);
        }
        s->loop_calls++;
        if (latency_us) *latency_us = std::chrono::duration<double, std::micro>(t1 - t0).count();
        return st;
    }
    // Large requests, and small ones that would find nothing queued to
    // group with, run inline on a free slot: a hand-off to a worker and back
    // cost a small call about 85 us.  A small DGEMM gives the same bits
    // either way (the grouped tile uses the GEMM core's arithmetic); a small
    // DTRSM runs inline as a grouped launch of its own, so its bits are
    // those of the grouped route whatever the load.
    const bool small = is_small(*op);
    {
        Slot *sl = nullptr;
        const auto t0 = clk::now();
        {
            std::lock_guard<std::mutex> lk(s->mu);
            if (s->stop) return GBX_ERR_ARG;
            bool group = false;
            if (small)
                for (auto *r : s->queue)
                    if (is_small(r->op)) {
                        group = true;
                        break;
                    }
            if (!group)
                for (auto &q : s->slots)
                    if (!q.busy) {
                        sl = &q;
                        q.busy = true;
                        break;
                    }
        }
        if (sl) {
            cudaSetDevice(s->device);
            const gbx_status st = (small && op->kind == GBX_OP_TRSM) ? run_grouped_on_slot(sl, *op)
                                                                      : run_on_slot(sl, *op);
            const auto t1 = clk::now();
            bool waiting;
            {
                std::lock_guard<std::mutex> lk(s->mu);
                sl->busy = false;
                s->batches++;
                record(s, t0, t1);
                waiting = !s->queue.empty();
            }
            // a queued request may be waiting for this slot; with an empty
            // queue nobody is (waking every worker per call cost the host
            // cores as many futex round trips as there are slots)
            if (waiting) s->cv_work.notify_all();
            if (latency_us) *latency_us = std::chrono::duration<double, std::micro>(t1 - t0).count();
            return st;
        }
    }
    uint64_t t;
    gbx_status st = gbx_server_submit(s, op, &t);
    if (st != GBX_OK) return st;
    return gbx_server_wait(s, t, latency_us);
}

extern "C" gbx_status gbx_server_admit(gbx_server *s, size_t bytes)
{
    if (!s) return GBX_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    if (bytes > s->budget) return GBX_ERR_ADMISSION;   // can never fit
    if (s->reserved + bytes > s->budget) s->admission_waits++;
    s->cv_mem.wait(lk, [&] { return s->reserved + bytes <= s->budget; });
    s->reserved += bytes;
    return GBX_OK;
}

extern "C" gbx_status gbx_server_release(gbx_server *s, size_t bytes)
{
    if (!s) return GBX_ERR_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->reserved = bytes > s->reserved ? 0 : s->reserved - bytes;
    }
    s->cv_mem.notify_all();
    return GBX_OK;
}

extern "C" gbx_status gbx_server_stats(gbx_server *s, uint64_t *completed, uint64_t *batches,
                                       uint64_t *grouped_calls, double *p50_us, double *p99_us,
                                       uint64_t *admission_waits)
{
    if (!s) return GBX_ERR_ARG;
    std::vector<float> v;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        v = s->lat;
        if (completed) *completed = s->completed;
        if (batches) *batches = s->batches;
        if (grouped_calls) *grouped_calls = s->grouped_calls;
        if (admission_waits) *admission_waits = s->admission_waits;
    }
    double p50 = 0.0, p99 = 0.0;
    if (!v.empty()) {
        std::sort(v.begin(), v.end());
        p50 = v[(size_t)(0.50 * (v.size() - 1))];
        p99 = v[(size_t)(0.99 * (v.size() - 1))];
    }
    if (p50_us) *p50_us = p50;
    if (p99_us) *p99_us = p99;
    return GBX_OK;
}

extern "C" gbx_status gbx_server_loop_stats(gbx_server *s, int *enabled, uint64_t *calls, uint64_t *launches)
{
    if (!s) return GBX_ERR_ARG;
    if (enabled) *enabled = s->loop != nullptr;
    if (calls) *calls = s->loop_calls.load();
    if (launches) *launches = gbx_loop_launches(s->loop);
    return GBX_OK;
}

extern "C" gbx_status gbx_server_reset_stats(gbx_server *s)
{
    if (!s) return GBX_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    s->lat.clear();
    s->lat_next = 0;
    s->completed = s->batches = s->grouped_calls = 0;
    s->admission_waits = 0;
    return GBX_OK;
}

extern "C" gbx_status gbx_server_destroy(gbx_server *s)
{
    if (!s) return GBX_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    s->cv_done.notify_all();
    for (auto &w : s->workers)
        if (w.joinable()) w.join();
    if (s->loop) gbx_loop_destroy(s->loop);
    for (auto *r : s->finished) delete r;
    for (auto &sl : s->slots) {
        if (sl.ctx) gbx_ctx_destroy(sl.ctx);
        if (sl.hi) cudaStreamDestroy(sl.hi);
    }
    delete s;
    return GBX_OK;
}
