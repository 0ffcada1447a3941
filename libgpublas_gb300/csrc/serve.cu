// serve.cu — continuous-batching serving loop for BLAS calls from many host
// threads (no reference counterpart: the reference runs one call at a time
// on one cuBLAS handle and the legacy stream, runtime-blas.c:14-23).
//
// Host threads submit operations on device-resident operands and wait on a
// ticket.  A dispatcher thread repeatedly takes everything queued, groups
// the small DGEMM/DTRSM requests into one grouped kernel launch and runs the
// large ones with the regular routines, each on the stream of a free slot
// (one context per slot), so work that arrives while other work is on the
// GPU is admitted as slots free up and overlaps with it.  A completion
// thread watches the slots' events, completes tickets and records per-call
// latency (submit to completion) for p50/p99.
//
// Routing depends only on the operation (small GEMM: m, n <= 512 and
// k <= 4096; small TRSM: order <= 256; everything else runs alone), so a
// result is bit-identical whether the call was served alone or in a mix.
//
// Admission by memory: callers that stage host operands reserve their bytes
// with gbx_server_admit (blocks while the reserved total would exceed the
// budget: a fraction of the free HBM when the server started, or an explicit
// cap) and give them back with gbx_server_release.
#include "gbx_internal.h"

#include <cuda_runtime.h>
#include <stdint.h>
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
    cudaEvent_t ev = nullptr;
    bool busy = false;       // taken by the dispatcher
    bool launched = false;   // its event was recorded behind the work
    std::vector<Request *> reqs;
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
    std::thread dispatcher, completer;
    // latency record (microseconds), ring of the last 1M calls
    std::vector<float> lat;
    size_t lat_next = 0, completed = 0, batches = 0, grouped_calls = 0;
    // memory admission
    size_t budget = 0, reserved = 0;
    uint64_t admission_waits = 0;
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
    case GBX_OP_SYRK_OZAKI:
        return gbx_dsyrk_ozaki(ctx, o.uplo, o.transa, o.n, o.k, o.alpha, o.A, o.lda, o.beta, o.C, o.ldc, 0.0, 0,
                               nullptr);
    default:
        return GBX_ERR_ARG;
    }
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

void dispatcher_loop(gbx_server *s)
{
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        s->cv_work.wait(lk, [&] {
            if (s->stop) return true;
            if (s->queue.empty()) return false;
            for (auto &sl : s->slots)
                if (!sl.busy) return true;
            return false;
        });
        if (s->stop && s->queue.empty()) break;
        if (s->queue.empty()) continue;
        // take everything queued; small ones go together into one slot
        std::vector<Request *> small, large;
        while (!s->queue.empty()) {
            Request *r = s->queue.front();
            s->queue.pop_front();
            (is_small(r->op) ? small : large).push_back(r);
        }
        auto take_slot = [&]() -> Slot * {
            for (auto &sl : s->slots)
                if (!sl.busy) return &sl;
            return nullptr;
        };
        std::vector<Request *> leftover;
        if (!small.empty()) {
            Slot *sl = take_slot();
            if (sl) {
                sl->busy = true;
                sl->reqs = small;
                std::vector<gbx_op> ops;
                ops.reserve(small.size());
                for (auto *r : small) ops.push_back(r->op);
                lk.unlock();
                gbx_status st = gbx_grouped_launch_inline(sl->ctx, ops.data(), (int)ops.size());
                cudaEventRecord(sl->ev, (cudaStream_t)gbx_ctx_get_stream(sl->ctx));
                lk.lock();
                sl->launched = true;
                for (auto *r : small) r->status = st;
                s->batches++;
                s->grouped_calls += small.size();
            } else {
                leftover.insert(leftover.end(), small.begin(), small.end());
            }
        }
        for (auto *r : large) {
            Slot *sl = take_slot();
            if (!sl) {
                leftover.push_back(r);
                continue;
            }
            sl->busy = true;
            sl->reqs.assign(1, r);
            lk.unlock();
            gbx_status st = run_request(sl->ctx, r->op);
            cudaEventRecord(sl->ev, (cudaStream_t)gbx_ctx_get_stream(sl->ctx));
            lk.lock();
            sl->launched = true;
            r->status = st;
            s->batches++;
        }
        // requests that found no free slot go back to the front, in order
        for (auto it = leftover.rbegin(); it != leftover.rend(); ++it) s->queue.push_front(*it);
        s->cv_done.notify_all();   // wake the completer
    }
}

void completer_loop(gbx_server *s)
{
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        bool any_busy = false, progressed = false;
        for (auto &sl : s->slots) {
            if (!sl.busy) continue;
            any_busy = true;
            if (!sl.launched) continue;   // the dispatcher is still enqueueing
            lk.unlock();
            cudaError_t q = cudaEventQuery(sl.ev);
            lk.lock();
            if (q == cudaErrorNotReady) continue;
            gbx_status st = GBX_OK;
            if (q != cudaSuccess) st = GBX_ERR_CUDA;
            else st = gbx_ctx_sync(sl.ctx);   // collects bounded-wait status words
            const auto now = clk::now();
            for (auto *r : sl.reqs) {
                if (r->status == GBX_OK) r->status = st;
                r->t_done = now;
                r->done = true;
                const float us =
                    (float)std::chrono::duration<double, std::micro>(r->t_done - r->t_submit).count();
                if (s->lat.size() < (1u << 20)) s->lat.push_back(us);
                else s->lat[s->lat_next++ % s->lat.size()] = us;
                s->completed++;
                s->finished.push_back(r);
            }
            sl.reqs.clear();
            sl.busy = false;
            sl.launched = false;
            progressed = true;
        }
        if (progressed) {
            s->cv_done.notify_all();
            s->cv_work.notify_all();
        }
        if (s->stop && !any_busy && s->queue.empty()) break;
        if (!any_busy) {
            s->cv_done.wait_for(lk, std::chrono::milliseconds(5));
        } else if (!progressed) {
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(20));
            lk.lock();
        }
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
    for (auto &sl : s->slots) {
        if (gbx_ctx_create(&sl.ctx, device) != GBX_OK ||
            cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) != cudaSuccess) {
            for (auto &q : s->slots) {
                if (q.ctx) gbx_ctx_destroy(q.ctx);
                if (q.ev) cudaEventDestroy(q.ev);
            }
            delete s;
            return GBX_ERR_CUDA;
        }
    }
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const size_t auto_budget = free_b / 10 * 8;   // 80% of what is free now
    s->budget = mem_budget ? std::min(mem_budget, auto_budget) : auto_budget;
    s->dispatcher = std::thread(dispatcher_loop, s);
    s->completer = std::thread(completer_loop, s);
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

extern "C" gbx_status gbx_server_call(gbx_server *s, const gbx_op *op, double *latency_us)
{
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
    if (s->dispatcher.joinable()) s->dispatcher.join();
    if (s->completer.joinable()) s->completer.join();
    for (auto *r : s->finished) delete r;
    for (auto &sl : s->slots) {
        if (sl.ctx) gbx_ctx_destroy(sl.ctx);
        if (sl.ev) cudaEventDestroy(sl.ev);
    }
    delete s;
    return GBX_OK;
}
