// trace_driver.cu — native driver of the serving workload: host threads, each
// running the call sequence of a blocked right-looking Cholesky factorisation
// (dpotrf of the diagonal block, dtrsm of the panel, then the trailing update
// block column by block column: dsyrk of the diagonal block, dgemm below it),
// either through the serving loop (gbx_server_call) or as plain per-call
// dispatch (one context per thread: gbx_ops_run, then gbx_ctx_sync).  This is
// what an application with C or Fortran threads does; a Python driver adds
// interpreter time and lock contention to every call of every thread, which
// is a property of the harness, not of the library.
//
// The threads start together; each call's latency is taken around the call
// on the calling thread.  Statistics come back in gbx_trace_stats.
#include "gbx_internal.h"
#include "gbxdiag.h"

#include <cuda_runtime.h>
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <mutex>
#include <thread>
#include <vector>

namespace {

using clk = std::chrono::steady_clock;

std::vector<gbx_op> cholesky_ops(int n, int nb, double *A, int lda, int *info, bool ozaki)
{
    std::vector<gbx_op> ops;
    auto at = [&](int i, int j) { return A + (size_t)j * lda + i; };
    for (int k = 0; k < n; k += nb) {
        const int kb = std::min(nb, n - k);
        gbx_op o{};
        o.kind = GBX_OP_POTRF;
        o.uplo = 'L';
        o.n = kb;
        o.C = at(k, k);
        o.ldc = lda;
        o.B = (const double *)info;
        ops.push_back(o);
        const int rest = n - k - kb;
        if (rest <= 0) continue;
        o = gbx_op{};   // L21 = A21 L11^-T
        o.kind = ozaki ? GBX_OP_TRSM_OZAKI : GBX_OP_TRSM;
        o.side = 'R';
        o.uplo = 'L';
        o.transa = 'T';
        o.diag = 'N';
        o.m = rest;
        o.n = kb;
        o.alpha = 1.0;
        o.A = at(k, k);
        o.lda = lda;
        o.C = at(k + kb, k);
        o.ldc = lda;
        ops.push_back(o);
        for (int j = k + kb; j < n; j += nb) {
            const int jb = std::min(nb, n - j);
            o = gbx_op{};
            o.kind = ozaki ? GBX_OP_SYRK_OZAKI : GBX_OP_SYRK;
            o.uplo = 'L';
            o.transa = 'N';
            o.n = jb;
            o.k = kb;
            o.alpha = -1.0;
            o.beta = 1.0;
            o.A = at(j, k);
            o.lda = lda;
            o.C = at(j, j);
            o.ldc = lda;
            ops.push_back(o);
            const int below = n - j - jb;
            if (below > 0) {
                o = gbx_op{};
                o.kind = ozaki ? GBX_OP_GEMM_OZAKI : GBX_OP_GEMM;
                o.transa = 'N';
                o.transb = 'T';
                o.m = below;
                o.n = jb;
                o.k = kb;
                o.alpha = -1.0;
                o.beta = 1.0;
                o.A = at(j + jb, k);
                o.lda = lda;
                o.B = at(j, k);
                o.ldb = lda;
                o.C = at(j + jb, j);
                o.ldc = lda;
                ops.push_back(o);
            }
        }
    }
    return ops;
}


// Runs plan[t] on thread t (all threads start together), through server or
// as plain per-call dispatch, and fills out.
gbx_status run_trace(gbx_server *server, int device, const std::vector<std::vector<gbx_op>> &plan,
                     gbx_trace_stats *out)
{
    const int nthreads = (int)plan.size();
    std::vector<std::vector<float>> lat(nthreads);
    std::vector<double> finish(nthreads, 0.0);
    std::vector<std::array<double, GBX_TRACE_KINDS>> ksum(nthreads);
    std::vector<std::array<uint64_t, GBX_TRACE_KINDS>> kcnt(nthreads);
    std::atomic<int> ready{0};
    std::atomic<bool> go{false};
    std::atomic<int> first_error{0};
    clk::time_point t0;
    auto worker = [&](int t) {
        cudaSetDevice(device);
        gbx_ctx *ctx = nullptr;
        if (!server && gbx_ctx_create(&ctx, device) != GBX_OK) {
            int z = 0;
            first_error.compare_exchange_strong(z, (int)GBX_ERR_CUDA);
        }
        ksum[t].fill(0.0);
        kcnt[t].fill(0);
        lat[t].reserve(plan[t].size());
        ready++;
        while (!go.load(std::memory_order_acquire)) std::this_thread::yield();
        for (const gbx_op &op : plan[t]) {
            if (first_error.load(std::memory_order_relaxed)) break;
            const auto c0 = clk::now();
            gbx_status st;
            if (server) {
                double us = 0.0;
                st = gbx_server_call(server, &op, &us);
            } else if (ctx) {
                st = gbx_ops_run(ctx, &op, 1);
                const gbx_status s2 = gbx_ctx_sync(ctx);
                if (st == GBX_OK) st = s2;
            } else {
                st = GBX_ERR_CUDA;
            }
            const double us = std::chrono::duration<double, std::micro>(clk::now() - c0).count();
            if (st != GBX_OK) {
                int z = 0;
                first_error.compare_exchange_strong(z, (int)st);
                break;
            }
            lat[t].push_back((float)us);
            const int kind = op.kind >= 0 && op.kind < GBX_TRACE_KINDS ? op.kind : 0;
            ksum[t][kind] += us;
            kcnt[t][kind]++;
        }
        finish[t] = std::chrono::duration<double>(clk::now() - t0).count();
        if (ctx) gbx_ctx_destroy(ctx);
    };
    std::vector<std::thread> threads;
    for (int t = 0; t < nthreads; t++) threads.emplace_back(worker, t);
    while (ready.load() < nthreads) std::this_thread::yield();
    t0 = clk::now();
    go.store(true, std::memory_order_release);
    for (auto &th : threads) th.join();
    out->wall_s = std::chrono::duration<double>(clk::now() - t0).count();
    std::vector<float> all;
    for (int t = 0; t < nthreads; t++) {
        all.insert(all.end(), lat[t].begin(), lat[t].end());
        out->thread_finish_s[t] = finish[t];
        for (int k = 0; k < GBX_TRACE_KINDS; k++) {
            out->kind_calls[k] += kcnt[t][k];
            out->kind_sum_us[k] += ksum[t][k];
        }
    }
    out->calls = all.size();
    if (!all.empty()) {
        std::sort(all.begin(), all.end());
        out->p50_us = all[all.size() / 2];
        out->p99_us = all[(size_t)(0.99 * (double)(all.size() - 1))];
    }
    out->first_error = first_error.load();
    return GBX_OK;
}

}  // namespace

extern "C" gbx_status gbx_diag_cholesky_trace(gbx_server *server, int device, int nthreads, const int *n,
                                              const int *nb, double *const *A, const int *lda, int *info,
                                              int ozaki, gbx_trace_stats *out)
{
    if (!out || nthreads < 1 || nthreads > GBX_TRACE_MAX_THREADS || !n || !nb || !A || !lda || !info)
        return GBX_ERR_ARG;
    *out = gbx_trace_stats{};
    std::vector<std::vector<gbx_op>> plan(nthreads);
    for (int t = 0; t < nthreads; t++) {
        if (n[t] < 1 || nb[t] < 1 || nb[t] > 256 || lda[t] < n[t] || !A[t]) return GBX_ERR_ARG;
        plan[t] = cholesky_ops(n[t], nb[t], A[t], lda[t], info + t, ozaki != 0);
    }
    return run_trace(server, device, plan, out);
}

extern "C" gbx_status gbx_diag_ops_trace(gbx_server *server, int device, int nthreads, const gbx_op *const *ops,
                                         const int *count, gbx_trace_stats *out)
{
    if (!out || nthreads < 1 || nthreads > GBX_TRACE_MAX_THREADS || !ops || !count) return GBX_ERR_ARG;
    *out = gbx_trace_stats{};
    std::vector<std::vector<gbx_op>> plan(nthreads);
    for (int t = 0; t < nthreads; t++) {
        if (count[t] < 0 || (count[t] > 0 && !ops[t])) return GBX_ERR_ARG;
        plan[t].assign(ops[t], ops[t] + count[t]);
    }
    return run_trace(server, device, plan, out);
}
