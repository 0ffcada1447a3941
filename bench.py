#!/usr/bin/env python
"""Headline benchmark: FP64 DGEMM throughput of libgbxblas on one GB300.

Workload (default): DGEMM 'N','N', M = N = K = 8192, column-major, lda = ldb =
ldc = 8192, alpha = 1, beta = 0.5, A, B, C uniform[-1,1] from SplitMix64 seed
1 (the plain FP64 drop-in sweep's DGEMM at n = 8192).  One step = one DGEMM
call.  Operands (3 x 512 MiB) are larger than the 129 MB L2, so no flush is
needed between steps.

  value  -- TFLOP/s (2*n^3 per step) with operands resident in HBM, timed
            with CUDA events on the library's stream (device C ABI, gbx_dgemm)
  e2e    -- the same metric through the drop-in Fortran symbol dgemm_ on
            pinned host buffers: every step copies A, B, C host->device and C
            device->host inside the timed region
  ozaki  -- the opt-in Ozaki split-precision DGEMM on the same operands
            (TFLOP/s counted as 2*n^3, relative Frobenius error against the
            double-double oracle on sampled entries, slices used)
  roofline -- the dominant kernel (DFMA GEMM core) against the FP64 FMA rate
            measured in the same run
  cpu_baseline -- the CPU BLAS the reference falls back to (OpenBLAS through
            its Fortran symbol) on this host's cores

--impl reference times that CPU BLAS alone on the same workload (the
reference's runnable path: dlsym(RTLD_NEXT) to the CPU BLAS).

Multi-GPU: calls are independent, so N > 1 runs N replicas (one per rank,
no collective on the data path); value = all ranks' flops / max time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--n", type=int, default=8192)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-ozaki", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    return p.parse_args()


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={CLOCK_FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names[1:], f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, v, device=None):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_inputs(n, seed):
    import oracle
    orc = oracle.get()
    a, s = orc.matrix(n, n, seed)
    b, s = orc.matrix(n, n, s)
    c, s = orc.matrix(n, n, s)
    return orc, a, b, c


def cpu_dgemm_rate(cb, a, b, c, n, reps, threads):
    """Median TFLOP/s of the CPU BLAS dgemm_ (1 warm-up + reps timed)."""
    cb.set_threads(threads)
    cc = c.copy(order="F")
    cb.dgemm("N", "N", n, n, n, 1.0, a, b, 0.5, cc)
    times = []
    for _ in range(reps):
        cc = c.copy(order="F")
        t0 = time.perf_counter()
        cb.dgemm("N", "N", n, n, n, 1.0, a, b, 0.5, cc)
        times.append(time.perf_counter() - t0)
    return 2.0 * n ** 3 / statistics.median(times) / 1e12, times


def config_block(n, ws):
    return {"workload": f"dgemm_NN_m{n}_n{n}_k{n}_fp64", "m": n, "n": n, "k": n,
            "lda": n, "alpha": 1.0, "beta": 0.5, "inputs": "uniform[-1,1] SplitMix64 seed 1",
            "l2": "operands 3 x %d MiB > 129 MB L2; no flush needed" % (n * n * 8 >> 20),
            "parallelism": "replicas" if ws > 1 else "single-gpu"}


def run_reference(args):
    ws, rank, local = dist_setup(args)
    if rank != 0:
        barrier(ws)
        return
    from oracle import cpublas
    cb = cpublas.get()
    threads = os.cpu_count() or 1
    n = args.n
    _, a, b, c = make_inputs(n, args.seed)
    cb.set_threads(threads)
    cc = c.copy(order="F")
    for _ in range(args.warmup):
        cb.dgemm("N", "N", n, n, n, 1.0, a, b, 0.5, cc)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cb.dgemm("N", "N", n, n, n, 1.0, a, b, 0.5, cc)
    dt = time.perf_counter() - t0
    value = 2.0 * n ** 3 * args.steps / dt / 1e12
    line = {
        "impl": "reference", "metric": "dgemm_tflops", "value": value, "unit": "TFLOP/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_block(n, ws),
        "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": threads, "kind": "reference",
                         "sample": f"CPU BLAS dgemm_ NN n={n}, {args.steps} timed calls after "
                                   f"{args.warmup} warm-up ({cb.config})"},
        "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    barrier(ws)


def traffic_from_profiles(name):
    """Per-launch DRAM bytes of a kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as fh:
            return json.load(fh).get(name)
    except (OSError, ValueError):
        return None


def run_ours(args):
    import torch
    ws, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    import libgpublas_gb300 as g
    from libgpublas_gb300 import build
    build.build_library()
    n = args.n
    orc, a, b, c = make_inputs(n, args.seed)
    flops = 2.0 * n ** 3

    dev = g.Device(local)
    stream = torch.cuda.ExternalStream(dev.stream())
    da = torch.from_numpy(a.ravel(order="F")).cuda()
    db = torch.from_numpy(b.ravel(order="F")).cuda()
    dc0 = torch.from_numpy(c.ravel(order="F")).cuda()
    dc = dc0.clone()
    torch.cuda.synchronize()

    # ---- device-resident timed region ------------------------------------
    for _ in range(args.warmup):
        dev.dgemm_checked("N", "N", n, n, n, 1.0, da, n, db, n, 0.5, dc, n)
    dev.sync()
    dev.enable_timing(True)
    l0 = dev.launches()
    barrier(ws)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            dev.dgemm_checked("N", "N", n, n, n, 1.0, da, n, db, n, 0.5, dc, n)
        ev1.record(stream)
        ev1.synchronize()
    torch.cuda.synchronize()
    barrier(ws)
    launches = dev.launches() - l0
    t = ev0.elapsed_time(ev1) / 1e3
    t_max = max_over_ranks(ws, t, device="cuda")
    value = flops * args.steps * ws / t_max / 1e12
    k_ms, k_n = dev.kernel_time(dev.TIMER_GEMM_FP64)
    dev.enable_timing(False)
    peak = dev.fp64_peak()
    achieved = flops / (k_ms / max(k_n, 1) / 1e3) / 1e12

    line = {
        "metric": "dgemm_tflops", "value": value, "unit": "TFLOP/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config_block(n, ws), "gpu_launches": int(launches),
        "roofline": {"bound": "fp64", "kernel": "gemm_simt_kernel<double,8,8,8>",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None,
                     "peak_source": "measured in this run: DFMA throughput loop "
                                    "(gbx_diag_fp64_peak); MEASURED_PEAKS.json has no FP64 figure",
                     "traffic": traffic_from_profiles("gemm_simt_kernel_dgemm_nn_8192"),
                     "algorithmic": "2*n^3 flop per launch"},
        "clocks": clk.summary(),
    }

    # ---- end to end through the Fortran symbol on pinned host buffers ----
    if not args.no_e2e:
        ha = torch.from_numpy(a.ravel(order="F")).pin_memory()
        hb = torch.from_numpy(b.ravel(order="F")).pin_memory()
        hc = torch.from_numpy(c.ravel(order="F")).pin_memory()
        f = g.F77()
        pa, pb, pc = ha.data_ptr(), hb.data_ptr(), hc.data_ptr()
        f.dgemm("N", "N", n, n, n, 1.0, pa, n, pb, n, 0.5, pc, n)
        s0 = g.stats()
        barrier(ws)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            f.dgemm("N", "N", n, n, n, 1.0, pa, n, pb, n, 0.5, pc, n)
        te = time.perf_counter() - t0
        s1 = g.stats()
        te = max_over_ranks(ws, te, device="cuda")
        line["e2e"] = {"value": flops * args.steps * ws / te / 1e12, "unit": "TFLOP/s",
                       "h2d_bytes_per_step": (s1["bytes_h2d"] - s0["bytes_h2d"]) // args.steps,
                       "d2h_bytes_per_step": (s1["bytes_d2h"] - s0["bytes_d2h"]) // args.steps,
                       "api": "dgemm_ (Fortran ABI), pinned host operands"}

    # ---- Ozaki split-precision on the same operands --------------------------
    if not args.no_ozaki:
        try:
            line["ozaki"] = bench_ozaki(args, dev, orc, a, b, c, da, db, dc0, n, stream)
        except g.GbxError as e:
            line["ozaki"] = {"unavailable": str(e)}

    # ---- CPU baseline: the CPU BLAS on this host --------------------------
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        from oracle import cpublas
        cb = cpublas.get()
        threads = os.cpu_count() or 1
        rate, times = cpu_dgemm_rate(cb, a, b, c, n, 3, threads)
        line["cpu_baseline"] = {"value": rate, "unit": "TFLOP/s", "cores": threads,
                                "kind": "reference",
                                "sample": f"CPU BLAS dgemm_ NN n={n}: median of 3 calls after 1 "
                                          f"warm-up ({cb.config})"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    dev.close()


def bench_ozaki(args, dev, orc, a, b, c, da, db, dc0, n, stream):
    import torch
    dc = dc0.clone()
    used = dev.dgemm_ozaki("N", "N", n, n, n, 1.0, da, n, db, n, 0.5, dc, n)
    for _ in range(max(0, args.warmup - 1)):
        dev.dgemm_ozaki("N", "N", n, n, n, 1.0, da, n, db, n, 0.5, dc, n)
    dev.sync()
    dev.enable_timing(True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        dev.dgemm_ozaki("N", "N", n, n, n, 1.0, da, n, db, n, 0.5, dc, n)
    ev1.record(stream)
    ev1.synchronize()
    t = ev0.elapsed_time(ev1) / 1e3
    mma_ms, mma_n = dev.kernel_time(dev.TIMER_OZAKI_MMA)
    dev.enable_timing(False)
    # accuracy on one fresh call, sampled against the double-double oracle
    dc = dc0.clone()
    dev.dgemm_ozaki("N", "N", n, n, n, 1.0, da, n, db, n, 0.5, dc, n)
    dev.sync()
    got = dc.cpu().numpy().reshape(n, n, order="F")
    rng = np.random.default_rng(0)
    rows = rng.integers(0, n, 2048)
    cols = rng.integers(0, n, 2048)
    ref = orc.dgemm_dd_sample("N", "N", n, 1.0, a, b, 0.5, c, rows, cols)
    err = float(np.linalg.norm(got[rows, cols] - ref) / np.linalg.norm(ref))
    flops = 2.0 * n ** 3
    return {"value": flops * args.steps / t / 1e12, "unit": "TFLOP/s",
            "ms_per_step": t / args.steps * 1e3, "slices": used, "rel_err_fro_sampled": err,
            "mma_ms_per_call": mma_ms / max(mma_n, 1)}


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
