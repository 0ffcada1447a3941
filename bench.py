#!/usr/bin/env python
"""Benchmarks of libgbxblas on one GB300 (one JSON line per run).

Default workload (the headline): DGEMM 'N','N', M = N = K = 8192,
column-major, lda = ldb = ldc = 8192, alpha = 1, beta = 0.5, A, B, C uniform
[-1,1] from SplitMix64 seed 1 -- the plain FP64 drop-in sweep's DGEMM at
n = 8192.  One step = one DGEMM call.  Operands (3 x 512 MiB) exceed the
129 MB L2, so no flush is needed between steps.

  value    TFLOP/s (2 n^3 per step), operands resident in HBM, CUDA events on
           the library's stream, device C ABI (gbx_dgemm)
  e2e      the same metric through the drop-in Fortran symbol dgemm_ on
           pinned host buffers: A, B, C host->device and C device->host in
           every step
  ozaki    the opt-in Ozaki split-precision DGEMM on the same operands:
           TFLOP/s counted as 2 n^3, relative Frobenius error against the
           double-double oracle on sampled entries, slices used
  roofline dominant kernel (DFMA GEMM core) against the FP64 FMA rate
           measured in the same run
  cpu_baseline  the CPU BLAS the reference falls back to, on this host

Other workloads (--workload), each from the plain FP64 sweep or the Ozaki
configuration: ozaki (Ozaki DGEMM as the value, roofline against the FP8
tensor peak), daxpy / ddot / dnrm2 / idamax (n = 2^28), dgemv (16384^2,
'N' or 'T'), dtrsm (left/lower/N/non-unit 8192 with 1024 right-hand sides),
dsyrk (lower, n = 8192, k = 2048).  Level-1/2 report GB/s of algorithmic
traffic against the measured HBM copy bandwidth.

--impl reference times the CPU BLAS alone on the same workload (the
reference's runnable path ends there: dlsym(RTLD_NEXT) to the CPU BLAS).

Multi-GPU: calls are independent, so N > 1 runs N replicas (one per rank,
no collective on the data path); value = all ranks' work / max time.
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
# The serving workload keeps 16 slot streams busy at once; with the default 8
# hardware work queues, streams would share queues and falsely serialise.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

import numpy as np  # noqa: E402

CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
WORKLOADS = ("dgemm", "ozaki", "daxpy", "ddot", "dnrm2", "idamax", "dgemv", "dtrsm", "dsyrk",
             "batched", "serving", "ozaki_sweep", "pipes")


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", choices=WORKLOADS, default="dgemm")
    p.add_argument("--n", type=int, default=0, help="problem size (0: the workload's default)")
    p.add_argument("--m", type=int, default=0, help="dgemm/ozaki: rows of C (0: n)")
    p.add_argument("--k", type=int, default=0, help="dgemm/ozaki: inner dimension (0: n)")
    p.add_argument("--trans", default="N", help="dgemv transposition")
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-ozaki", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-sweep", action="store_true",
                   help="dgemm: skip the rest of the FP64 sweep and the Ozaki spreads")
    p.add_argument("--no-open-loop", action="store_true", help="serving: skip the Poisson-arrival sweep")
    return p.parse_args()


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return d, "MEASURED_PEAKS.json"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback (6.8 TB/s, 1.9 PFLOP/s bf16)"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region.

    Sampling runs every 200 ms.  A timed region shorter than that (the
    Level-1 kernels run for milliseconds) is bracketed instead: entering
    waits for the first sample, leaving waits for one sample taken after the
    region ended, so every line carries at least two samples."""

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def _wait_lines(self, count, timeout):
        t_end = time.time() + timeout
        while len(self.lines) < count and time.time() < t_end and self.proc.poll() is None:
            time.sleep(0.01)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={CLOCK_FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            self._wait_lines(1, 5.0)
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self._wait_lines(len(self.lines) + 1, 1.0)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
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
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
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


# --------------------------------------------------------------------------
# workload definitions
# --------------------------------------------------------------------------
class Work:
    """Inputs, a device step, a Fortran-ABI step and the CPU-BLAS step."""

    def __init__(self, args):
        import oracle
        self.orc = oracle.get()
        self.args = args
        self.kind = args.workload
        w = self.kind
        seed = args.seed
        o = self.orc
        if w in ("dgemm", "ozaki"):
            n = args.n or 8192
            m, k = args.m or n, args.k or n
            self.n, self.m, self.k = n, m, k
            self.a, s = o.matrix(m, k, seed)
            self.b, s = o.matrix(k, n, s)
            self.c, s = o.matrix(m, n, s)
            self.units, self.unit, self.metric = 2.0 * m * n * k / 1e12, "TFLOP/s", f"{w}_tflops"
            self.config = {"workload": f"{w}_NN_m{m}_n{n}_k{k}", "m": m, "n": n, "k": k, "lda": m,
                           "alpha": 1.0, "beta": 0.5}
        elif w in ("daxpy", "ddot", "dnrm2", "idamax"):
            n = args.n or (1 << 28)
            self.n = n
            self.x, s = o.uniform(n, seed)
            self.y, _ = o.uniform(n, s) if w in ("daxpy", "ddot") else (None, s)
            nbytes = {"daxpy": 24, "ddot": 16, "dnrm2": 8, "idamax": 8}[w] * n
            self.units, self.unit, self.metric = nbytes / 1e9, "GB/s", f"{w}_gbs"
            self.config = {"workload": f"{w}_n{n}", "n": n, "incx": 1, "incy": 1,
                           "bytes_per_step": nbytes}
        elif w == "dgemv":
            n = args.n or 16384
            self.n = n
            self.trans = args.trans.upper()
            self.a, s = o.matrix(n, n, seed)
            self.x, s = o.uniform(n, s)
            self.y, _ = o.uniform(n, s)
            nbytes = 8 * (n * n + n + 2 * n)
            self.units, self.unit, self.metric = nbytes / 1e9, "GB/s", "dgemv_gbs"
            self.config = {"workload": f"dgemv_{self.trans}_m{n}_n{n}", "m": n, "n": n,
                           "alpha": 1.0, "beta": 0.5, "bytes_per_step": nbytes}
        elif w == "dtrsm":
            m = args.n or 8192
            nrhs = 1024
            self.m, self.nrhs = m, nrhs
            self.a, s = o.trsm_matrix(m, seed)
            self.b, _ = o.matrix(m, nrhs, s)
            self.units, self.unit, self.metric = float(m) * m * nrhs / 1e12, "TFLOP/s", "dtrsm_tflops"
            self.config = {"workload": f"dtrsm_LLNN_m{m}_n{nrhs}", "side": "L", "uplo": "L",
                           "transa": "N", "diag": "N", "m": m, "n": nrhs, "alpha": 1.0}
        elif w == "dsyrk":
            n = args.n or 8192
            k = 2048
            self.n, self.k = n, k
            self.a, s = o.matrix(n, k, seed)
            self.c, _ = o.matrix(n, n, s)
            self.units, self.unit, self.metric = float(n) * (n + 1) * k / 1e12, "TFLOP/s", "dsyrk_tflops"
            self.config = {"workload": f"dsyrk_LN_n{n}_k{k}", "uplo": "L", "trans": "N", "n": n,
                           "k": k, "alpha": 1.0, "beta": 0.5}
        self.config["inputs"] = f"uniform[-1,1] SplitMix64 seed {seed}" + (
            "; A diag uniform[1,2], off-diagonal uniform[-1,1]/m" if w == "dtrsm" else "")
        self.config["l2"] = "operands larger than the 129 MB L2; no flush needed"

    # ---- device-resident step (gbx_* C ABI) -----------------------------
    def to_device(self):
        import torch

        def d(a):
            return None if a is None else torch.from_numpy(np.asarray(a).ravel(order="F")).cuda()
        self.d = {k: d(getattr(self, k, None)) for k in ("a", "b", "c", "x", "y")}
        self.d["res"] = torch.zeros(2, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()

    def timer_tag(self, dev):
        return {"dgemm": dev.TIMER_GEMM_FP64, "ozaki": dev.TIMER_OZAKI_MMA,
                "dtrsm": dev.TIMER_GEMM_FP64, "dsyrk": dev.TIMER_GEMM_FP64,
                "dgemv": dev.TIMER_GEMV}.get(self.kind, dev.TIMER_LEVEL1)

    def device_step(self, dev):
        d, w = self.d, self.kind
        if w == "dgemm":
            m, n, k = self.m, self.n, self.k
            dev.dgemm_checked("N", "N", m, n, k, 1.0, d["a"], m, d["b"], k, 0.5, d["c"], m)
        elif w == "ozaki":
            m, n, k = self.m, self.n, self.k
            # asynchronous like a C caller's: no slice-count read-back per call
            dev.dgemm_ozaki("N", "N", m, n, k, 1.0, d["a"], m, d["b"], k, 0.5, d["c"], m,
                            want_slices=False)
        elif w == "daxpy":
            dev.daxpy(self.n, 0.5, d["x"], 1, d["y"], 1)
        elif w == "ddot":
            dev.ddot(self.n, d["x"], 1, d["y"], 1, d["res"])
        elif w == "dnrm2":
            dev.dnrm2(self.n, d["x"], 1, d["res"])
        elif w == "idamax":
            dev.idamax(self.n, d["x"], 1, d["res"])
        elif w == "dgemv":
            n = self.n
            dev.dgemv(self.trans, n, n, 1.0, d["a"], n, d["x"], 1, 0.5, d["y"], 1)
        elif w == "dtrsm":
            dev.dtrsm("L", "L", "N", "N", self.m, self.nrhs, 1.0, d["a"], self.m, d["b"], self.m)
        elif w == "dsyrk":
            dev.dsyrk("L", "N", self.n, self.k, 1.0, d["a"], self.n, 0.5, d["c"], self.n)

    # ---- end to end through the Fortran symbols on pinned host memory ----
    def to_pinned(self):
        import torch

        def pin(a):
            return None if a is None else torch.from_numpy(np.asarray(a).ravel(order="F")).pin_memory()
        self.h = {k: pin(getattr(self, k, None)) for k in ("a", "b", "c", "x", "y")}
        self.hp = {k: (v.data_ptr() if v is not None else None) for k, v in self.h.items()}

    def f77_step(self, f):
        p, w = self.hp, self.kind
        if w in ("dgemm", "ozaki"):
            m, n, k = self.m, self.n, self.k
            f.dgemm("N", "N", m, n, k, 1.0, p["a"], m, p["b"], k, 0.5, p["c"], m)
        elif w == "daxpy":
            f.daxpy(self.n, 0.5, p["x"], 1, p["y"], 1)
        elif w == "ddot":
            f.ddot(self.n, p["x"], 1, p["y"], 1)
        elif w == "dnrm2":
            f.dnrm2(self.n, p["x"], 1)
        elif w == "idamax":
            f.idamax(self.n, p["x"], 1)
        elif w == "dgemv":
            n = self.n
            f.dgemv(self.trans, n, n, 1.0, p["a"], n, p["x"], 1, 0.5, p["y"], 1)
        elif w == "dtrsm":
            f.dtrsm("L", "L", "N", "N", self.m, self.nrhs, 1.0, p["a"], self.m, p["b"], self.m)
        elif w == "dsyrk":
            f.dsyrk("L", "N", self.n, self.k, 1.0, p["a"], self.n, 0.5, p["c"], self.n)

    # ---- CPU BLAS step -----------------------------------------------------
    def cpu_prepare(self):
        self.cc = {k: (np.asarray(getattr(self, k)).copy(order="F") if getattr(self, k, None) is not None
                       else None) for k in ("a", "b", "c", "x", "y")}

    def cpu_step(self, cb):
        c, w = self.cc, self.kind
        if w in ("dgemm", "ozaki"):
            cb.dgemm("N", "N", self.m, self.n, self.k, 1.0, c["a"], c["b"], 0.5, c["c"])
        elif w == "daxpy":
            cb.daxpy(self.n, 0.5, c["x"], 1, c["y"], 1)
        elif w == "ddot":
            cb.ddot(self.n, c["x"], 1, c["y"], 1)
        elif w == "dnrm2":
            cb.dnrm2(self.n, c["x"], 1)
        elif w == "idamax":
            cb.idamax(self.n, c["x"], 1)
        elif w == "dgemv":
            cb.dgemv(self.trans, self.n, self.n, 1.0, c["a"], c["x"], 1, 0.5, c["y"], 1)
        elif w == "dtrsm":
            cb.dtrsm("L", "L", "N", "N", self.m, self.nrhs, 1.0, c["a"], c["b"])
        elif w == "dsyrk":
            cb.dsyrk("L", "N", self.n, self.k, 1.0, c["a"], 0.5, c["c"])


def common_line(args, work, ws, value, ms_per_step):
    return {"metric": work.metric, "value": value, "unit": work.unit, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": dict(work.config,
                                                parallelism="replicas" if ws > 1 else "single-gpu")}


def cpu_rate(work, cb, threads, target_s=12.0, max_reps=5):
    """Median rate of the CPU BLAS on the workload: 1 warm-up, then up to
    max_reps calls bounded by ~target_s seconds of CPU work."""
    cb.set_threads(threads)
    work.cpu_prepare()
    t0 = time.perf_counter()
    work.cpu_step(cb)
    first = time.perf_counter() - t0
    reps = int(max(1, min(max_reps, target_s / max(first, 1e-6))))
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        work.cpu_step(cb)
        times.append(time.perf_counter() - t0)
    return work.units / statistics.median(times), reps


def run_reference(args):
    ws, rank, local = dist_setup(args)
    if rank != 0:
        barrier(ws)
        return
    from oracle import cpublas
    cb = cpublas.get()
    threads = os.cpu_count() or 1
    work = Work(args)
    cb.set_threads(threads)
    work.cpu_prepare()
    for _ in range(args.warmup):
        work.cpu_step(cb)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        work.cpu_step(cb)
    dt = time.perf_counter() - t0
    value = work.units * args.steps / dt
    line = common_line(args, work, ws, value, dt / args.steps * 1e3)
    line["impl"] = "reference"
    line["cpu_baseline"] = {"value": value, "unit": work.unit, "cores": threads, "kind": "reference",
                            "sample": f"CPU BLAS ({cb.config}) on the full workload, {args.steps} "
                                      f"timed calls after {args.warmup} warm-up"}
    line["e2e"] = {"value": value, "unit": work.unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    print(json.dumps(line), flush=True)
    barrier(ws)


def traffic_from_profiles(key):
    """Per-launch DRAM bytes of a kernel from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
            return json.load(fh).get(key)
    except (OSError, ValueError):
        return None


def run_ours(args):
    import torch
    ws, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    import libgpublas_gb300 as g
    from libgpublas_gb300 import build
    build.build_library()
    work = Work(args)
    work.to_device()
    dev = g.Device(local)
    stream = torch.cuda.ExternalStream(dev.stream())
    peaks, peak_src = measured_peaks()

    for _ in range(args.warmup):
        work.device_step(dev)
    dev.sync()
    dev.enable_timing(True)
    l0 = dev.launches()
    barrier(ws)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            work.device_step(dev)
        ev1.record(stream)
        ev1.synchronize()
    dev.sync()
    barrier(ws)
    launches = dev.launches() - l0
    t = ev0.elapsed_time(ev1) / 1e3
    t_max = max_over_ranks(ws, t, device="cuda")
    value = work.units * args.steps * ws / t_max
    k_ms, k_n = dev.kernel_time(work.timer_tag(dev))
    dev.enable_timing(False)
    per_launch_s = (k_ms / max(k_n, 1)) / 1e3
    line = common_line(args, work, ws, value, t_max / args.steps * 1e3)
    line["gpu_launches"] = int(launches)
    line["clocks"] = clk.summary()

    w = work.kind
    if w in ("dgemm", "dtrsm", "dsyrk"):
        peak = dev.fp64_peak()
        # DGEMM and DSYRK are one launch per call.  DTRSM is hundreds of
        # launches (GEMM updates, leaf solves, the block inversion), more than
        # the timer keeps, so its achieved rate is the whole call's rate.
        if w == "dtrsm":
            achieved = value / ws
        else:
            achieved = work.units * args.steps / (k_ms / 1e3) if k_ms > 0 else None
        line["roofline"] = {"bound": "fp64", "kernel": "gemm_simt_kernel<double,4,4,8>",
                            "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                            "frac": achieved / peak if (achieved and peak) else None,
                            "peak_source": "measured in this run: DFMA throughput loop "
                                           "(gbx_diag_fp64_peak); MEASURED_PEAKS.json has no "
                                           "FP64 figure",
                            "traffic": traffic_from_profiles(f"{w}_{work.config['workload']}"),
                            "kernel_launches_timed": int(k_n)}
    elif w == "ozaki":
        d = work.d
        # the slice count of this workload (one more call, outside the timed region)
        s = dev.dgemm_ozaki("N", "N", work.m, work.n, work.k, 1.0, d["a"], work.m, d["b"], work.k, 0.5,
                            d["c"], work.m)
        raw = s * (s + 1) / 2 * work.units   # FP8 tensor TFLOP per step
        peak = 2.0 * peaks.get("bf16_tflops", 1900.0)
        achieved = raw / per_launch_s if per_launch_s > 0 else None
        kname = "oz_gemm_sk_kernel" if work.k <= 1024 else "oz_gemm_kernel"
        line["roofline"] = {"bound": "tensor", "kernel": f"{kname} (tcgen05 kind::f8f6f4)",
                            "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                            "frac": achieved / peak if achieved else None,
                            "peak_source": f"2 x bf16_tflops of {peak_src} (FP8 dense = 2x bf16 "
                                           "dense on this part)",
                            "traffic": traffic_from_profiles(f"ozaki_{work.config['workload']}"),
                            "algorithmic": "S(S+1)/2 * 2 n^3 FP8 flop per launch",
                            "slices": s}
    else:
        peak = peaks.get("hbm_gbs", 6800.0)
        achieved = work.units / per_launch_s if per_launch_s > 0 else None
        line["roofline"] = {"bound": "hbm", "kernel": {"dgemv": "gemv_n_partial/gemv_t_warp"}.get(
                                w, f"{w} streaming kernel"),
                            "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak if achieved else None,
                            "peak_source": f"hbm_gbs of {peak_src}",
                            "traffic": traffic_from_profiles(f"{w}_{work.config['workload']}"),
                            "algorithmic": f"{work.config.get('bytes_per_step')} bytes per launch"}

    # ---- end to end through the Fortran symbol on pinned host buffers ----
    if not args.no_e2e:
        work.to_pinned()
        f = g.F77()
        if w == "ozaki" and "precision=ozaki" not in os.environ.get("BLAS2CUDA_OPTIONS", ""):
            # dgemm_ takes the Ozaki path only when the process starts with
            # BLAS2CUDA_OPTIONS=precision=ozaki (read once, as in the
            # reference): measure it in a child process started that way
            line["e2e"] = ozaki_e2e_child(args)
        else:
            work.f77_step(f)
            # the Fortran symbols run on this thread's own context: its
            # event timers split each step into copies in, kernel, copy out
            tctx = g.Device.of_thread()
            tctx.enable_timing(True)
            s0 = g.stats()
            barrier(ws)
            with ClockSampler(local) as eclk:
                t0 = time.perf_counter()
                for _ in range(args.steps):
                    work.f77_step(f)
                te = max_over_ranks(ws, time.perf_counter() - t0, device="cuda")
            s1 = g.stats()
            phases = {}
            for name, tag in (("h2d_ms", tctx.TIMER_H2D), ("kernel_ms", work.timer_tag(tctx)),
                              ("d2h_ms", tctx.TIMER_D2H)):
                ms, cnt = tctx.kernel_time(tag)
                phases[name] = ms / args.steps if cnt else None
            tctx.enable_timing(False)
            phases["wall_ms"] = te / args.steps * 1e3
            if phases.get("kernel_ms"):
                # host time not covered by the products: copies that did not
                # overlap them, plus call overhead
                phases["exposed_ms"] = phases["wall_ms"] - phases["kernel_ms"]
            line["e2e"] = {"value": work.units * args.steps * ws / te, "unit": work.unit,
                           "h2d_bytes_per_step": (s1["bytes_h2d"] - s0["bytes_h2d"]) // args.steps,
                           "d2h_bytes_per_step": (s1["bytes_d2h"] - s0["bytes_d2h"]) // args.steps,
                           "api": "Fortran ABI symbol, pinned host operands",
                           "per_step": phases, "clocks": eclk.summary()}

    if w == "dgemm":
        line["accuracy"] = plain_accuracy(dev, work)
    if w == "dgemm" and not args.no_ozaki:
        try:
            line["ozaki"] = bench_ozaki(args, dev, work, stream)
            if not args.no_e2e and ws == 1:
                line["ozaki"]["e2e"] = ozaki_e2e_child(args)
        except g.GbxError as e:
            line["ozaki"] = {"unavailable": str(e)}
    if w == "ozaki":
        line["ozaki_accuracy"] = ozaki_accuracy(dev, work)
    if w == "dgemm" and not args.no_sweep and ws == 1:
        del work.d
        import torch
        torch.cuda.empty_cache()
        fp64_peak = line["roofline"]["peak"]
        line["sweep"] = run_sweep(dev, stream, work.orc, fp64_peak, peaks.get("hbm_gbs", 6800.0),
                                  2.0 * peaks.get("bf16_tflops", 1900.0), log=sys.stderr)
        line["sweep_peaks"] = {"fp64_tflops": fp64_peak, "hbm_gbs": peaks.get("hbm_gbs"),
                               "tensor_fp8_tflops": 2.0 * peaks.get("bf16_tflops", 1900.0),
                               "source": f"FP64: measured in this run; HBM and bf16: {peak_src}"}

    if w == "dgemm" and not args.no_sweep and ws == 1:
        # the serving trace, shortened (16 threads, n in [1024, 4096]): the
        # loop against plain per-call dispatch in the same precision
        sizes, nbs, modes = serving_trace(g, 16, 1024, 4096)
        line["serving"] = {
            "workload": "cholesky_trace_16threads_n1024-4096",
            "n": sizes, "nb": nbs,
            "modes": {m: {k: v[k] for k in ("calls", "calls_per_s", "p50_us", "p99_us", "tflops",
                                            "residual_sampled", "wall_s", "first_error", "chains")}
                      for m, v in modes.items()},
            "ratios": serving_ratios(modes, line["roofline"]["peak"]),
            # latency-bound FP64 calls (DGEMM 64^3), 1 and 16 caller threads
            "small_calls": {"dgemm_64_threads1": small_call_trace(g, 1, 2000),
                            "dgemm_64_threads16": small_call_trace(g, 16, 500)}}
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        from oracle import cpublas
        cb = cpublas.get()
        threads = os.cpu_count() or 1
        rate, reps = cpu_rate(work, cb, threads)
        line["cpu_baseline"] = {"value": rate, "unit": work.unit, "cores": threads,
                                "kind": "reference",
                                "sample": f"CPU BLAS ({cb.config}) on the full workload: median of "
                                          f"{reps} calls after 1 warm-up"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    dev.close()


def sample_indices(m, n, count, seed):
    """count random (row, col) pairs plus 64 on the last row and 64 on the
    last column (the edge tiles)."""
    rng = np.random.default_rng(seed)
    rows = np.concatenate([rng.integers(0, m, count), np.full(64, m - 1), rng.integers(0, m, 64)])
    cols = np.concatenate([rng.integers(0, n, count), rng.integers(0, n, 64), np.full(64, n - 1)])
    return rows, cols


def plain_accuracy(dev, work, ta="N"):
    """The benchmarked kernel checks its own result: one fresh FP64 DGEMM
    of the workload (same operands, C restored), sampled entries against the
    double-double oracle.  Tolerance of the FP64 routines: 1e-13."""
    import torch
    m, n, k = work.m, work.n, work.k
    dc = torch.from_numpy(work.c.ravel(order="F")).cuda()
    lda = m if ta == "N" else k
    dev.dgemm_checked(ta, "N", m, n, k, 1.0, work.d["a"], lda, work.d["b"], k, 0.5, dc, m)
    dev.sync()
    got = dc.view(n, m)   # column j is row j of this view
    rows, cols = sample_indices(m, n, 2048, 1)
    vals = got[torch.from_numpy(cols).cuda(), torch.from_numpy(rows).cuda()].cpu().numpy()
    ref = work.orc.dgemm_dd_sample(ta, "N", k, 1.0, work.a, work.b, 0.5, work.c, rows, cols)
    err = float(np.linalg.norm(vals - ref) / np.linalg.norm(ref))
    del dc
    return {"rel_err_fro_sampled": err, "samples": int(len(rows)), "tol": 1e-13,
            "ok": bool(err <= 1e-13), "oracle": "double-double dot products of the sampled entries"}


# --------------------------------------------------------------------------
# the rest of the plain FP64 sweep and of the Ozaki configuration, reported
# beside the headline: DGEMM n in {1024, 4096, 8192, 16384} NN and TN, DSYRK
# lower n = 8192 k = 2048, DTRSM LLNN 8192 with 1024 right-hand sides, DGEMV
# 16384^2 N and T, DAXPY / DDOT / DNRM2 / IDAMAX at n = 2^28, Ozaki DGEMM 8192
# at spreads 8 and 24.  Every entry is device-resident, timed with CUDA
# events on the library's stream, carries its roofline fraction and checks
# its own output against the oracle.
# --------------------------------------------------------------------------
def _timed(stream, fn, steps):
    import torch
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        fn()
    ev1.record(stream)
    ev1.synchronize()
    return ev0.elapsed_time(ev1) / 1e3 / steps


def _measure(dev, stream, call, est_s, budget_s=0.6, hi=20):
    """Time call(): one warm-up call unless a call is estimated to take more
    than 2 s (the kernel is warm from earlier entries then), then enough
    calls for about budget_s.  Returns (seconds per call, timed calls,
    calls made in all)."""
    warm = est_s <= 2.0
    if warm:
        call()
        dev.sync()
    steps = int(max(1, min(hi, budget_s / max(est_s, 1e-6))))
    return _timed(stream, call, steps), steps, steps + int(warm)


def run_sweep(dev, stream, orc, fp64_peak, hbm_peak, tc_peak, seed=1, log=None):
    import torch
    out = []

    def dd(a):
        return torch.from_numpy(np.asarray(a).ravel(order="F")).cuda()

    def note(e):
        out.append(e)
        if log:
            print(json.dumps(e), file=log, flush=True)

    def rel(x, r):
        return float(np.linalg.norm(np.asarray(x) - r) / np.linalg.norm(r))

    # ---- DGEMM, both transposition forms, C := A op(B) + 0.5 C repeated:
    # after s calls C = (2 - 2^(1-s)) op(A) B + 2^-s C0, checked on samples
    for n in (1024, 4096, 8192, 16384):
        a, st = orc.matrix(n, n, seed)
        b, st = orc.matrix(n, n, st)
        c, st = orc.matrix(n, n, st)
        A, B = dd(a), dd(b)
        for ta in ("N", "T"):
            if n == 8192 and ta == "N":
                continue                      # the headline line itself
            C = dd(c)
            call = lambda: dev.dgemm_checked(ta, "N", n, n, n, 1.0, A, n, B, n, 0.5, C, n)  # noqa: E731
            t, steps, s_total = _measure(dev, stream, call, 2.0 * n ** 3 / (fp64_peak * 1e12))
            rows, cols = sample_indices(n, n, 512, n)
            got = C.view(n, n)[torch.from_numpy(cols).cuda(), torch.from_numpy(rows).cuda()].cpu().numpy()
            ref = orc.dgemm_dd_sample(ta, "N", n, 2.0 - 2.0 ** (1 - s_total), a, b, 0.5 ** s_total, c, rows, cols)
            tf = 2.0 * n ** 3 / t / 1e12
            note({"routine": "dgemm", "trans": ta + "N", "m": n, "n": n, "k": n, "tflops": tf, "ms": t * 1e3,
                  "steps": steps, "frac_fp64": tf / fp64_peak, "rel_err_sampled": rel(got, ref)})
            del C
        del A, B, a, b, c
        torch.cuda.empty_cache()

    # ---- DSYRK lower, n = 8192, k = 2048 (alpha 1, beta 0.5, repeated)
    n, k = 8192, 2048
    a, st = orc.matrix(n, k, seed)
    c, st = orc.matrix(n, n, st)
    A, C = dd(a), dd(c)
    call = lambda: dev.dsyrk("L", "N", n, k, 1.0, A, n, 0.5, C, n)  # noqa: E731
    t, steps, s_total = _measure(dev, stream, call, float(n) * (n + 1) * k / (fp64_peak * 1e12))
    rows, cols = sample_indices(n, n, 1024, 5)
    keep = rows >= cols
    rows, cols = rows[keep], cols[keep]
    got = C.view(n, n)[torch.from_numpy(cols).cuda(), torch.from_numpy(rows).cuda()].cpu().numpy()
    ref = orc.dgemm_dd_sample("N", "T", k, 2.0 - 2.0 ** (1 - s_total), a, a, 0.5 ** s_total, c, rows, cols)
    tf = float(n) * (n + 1) * k / t / 1e12
    note({"routine": "dsyrk", "uplo": "L", "trans": "N", "n": n, "k": k, "tflops": tf, "ms": t * 1e3,
          "steps": steps, "frac_fp64": tf / fp64_peak, "rel_err_sampled": rel(got, ref)})
    del A, C, a, c

    # ---- DTRSM LLNN, 8192 x 8192 triangle, 1024 right-hand sides
    m, nrhs = 8192, 1024
    a, st = orc.trsm_matrix(m, seed)
    b, st = orc.matrix(m, nrhs, st)
    A, B0 = dd(a), dd(b)
    B = B0.clone()
    call = lambda: dev.dtrsm("L", "L", "N", "N", m, nrhs, 1.0, A, m, B, m)  # noqa: E731
    t, steps, _ = _measure(dev, stream, call, float(m) * m * nrhs / (fp64_peak * 1e12), hi=10)
    B.copy_(B0)
    torch.cuda.synchronize()      # torch's stream does not order with the library's
    call()
    dev.sync()
    cols = np.array([0, 377, 801, nrhs - 1])
    xs = B.view(nrhs, m)[torch.from_numpy(cols).cuda()].cpu().numpy().T.copy(order="F")
    want = np.asfortranarray(b[:, cols])
    orc.dtrsm("L", "L", "N", "N", m, len(cols), 1.0, a, want)
    tf = float(m) * m * nrhs / t / 1e12
    note({"routine": "dtrsm", "side": "L", "uplo": "L", "trans": "N", "diag": "N", "m": m, "n": nrhs,
          "tflops": tf, "ms": t * 1e3, "steps": steps, "frac_fp64": tf / fp64_peak,
          "rel_err_sampled": rel(xs, want), "checked": "4 solution columns against the oracle's substitution"})
    del A, B, B0, a, b
    torch.cuda.empty_cache()

    # ---- DGEMV 16384^2, N and T (y := A x + 0.5 y repeated)
    n = 16384
    a, st = orc.matrix(n, n, seed)
    x, st = orc.uniform(n, st)
    y, st = orc.uniform(n, st)
    A, X = dd(a), dd(x)
    for tr in ("N", "T"):
        Y = dd(y)
        call = lambda: dev.dgemv(tr, n, n, 1.0, A, n, X, 1, 0.5, Y, 1)  # noqa: E731
        t, steps, s_total = _measure(dev, stream, call, 8.0 * n * n / (hbm_peak * 1e9), budget_s=0.3)
        rows = np.random.default_rng(7).integers(0, n, 256)
        got = Y.cpu().numpy()[rows]
        ref = orc.dgemm_dd_sample(tr, "N", n, 2.0 - 2.0 ** (1 - s_total), a, x.reshape(n, 1, order="F"),
                                  0.5 ** s_total, y.reshape(n, 1, order="F"), rows, np.zeros_like(rows))
        gbs = 8.0 * (n * n + n + 2 * n) / t / 1e9
        note({"routine": "dgemv", "trans": tr, "m": n, "n": n, "gbs": gbs, "ms": t * 1e3, "steps": steps,
              "frac_hbm": gbs / hbm_peak, "rel_err_sampled": rel(got, ref)})
        del Y
    del A, X, a

    # ---- Level 1 at n = 2^28
    n = 1 << 28
    x, st = orc.uniform(n, seed)
    y, st = orc.uniform(n, st)
    X, Y = dd(x), dd(y)
    res = torch.zeros(2, dtype=torch.float64, device="cuda")
    for r, nbytes in (("daxpy", 24), ("ddot", 16), ("dnrm2", 8), ("idamax", 8)):
        if r == "daxpy":
            Yw = Y.clone()
            call = lambda: dev.daxpy(n, 0.5, X, 1, Yw, 1)  # noqa: E731
        elif r == "ddot":
            call = lambda: dev.ddot(n, X, 1, Y, 1, res)  # noqa: E731
        elif r == "dnrm2":
            call = lambda: dev.dnrm2(n, X, 1, res)  # noqa: E731
        else:
            call = lambda: dev.idamax(n, X, 1, res)  # noqa: E731
        t, steps, s_total = _measure(dev, stream, call, float(nbytes) * n / (hbm_peak * 1e9), budget_s=0.2)
        dev.sync()
        if r == "daxpy":
            idx = np.random.default_rng(3).integers(0, n, 4096)
            got = Yw[torch.from_numpy(idx).cuda()].cpu().numpy()
            err = rel(got, y[idx] + 0.5 * s_total * x[idx])
            del Yw
        elif r == "ddot":
            err = abs(float(res[0].item()) - orc.ddot_dd(n, x, 1, y, 1)) / float(np.abs(x) @ np.abs(y))
        elif r == "dnrm2":
            ref = orc.dnrm2(n, x, 1)
            err = abs(float(res[0].item()) - ref) / ref
        else:
            got = int(res.view(torch.int32)[0].item())
            err = 0.0 if got == orc.idamax(n, x, 1) else 1.0
        gbs = float(nbytes) * n / t / 1e9
        note({"routine": r, "n": n, "gbs": gbs, "ms": t * 1e3, "steps": steps, "frac_hbm": gbs / hbm_peak,
              ("index_mismatch" if r == "idamax" else "rel_err"): err})
    del X, Y, x, y, res
    torch.cuda.empty_cache()

    # ---- Ozaki DGEMM n = 8192 at exponent spreads 8 and 24 (tol 1e-14)
    n = 8192
    for spread in (8, 24):
        st = 1000 + n + spread
        a, st = orc.spread((n, n), spread, st)
        b, st = orc.spread((n, n), spread, st)
        A, B = dd(a), dd(b)
        C = torch.zeros(n * n, dtype=torch.float64, device="cuda")
        used = dev.dgemm_ozaki("N", "N", n, n, n, 1.0, A, n, B, n, 0.0, C, n)
        call = lambda: dev.dgemm_ozaki("N", "N", n, n, n, 1.0, A, n, B, n, 0.0, C, n,  # noqa: E731
                                       want_slices=False)
        t, steps, _ = _measure(dev, stream, call, 0.03, budget_s=0.3)
        rows, cols = sample_indices(n, n, 512, spread)
        got = C.view(n, n)[torch.from_numpy(cols).cuda(), torch.from_numpy(rows).cuda()].cpu().numpy()
        ref = orc.dgemm_dd_sample("N", "N", n, 1.0, a, b, 0.0, np.zeros((1, 1), order="F"), rows, cols)
        tf = 2.0 * n ** 3 / t / 1e12
        raw = used * (used + 1) / 2 * 2.0 * n ** 3 / t / 1e12
        note({"routine": "dgemm_ozaki", "spread": spread, "m": n, "n": n, "k": n, "slices": used,
              "tflops": tf, "ms": t * 1e3, "steps": steps, "vs_plain_fp64": tf / fp64_peak,
              "frac_tensor": raw / tc_peak, "rel_err_sampled": rel(got, ref)})
        del A, B, C, a, b
        torch.cuda.empty_cache()
    return out


def ozaki_accuracy(dev, work):
    """Relative Frobenius error of one fresh Ozaki call against the
    double-double oracle on 2048 sampled entries."""
    import torch
    m, n, k = work.m, work.n, work.k
    dc = torch.from_numpy(work.c.ravel(order="F")).cuda()
    used = dev.dgemm_ozaki("N", "N", m, n, k, 1.0, work.d["a"], m, work.d["b"], k, 0.5, dc, m)
    got = dc.cpu().numpy().reshape(m, n, order="F")
    rng = np.random.default_rng(0)
    rows = rng.integers(0, m, 2048)
    cols = rng.integers(0, n, 2048)
    ref = work.orc.dgemm_dd_sample("N", "N", k, 1.0, work.a, work.b, 0.5, work.c, rows, cols)
    err = float(np.linalg.norm(got[rows, cols] - ref) / np.linalg.norm(ref))
    return {"rel_err_fro_sampled": err, "slices": used, "samples": 2048, "tol": 1e-14}


def ozaki_e2e_child(args):
    """The Ozaki product end to end through dgemm_ on pinned host operands:
    a child `bench.py --workload ozaki` started with
    BLAS2CUDA_OPTIONS=precision=ozaki, whose e2e object is returned."""
    import subprocess
    n = args.n or 8192
    cmd = [sys.executable, os.path.abspath(__file__), "--workload", "ozaki", "--n", str(n),
           "--steps", str(max(args.steps, 5)), "--warmup", str(max(args.warmup, 3)), "--no-cpu-baseline"]
    if args.m:
        cmd += ["--m", str(args.m)]
    if args.k:
        cmd += ["--k", str(args.k)]
    env = dict(os.environ, BLAS2CUDA_OPTIONS="precision=ozaki")
    for k in ("RANK", "LOCAL_RANK", "WORLD_SIZE", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    try:
        r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=600)
        lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
        if r.returncode != 0 or not lines:
            return {"unavailable": f"child exited {r.returncode}: {r.stderr.strip()[-300:]}"}
        e2e = json.loads(lines[-1]).get("e2e") or {}
        e2e["api"] = "dgemm_ with BLAS2CUDA_OPTIONS=precision=ozaki, pinned host operands"
        return e2e
    except subprocess.TimeoutExpired:
        return {"unavailable": "child timed out"}


def bench_ozaki(args, dev, work, stream):
    import torch
    m, n, k = work.m, work.n, work.k
    d = work.d
    for _ in range(max(1, args.warmup - 1)):
        dev.dgemm_ozaki("N", "N", m, n, k, 1.0, d["a"], m, d["b"], k, 0.5, d["c"], m)
    dev.sync()
    dev.enable_timing(True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        dev.dgemm_ozaki("N", "N", m, n, k, 1.0, d["a"], m, d["b"], k, 0.5, d["c"], m)
    ev1.record(stream)
    ev1.synchronize()
    t = ev0.elapsed_time(ev1) / 1e3
    mma_ms, mma_n = dev.kernel_time(dev.TIMER_OZAKI_MMA)
    dev.enable_timing(False)
    acc = ozaki_accuracy(dev, work)
    return {"value": work.units * args.steps / t, "unit": "TFLOP/s",
            "ms_per_step": t / args.steps * 1e3, "slices": acc["slices"],
            "rel_err_fro_sampled": acc["rel_err_fro_sampled"],
            "mma_ms_per_call": mma_ms / max(mma_n, 1)}


# --------------------------------------------------------------------------
# grouped execution: 20,000 DGEMM (M, N, K log-uniform in [8, 512], seed 3)
# interleaved with 5,000 DTRSM (order log-uniform in [8, 256], diagonal
# uniform[1,2], 16 right-hand sides); one persistent grouped kernel replayed
# from a CUDA graph, against one launch per call
# --------------------------------------------------------------------------
def loguni(rng, lo, hi, size):
    return np.rint(np.exp(rng.uniform(np.log(lo), np.log(hi), size))).astype(np.int64)


def build_batched(ngemm, ntrsm, seed, device_buffer_factory):
    import libgpublas_gb300 as g
    rng = np.random.default_rng(seed)
    mnk = loguni(rng, 8, 512, (ngemm, 3))
    orders = loguni(rng, 8, 256, ntrsm)
    sizes = [int(m * k + k * n + m * n) for m, n, k in mnk] + [int(o * o + 16 * o) for o in orders]
    padded = [s + (-s % 4) for s in sizes]
    total = int(sum(padded))
    buf = device_buffer_factory(total)
    base = buf.data_ptr()
    ops, off, flops, gi, ti = [], 0, 0.0, 0, 0
    # interleave: four GEMMs, then one TRSM
    while gi < ngemm or ti < ntrsm:
        for _ in range(4):
            if gi < ngemm:
                m, n, k = (int(v) for v in mnk[gi])
                pa, pb, pc = base + 8 * off, base + 8 * (off + m * k), base + 8 * (off + m * k + k * n)
                ops.append(g.GbxOp(kind=1, transa=b"N", transb=b"N", m=m, n=n, k=k, alpha=1.0, beta=0.5,
                                   A=pa, lda=m, B=pb, ldb=k, C=pc, ldc=m))
                flops += 2.0 * m * n * k
                off += padded[gi]
                gi += 1
        if ti < ntrsm:
            o = int(orders[ti])
            ops.append(g.GbxOp(kind=2, transa=b"N", side=b"L", uplo=b"L", diag=b"N", m=o, n=16,
                               alpha=1.0, A=base + 8 * off, lda=o, C=base + 8 * (off + o * o), ldc=o))
            flops += float(o) * o * 16
            off += padded[ngemm + ti]
            ti += 1
    return buf, ops, flops


def fill_batched(buf, ops, seed):
    """uniform[-1,1] everywhere, then triangles get diagonal uniform[1,2]."""
    import torch
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    buf.uniform_(-1.0, 1.0, generator=gen)
    base = buf.data_ptr()
    for op in ops:
        if op.kind == 2:
            o = op.m
            start = (op.A - base) // 8
            tri = buf[start: start + o * o].view(o, o)
            tri.diagonal().uniform_(1.0, 2.0, generator=gen)
    torch.cuda.synchronize()


def run_batched(args):
    import torch
    import libgpublas_gb300 as g
    from libgpublas_gb300 import build
    build.build_library()
    ngemm = args.n or 20000
    ntrsm = ngemm // 4
    dev = g.Device(0)
    buf, ops, flops = build_batched(ngemm, ntrsm, 3,
                                    lambda n: torch.empty(n, dtype=torch.float64, device="cuda"))
    fill_batched(buf, ops, 3)
    arr = (g.GbxOp * len(ops))(*ops)
    stream = torch.cuda.ExternalStream(dev.stream())
    plan = dev.plan_create(ops)             # autotunes unseen size buckets once
    items, _ = dev.plan_info(plan)

    def timed(fn, steps):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(steps):
            fn()
        ev1.record(stream)
        ev1.synchronize()
        return ev0.elapsed_time(ev1) / 1e3 / steps

    for _ in range(args.warmup):
        dev.plan_launch(plan, graph=True)
    dev.sync()
    l0 = dev.launches()
    with ClockSampler(0) as clk:
        t_group = timed(lambda: dev.plan_launch(plan, graph=True), args.steps)
    launches = dev.launches() - l0
    dev.sync()
    dev.ops_run(arr, len(ops))              # warm the per-call path
    dev.sync()
    t_call = timed(lambda: dev.ops_run(arr, len(ops)), max(1, min(args.steps, 3)))
    dev.plan_destroy(plan)
    peak = dev.fp64_peak()
    value = flops / t_group / 1e12
    line = {"metric": "batched_tflops", "value": value, "unit": "TFLOP/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_group * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": f"grouped_{ngemm}dgemm_{ntrsm}dtrsm",
                       "gemm": "M, N, K log-uniform [8, 512], NN, alpha 1, beta 0.5",
                       "trsm": "LLNN, order log-uniform [8, 256], diag uniform[1,2], 16 rhs",
                       "inputs": "uniform[-1,1] (torch device generator, seed 3)",
                       "execution": "one persistent grouped kernel replayed from a CUDA graph",
                       "work_items": items, "flops_per_step": flops},
            "gpu_launches": int(launches), "clocks": clk.summary(),
            "calls_per_s": len(ops) / t_group,
            "per_call": {"value": flops / t_call / 1e12, "unit": "TFLOP/s",
                         "calls_per_s": len(ops) / t_call, "ms_per_step": t_call * 1e3,
                         "execution": "one launch per call through gbx_dgemm / gbx_dtrsm"},
            "speedup_vs_per_call": t_call / t_group,
            "roofline": {"bound": "fp64", "kernel": "grouped_kernel", "achieved": value,
                         "peak": peak, "unit": "TFLOP/s", "frac": value / peak,
                         "peak_source": "measured in this run (gbx_diag_fp64_peak)",
                         "traffic": None},
            "e2e": {"unavailable": "operands are device-resident by design of this workload"}}
    print(json.dumps(line), flush=True)
    dev.close()


# --------------------------------------------------------------------------
# serving trace: 16 host threads each factorise A = G G^T + n I (blocked
# right-looking Cholesky, n log-uniform in [1024, 16384], nb in {128, 256});
# the calls are dpotrf (diagonal block), dtrsm (panel), dsyrk (diagonal
# block of the trailing update), dgemm (rest of the trailing update), then
# ddot residual checks on sampled entries.  Plain per-call dispatch (every
# thread calls the library on its own stream and waits) against the serving
# loop (every thread submits to one server and waits).
# --------------------------------------------------------------------------
OP_NAMES = {1: "dgemm", 2: "dtrsm", 3: "dsyrk", 4: "ddot", 5: "dnrm2", 6: "dpotrf", 7: "dgemm_ozaki",
            8: "dsyrk_ozaki", 9: "dtrsm_ozaki"}


def cholesky_calls(n, nb, base, lda, info_ptr, ozaki=False):
    import libgpublas_gb300 as g
    calls = []
    at = lambda i, j: base + 8 * (j * lda + i)   # noqa: E731
    for k in range(0, n, nb):
        kb = min(nb, n - k)
        calls.append(g.GbxOp(kind=6, uplo=b"L", n=kb, C=at(k, k), ldc=lda, B=info_ptr))
        rest = n - k - kb
        if rest <= 0:
            continue
        # L21 = A21 L11^-T
        calls.append(g.GbxOp(kind=9 if ozaki else 2, side=b"R", uplo=b"L", transa=b"T", diag=b"N", m=rest, n=kb,
                             alpha=1.0, A=at(k, k), lda=lda, C=at(k + kb, k), ldc=lda))
        # trailing update, block column by block column
        for j in range(k + kb, n, nb):
            jb = min(nb, n - j)
            calls.append(g.GbxOp(kind=8 if ozaki else 3, uplo=b"L", transa=b"N", n=jb, k=kb,
                                 alpha=-1.0, beta=1.0, A=at(j, k), lda=lda, C=at(j, j), ldc=lda))
            below = n - j - jb
            if below > 0:
                calls.append(g.GbxOp(kind=7 if ozaki else 1, transa=b"N", transb=b"T", m=below, n=jb,
                                     k=kb, alpha=-1.0, beta=1.0, A=at(j + jb, k), lda=lda,
                                     B=at(j, k), ldb=lda, C=at(j + jb, j), ldc=lda))
    return calls


MODES = {
    # name: (through the serving layer, Ozaki forms of dtrsm/dsyrk/dgemm,
    # device-side request loop on)
    "plain": (False, False, False),         # FP64, plain per-call dispatch
    "served": (True, False, False),         # FP64, serving layer as created by default
    "served_loop": (True, False, True),     # FP64, serving layer with its device-side loop (opt-in)
    "served_loop_all": (True, False, "all"),  # FP64, the same with the loop on every SM
    "ozaki_plain": (False, True, False),    # Ozaki, plain per-call dispatch
    "ozaki": (True, True, False),           # Ozaki, serving layer
}


def make_server(g, slots, loop):
    """A Server with its device-side request loop off, on (a quarter of the
    SMs) or on every SM ("all"); both variables are read at creation."""
    import torch
    env = {"GBX_SERVE_LOOP": "1" if loop else "0",
           "GBX_SERVE_LOOP_CTAS": str(torch.cuda.get_device_properties(0).multi_processor_count)
           if loop == "all" else None}
    old = {k: os.environ.get(k) for k in env}
    for k, v in env.items():
        if v is None:
            os.environ.pop(k, None)
        else:
            os.environ[k] = v
    try:
        return g.Server(0, slots=slots)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def serving_trace(g, nthreads, nmin, nmax, seed=5, modes=("plain", "served", "served_loop", "ozaki_plain", "ozaki"),
                  chains=True):
    """Closed-loop Cholesky trace: nthreads native caller threads, thread t
    factorising A = G G^T + n I (G uniform[-1,1], n log-uniform in
    [nmin, nmax], nb in {128, 256}) through the library, once per mode.
    Returns (sizes, nbs, {mode: stats}); each mode reports calls/s, p50/p99
    per-call latency, the sampled residual |A - L L^T| / |A| and the time of
    each thread's chain."""
    import torch
    rng = np.random.default_rng(seed)
    sizes = [int(v) for v in loguni(rng, nmin, nmax, nthreads)]
    nbs = [int(v) for v in rng.choice([128, 256], nthreads)]
    dev = g.Device(0)
    origs = []
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    for n in sizes:
        G = torch.empty(n * n, dtype=torch.float64, device="cuda").uniform_(-1.0, 1.0, generator=gen)
        A = torch.empty(n * n, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        # A = G G^T + n I, both triangles (setup, FP64)
        dev.dgemm_checked("N", "T", n, n, n, 1.0, G, n, G, n, 0.0, A, n)
        dev.sync()
        A.view(n, n).diagonal().add_(float(n))
        torch.cuda.synchronize()
        del G
        origs.append(A)
    info = torch.zeros(nthreads, dtype=torch.int32, device="cuda")
    results = {}
    for mode in modes:
        use_server, ozaki, loop = MODES[mode]
        info.zero_()
        # the caller threads are native (gbx_diag_cholesky_trace): C++
        # threads calling the library as a C or Fortran application would,
        # without interpreter time or lock contention on every call
        server = make_server(g, nthreads, loop) if use_server else None
        work = [o.clone() for o in origs]
        torch.cuda.synchronize()
        r = g.cholesky_trace(server, 0, sizes, nbs, [w.data_ptr() for w in work], info.data_ptr(), ozaki)
        wall = r["wall_s"]
        by_kind = {k: (c, r["kind_sum_us"][k]) for k, c in enumerate(r["kind_calls"]) if c}
        srv_stats = server.stats() if server else None
        if server:
            on, lcalls, llaunch = server.loop_stats()
            srv_stats.update(loop_enabled=on, loop_calls=lcalls, loop_launches=llaunch)
        if server:
            server.close()
        # residual on sampled entries: (L L^T)_ij through ddot on rows of L
        res_num = res_den = 0.0
        out = torch.zeros(1, dtype=torch.float64, device="cuda")
        srng = np.random.default_rng(9)
        for t in range(nthreads):
            n = sizes[t]
            L = work[t]
            for _ in range(8):
                i, j = sorted(int(v) for v in srng.integers(0, n, 2))[::-1]   # i >= j
                dev.ddot(j + 1, L.data_ptr() + 8 * i, n, L.data_ptr() + 8 * j, n, out)
                dev.sync()
                aij = float(origs[t][j * n + i].item())
                res_num += (out.item() - aij) ** 2
                res_den += aij ** 2
        flops = sum(float(n) ** 3 / 3 for n in sizes)
        # each thread's chain alone on the GPU (plain per-call dispatch, one
        # caller thread): a caller's calls are synchronous and dependent, so
        # no scheduler can finish the trace before its slowest lone chain
        chain = None
        if chains and not use_server:
            alone = []
            for t in range(nthreads):
                wt = origs[t].clone()
                torch.cuda.synchronize()
                ra = g.cholesky_trace(None, 0, [sizes[t]], [nbs[t]], [wt.data_ptr()], info.data_ptr() + 4 * t,
                                      ozaki)
                alone.append(ra["wall_s"])
                del wt
            chain = {"alone_s": [round(x, 5) for x in alone], "longest_alone_s": max(alone),
                     "sum_alone_s": sum(alone)}
        results[mode] = {"calls": r["calls"], "wall_s": wall, "calls_per_s": r["calls"] / wall,
                         "chains": chain,
                         "p50_us": r["p50_us"], "p99_us": r["p99_us"],
                         "tflops": flops / wall / 1e12, "flops": flops,
                         "residual_sampled": (res_num / res_den) ** 0.5 if res_den else None,
                         "info_nonzero": int((info != 0).sum().item()),
                         "first_error": r["first_error"], "server": srv_stats,
                         # per operation kind: calls, mean and summed latency
                         "by_kind": {OP_NAMES.get(k, str(k)): {"calls": c, "mean_us": tot / c, "sum_s": tot / 1e6}
                                     for k, (c, tot) in sorted(by_kind.items())},
                         # each thread's finish time: the slowest thread's call chain bounds the wall
                         "thread_finish_s": [round(x, 3) for x in r["thread_finish_s"]]}
        del work
        torch.cuda.synchronize()
    origs.clear()
    dev.close()
    torch.cuda.empty_cache()
    return sizes, nbs, results


def small_call_trace(g, nthreads, ncalls, size=64, modes=("plain", "served", "served_loop", "served_loop_all")):
    """Latency-bound calls: nthreads native threads each issue ncalls FP64
    DGEMMs of size^3 (C += A B on the thread's own operands), one at a time,
    per mode: plain per-call dispatch, the serving layer as created by
    default, and with its device-side loop (on a quarter of the SMs, and on
    every SM).  Returns calls/s, p50/p99 per mode and the gains over plain
    dispatch."""
    import torch
    n = size
    bufs = []
    for t in range(nthreads):
        a = torch.rand(n * n, dtype=torch.float64, device="cuda") * 2 - 1
        b = torch.rand(n * n, dtype=torch.float64, device="cuda") * 2 - 1
        c = torch.zeros(n * n, dtype=torch.float64, device="cuda")
        bufs.append((a, b, c))
    torch.cuda.synchronize()
    ops = [[g.GbxOp(kind=1, transa=b"N", transb=b"N", m=n, n=n, k=n, alpha=1.0, beta=1.0, A=a.data_ptr(), lda=n,
                    B=b.data_ptr(), ldb=n, C=c.data_ptr(), ldc=n)] * ncalls for a, b, c in bufs]
    out = {}
    for mode in modes:
        use_server, _, loop = MODES[mode]
        for _, _, c in bufs:
            c.zero_()
        torch.cuda.synchronize()
        server = make_server(g, max(2, min(16, nthreads)), loop) if use_server else None
        r = g.ops_trace(server, 0, ops)
        if server:
            server.close()
        a, b, c = bufs[0]
        want = ncalls * (a.view(n, n).T @ b.view(n, n).T)       # column-major: A = a.view(n, n).T
        got = c.view(n, n).T
        err = float((got - want).norm() / want.norm())
        out[mode] = {"calls": r["calls"], "calls_per_s": r["calls"] / r["wall_s"], "p50_us": r["p50_us"],
                     "p99_us": r["p99_us"], "rel_err_thread0": err, "first_error": r["first_error"]}
    for mode in ("served", "served_loop", "served_loop_all"):
        if "plain" in out and mode in out:
            out[f"{mode}_vs_plain"] = out[mode]["calls_per_s"] / out["plain"]["calls_per_s"]
    return out


def serving_ratios(results, fp64_peak_tflops=None):
    """Same-precision ratios (the loop's own effect) and the precision's,
    and the bounds on what any scheduler could gain over plain dispatch."""
    def ratio(a, b):
        return results[a]["calls_per_s"] / results[b]["calls_per_s"] if a in results and b in results else None
    out = {"served_vs_plain_fp64": ratio("served", "plain"),
           "served_loop_vs_plain_fp64": ratio("served_loop", "plain"),
           "served_vs_plain_ozaki": ratio("ozaki", "ozaki_plain"),
           "ozaki_plain_vs_fp64_plain": ratio("ozaki_plain", "plain"),
           "ozaki_served_vs_fp64_plain": ratio("ozaki", "plain")}
    # the most any scheduler could gain over plain dispatch in the same
    # precision: the plain wall over the slowest caller's chain run alone
    for prec, plain in (("fp64", "plain"), ("ozaki", "ozaki_plain")):
        ch = results.get(plain, {}).get("chains")
        if ch:
            out[f"plain_wall_over_longest_chain_{prec}"] = results[plain]["wall_s"] / ch["longest_alone_s"]
    if fp64_peak_tflops and "plain" in results:
        # FP64: the trace's n^3/3 flops at the measured DFMA rate
        fb = results["plain"]["flops"] / (fp64_peak_tflops * 1e12)
        out["fp64_pipe_bound_s"] = fb
        ch = results["plain"].get("chains")
        if ch:
            out["max_gain_fp64_any_scheduler"] = results["plain"]["wall_s"] / max(fb, ch["longest_alone_s"])
    return out


def run_serving(args):
    import libgpublas_gb300 as g
    from libgpublas_gb300 import build
    build.build_library()
    nthreads = 16
    sizes, nbs, results = serving_trace(g, nthreads, 1024, args.n or 16384)
    open_loop = None if args.no_open_loop else run_serving_open_loop(g, results)
    head = results["ozaki"]
    line = {"metric": "serving_calls_per_s", "value": head["calls_per_s"],
            "unit": "calls/s", "n_gpus": 1, "steps": 1, "warmup": 0,
            "ms_per_step": head["wall_s"] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "cholesky_trace_16threads", "n": sizes, "nb": nbs,
                       "matrix": "A = G G^T + n I, G uniform[-1,1] (device generator, seed 5)",
                       "driver": "16 native host threads (gbx_diag_cholesky_trace), one call at a time each",
                       "calls": "dpotrf(diag) dtrsm dsyrk dgemm + ddot residual checks",
                       "headline_mode": "ozaki: serving layer, dgemm/dsyrk/dtrsm through the Ozaki path "
                                        "(tolerance 1e-14, FP64 results), dpotrf in FP64"},
            "modes": results,
            "ratios": serving_ratios(results, g.Device(0).fp64_peak()),
            "small_calls": {"dgemm_64_threads1": small_call_trace(g, 1, 2000),
                            "dgemm_64_threads16": small_call_trace(g, 16, 500)},
            "residual_sampled": {m: results[m]["residual_sampled"] for m in results},
            "open_loop": open_loop,
            "e2e": {"unavailable": "operands are device-resident by design of this workload"}}
    print(json.dumps(line), flush=True)


def run_serving_open_loop(g, closed, njobs=48, nmax=4096, workers=16, seed=11):
    """Open-loop form of the Cholesky trace: factorisation jobs (n
    log-uniform in [1024, nmax], nb in {128, 256}) arrive as a Poisson
    process at swept rates and a pool of worker threads takes them in
    arrival order.  Reports, per mode and offered rate, the achieved calls/s,
    per-call latency p50/p99 and job latency (arrival to last call) p50/p99.
    The rates are fractions of each mode's closed-loop capacity in jobs/s,
    estimated from the closed-loop calls/s and the jobs' mean call count."""
    import threading
    import torch
    rng = np.random.default_rng(seed)
    sizes = [int(v) for v in loguni(rng, 1024, nmax, njobs)]
    nbs = [int(v) for v in rng.choice([128, 256], njobs)]
    dev = g.Device(0)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    origs = []
    for n in sizes:
        G = torch.empty(n * n, dtype=torch.float64, device="cuda").uniform_(-1.0, 1.0, generator=gen)
        A = torch.empty(n * n, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        dev.dgemm_ozaki("N", "T", n, n, n, 1.0, G, n, G, n, 0.0, A, n)
        A.view(n, n).diagonal().add_(float(n))
        dev.sync()
        del G
        origs.append(A)
    info = torch.zeros(njobs, dtype=torch.int32, device="cuda")
    ncalls = [len(cholesky_calls(n, nb, 0, n, 0)) for n, nb in zip(sizes, nbs)]
    out = {}
    for mode in ("plain", "served", "ozaki_plain", "ozaki"):
        use_server, ozaki, loop = MODES[mode]
        cap = closed[mode]["calls_per_s"] / (sum(ncalls) / njobs)   # jobs/s at closed-loop throughput
        rows = []
        for frac in (0.25, 0.5, 0.75, 1.0):
            rate = frac * cap
            arrivals = np.cumsum(np.random.default_rng(seed + 1).exponential(1.0 / rate, njobs))
            work = [o.clone() for o in origs]
            info.zero_()
            torch.cuda.synchronize()
            server = make_server(g, workers, loop) if use_server else None
            lat, job_lat, errs = [], [0.0] * njobs, []
            lock = threading.Lock()
            nxt = [0]
            t0 = time.perf_counter()

            def worker():
                d = g.Device(0) if server is None else None
                local = []
                while True:
                    with lock:
                        j = nxt[0]
                        nxt[0] += 1
                    if j >= njobs:
                        break
                    wait = t0 + arrivals[j] - time.perf_counter()
                    if wait > 0:
                        time.sleep(wait)
                    calls = cholesky_calls(sizes[j], nbs[j], work[j].data_ptr(), sizes[j],
                                           info.data_ptr() + 4 * j, ozaki=ozaki)
                    for op in calls:
                        if server is None:
                            c0 = time.perf_counter()
                            st = d.L.gbx_ops_run(d.ctx, ctypes_ref(op), 1) or d.L.gbx_ctx_sync(d.ctx)
                            us = (time.perf_counter() - c0) * 1e6
                        else:
                            st, us = server.call(op)
                        local.append(us)
                        if st:
                            errs.append((j, st))
                            break
                    job_lat[j] = time.perf_counter() - (t0 + arrivals[j])
                if d is not None:
                    d.close()
                with lock:
                    lat.extend(local)

            threads = [threading.Thread(target=worker) for _ in range(workers)]
            for th in threads:
                th.start()
            for th in threads:
                th.join()
            wall = time.perf_counter() - t0
            if server:
                server.close()
            torch.cuda.synchronize()
            lat.sort()
            jl = sorted(job_lat)
            rows.append({"offered_jobs_per_s": rate, "load_fraction": frac, "calls": len(lat),
                         "wall_s": wall, "calls_per_s": len(lat) / wall,
                         "p50_us": lat[len(lat) // 2], "p99_us": lat[int(0.99 * (len(lat) - 1))],
                         "job_p50_ms": jl[njobs // 2] * 1e3, "job_p99_ms": jl[int(0.99 * (njobs - 1))] * 1e3,
                         "info_nonzero": int((info != 0).sum().item()), "errors": errs[:4]})
            del work
        out[mode] = rows
    dev.close()
    return {"jobs": njobs, "n": sizes, "nb": nbs, "workers": workers,
            "arrivals": f"Poisson, seed {seed + 1}; rate = fraction x closed-loop capacity in jobs/s",
            "modes": out}


# --------------------------------------------------------------------------
# Ozaki configuration: DGEMM and ZGEMM at n in {4096, 8192, 16384}, entries
# u * 2^e (u uniform[-1,1], e uniform integer in [-s, s]) for s in {0, 8, 24};
# ZGEMM real and imaginary parts drawn independently the same way.  Reports
# TFLOP/s (2n^3 real, 8n^3 complex), the slice count chosen for 1e-14 and
# the relative Frobenius error against the double-double oracle on sampled
# entries.
# --------------------------------------------------------------------------
def run_ozaki_sweep(args):
    import torch
    import libgpublas_gb300 as g
    import oracle
    from libgpublas_gb300 import build
    build.build_library()
    orc = oracle.get()
    dev = g.Device(0)
    stream = torch.cuda.ExternalStream(dev.stream())
    sizes = [args.n] if args.n else [4096, 8192, 16384]
    rows_out = []
    for n in sizes:
        for s in (0, 8, 24):
            st = 1000 + n + s
            a, st = orc.spread((n, n), s, st)
            b, st = orc.spread((n, n), s, st)
            da = torch.from_numpy(a.ravel(order="F")).cuda()
            db = torch.from_numpy(b.ravel(order="F")).cuda()
            dc = torch.zeros(n * n, dtype=torch.float64, device="cuda")
            used = dev.dgemm_ozaki("N", "N", n, n, n, 1.0, da, n, db, n, 0.0, dc, n)
            dev.sync()
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            for _ in range(args.steps):
                dev.dgemm_ozaki("N", "N", n, n, n, 1.0, da, n, db, n, 0.0, dc, n)
            ev1.record(stream)
            ev1.synchronize()
            t = ev0.elapsed_time(ev1) / 1e3 / args.steps
            got = dc.cpu().numpy().reshape(n, n, order="F")
            rng = np.random.default_rng(n + s)
            ri, ci = rng.integers(0, n, 1024), rng.integers(0, n, 1024)
            ref = orc.dgemm_dd_sample("N", "N", n, 1.0, a, b, 0.0, np.zeros((1, 1), order="F"), ri, ci)
            err = float(np.linalg.norm(got[ri, ci] - ref) / np.linalg.norm(ref))
            rows_out.append({"routine": "dgemm", "n": n, "spread": s, "slices": used,
                             "tflops": 2.0 * n ** 3 / t / 1e12, "ms": t * 1e3, "rel_err": err})
            del da, db, dc
            # ZGEMM: independent real and imaginary parts, same distribution
            ai, st = orc.spread((n, n), s, st)
            bi, st = orc.spread((n, n), s, st)
            za = np.empty((n, n), dtype=np.complex128, order="F")
            za.real, za.imag = a, ai
            zb = np.empty((n, n), dtype=np.complex128, order="F")
            zb.real, zb.imag = b, bi
            del ai, bi
            dza = torch.from_numpy(za.ravel(order="F").view(np.float64)).cuda()
            dzb = torch.from_numpy(zb.ravel(order="F").view(np.float64)).cuda()
            dzc = torch.zeros(2 * n * n, dtype=torch.float64, device="cuda")
            used = dev.zgemm_ozaki("N", "N", n, n, n, 1.0, dza, n, dzb, n, 0.0, dzc, n)
            dev.sync()
            ev0.record(stream)
            for _ in range(args.steps):
                dev.zgemm_ozaki("N", "N", n, n, n, 1.0, dza, n, dzb, n, 0.0, dzc, n)
            ev1.record(stream)
            ev1.synchronize()
            t = ev0.elapsed_time(ev1) / 1e3 / args.steps
            zgot = dzc.cpu().numpy().view(np.complex128).reshape(n, n, order="F")
            zref = orc.zgemm_dd_sample("N", "N", n, 1.0, za, zb, 0.0,
                                       np.zeros((1, 1), dtype=np.complex128, order="F"), ri, ci)
            err = float(np.linalg.norm(zgot[ri, ci] - zref) / np.linalg.norm(zref))
            rows_out.append({"routine": "zgemm", "n": n, "spread": s, "slices": used,
                             "tflops": 8.0 * n ** 3 / t / 1e12, "ms": t * 1e3, "rel_err": err})
            del dza, dzb, dzc, za, zb, a, b
            torch.cuda.empty_cache()
            print(json.dumps(rows_out[-2]), json.dumps(rows_out[-1]), file=sys.stderr, flush=True)
    head = next(r for r in rows_out if r["routine"] == "dgemm" and r["n"] == max(sizes) and r["spread"] == 0)
    line = {"metric": "ozaki_dgemm_tflops", "value": head["tflops"], "unit": "TFLOP/s", "n_gpus": 1,
            "steps": args.steps, "warmup": 1, "ms_per_step": head["ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"ozaki_sweep_dgemm_zgemm_n{'_'.join(map(str, sizes))}",
                       "inputs": "u * 2^e, u uniform[-1,1], e uniform in [-s, s], SplitMix64",
                       "tol": 1e-14, "value_is": f"DGEMM n={max(sizes)} s=0"},
            "sweep": rows_out,
            "e2e": {"unavailable": "device-resident sweep; see the dgemm workload for e2e"}}
    print(json.dumps(line), flush=True)
    dev.close()


# --------------------------------------------------------------------------
# arithmetic pipes of the GPU (the measurements behind the kernel choices):
# SIMT DFMA and the legacy mma.sync paths, dependent-chain latencies, and
# the issue cost of tcgen05.mma for the Ozaki tile widths
# --------------------------------------------------------------------------
def run_pipes(args):
    import libgpublas_gb300 as g
    from libgpublas_gb300 import build
    build.build_library()
    dev = g.Device(0)
    with ClockSampler(0) as clk:
        rates = dev.pipe_rates()
        sms = 152
        try:
            import torch
            sms = torch.cuda.get_device_properties(0).multi_processor_count
        except Exception:
            pass
        issue = []
        for n in (16, 32, 64, 128, 256):
            for grid in (1, sms):
                i_cyc, d_cyc = dev.mma_issue(n, 1024, grid)
                issue.append({"n": n, "count": 1024, "ctas": grid, "issue_cycles": i_cyc, "done_cycles": d_cyc})
    line = {"metric": "dfma_tflops", "value": rates["dfma_tflops"], "unit": "TFLOP/s", "n_gpus": 1,
            "steps": 3, "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "pipe_throughput_and_tcgen05_issue"},
            "pipes": rates, "tcgen05_mma_issue": issue, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    dev.close()


def ctypes_ref(op):
    import ctypes
    return ctypes.byref(op)


def main():
    args = parse_args()
    if args.workload == "batched":
        return run_batched(args) if args.impl == "ours" else print(json.dumps(
            {"impl": "reference", "unavailable": "the reference has no grouped execution; "
                                                 "the CPU BLAS runs one call at a time"}))
    if args.workload == "serving":
        return run_serving(args) if args.impl == "ours" else print(json.dumps(
            {"impl": "reference", "unavailable": "the reference has no serving loop"}))
    if args.workload == "pipes":
        return run_pipes(args) if args.impl == "ours" else print(json.dumps(
            {"impl": "reference", "unavailable": "a measurement of the GPU, not of a BLAS path"}))
    if args.workload == "ozaki_sweep":
        return run_ozaki_sweep(args) if args.impl == "ours" else print(json.dumps(
            {"impl": "reference", "unavailable": "the reference has no Ozaki path"}))
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
