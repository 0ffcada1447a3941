"""The serving layer's device-side request loop.

FP64 DGEMM and DSYRK with m, n <= 512 and k <= 4096, and DTRSM with a
triangle of order <= 256 and at most 256 right-hand sides, made through
gbx_server_call run, on a server created with GBX_SERVE_LOOP=1, on a
resident kernel fed through a ring in pinned host memory.  Checked here:
  * results: DGEMM and DSYRK bit-identical to the same call on the stream
    path (the same GEMM core, one FMA chain per element over K in order);
    DTRSM within a backward residual of 1e-14 of the double-double oracle;
  * the calls really ran on the loop (its counters), and the resident kernel
    comes back after it left the GPU for lack of work;
  * 16 host threads at once: every result equal to the one served alone;
  * without GBX_SERVE_LOOP=1 (the default) the same calls run on the slot
    streams.
"""
import os
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def loop_server(g, slots):
    """A server with its device-side request loop on (GBX_SERVE_LOOP=1 is
    read at creation)."""
    old = os.environ.get("GBX_SERVE_LOOP")
    os.environ["GBX_SERVE_LOOP"] = "1"
    try:
        return g.Server(0, slots=slots)
    finally:
        if old is None:
            del os.environ["GBX_SERVE_LOOP"]
        else:
            os.environ["GBX_SERVE_LOOP"] = old


def to_dev(a):
    import torch
    t = torch.from_numpy(np.asfortranarray(a).ravel(order="F").copy()).cuda()
    torch.cuda.synchronize()
    return t


def ops_for(g, orc, seed):
    """A mix of GEMM / SYRK / TRSM requests on device operands; returns the
    ops, a reset function and a reader of every output."""
    import torch
    rng = np.random.default_rng(seed)
    specs, ops = [], []
    s = seed
    for i in range(24):
        kind = (1, 3, 2)[i % 3]
        if kind == 1:
            m, n, k = (int(v) for v in rng.integers(8, 513, 3))   # the loop takes m, n <= 512
            ta, tb = rng.choice(["N", "T"], 2)
            ra, ca = (m, k) if ta == "N" else (k, m)
            rb, cb = (k, n) if tb == "N" else (n, k)
            a, s = orc.matrix(ra, ca, s)
            b, s = orc.matrix(rb, cb, s)
            c, s = orc.matrix(m, n, s)
            A, B, Cd = to_dev(a), to_dev(b), to_dev(c)
            specs.append(dict(kind=1, ta=ta, tb=tb, m=m, n=n, k=k, a=a, b=b, c=c, A=A, B=B, C=Cd, c0=Cd.clone()))
            ops.append(g.GbxOp(kind=1, transa=ta.encode(), transb=tb.encode(), m=m, n=n, k=k, alpha=1.25, beta=-0.5,
                               A=A.data_ptr(), lda=ra, B=B.data_ptr(), ldb=rb, C=Cd.data_ptr(), ldc=m))
        elif kind == 3:
            n, k = (int(v) for v in rng.integers(16, 513, 2))
            uplo, tr = rng.choice(["L", "U"]), rng.choice(["N", "T"])
            ra, ca = (n, k) if tr == "N" else (k, n)
            a, s = orc.matrix(ra, ca, s)
            c, s = orc.matrix(n, n, s)
            A, Cd = to_dev(a), to_dev(c)
            specs.append(dict(kind=3, uplo=uplo, tr=tr, n=n, k=k, a=a, c=c, A=A, C=Cd, c0=Cd.clone()))
            ops.append(g.GbxOp(kind=3, uplo=uplo.encode(), transa=tr.encode(), n=n, k=k, alpha=-1.0, beta=1.0,
                               A=A.data_ptr(), lda=ra, C=Cd.data_ptr(), ldc=n))
        else:
            order = int(rng.integers(8, 257))
            side, uplo, ta = rng.choice(["L", "R"]), rng.choice(["L", "U"]), rng.choice(["N", "T"])
            nrhs = int(rng.integers(1, 257))       # the loop takes solves of <= 256 right-hand sides
            m, n = (order, nrhs) if side == "L" else (nrhs, order)
            a, s = orc.trsm_matrix(order, s)
            b, s = orc.matrix(m, n, s)
            A, Bd = to_dev(a), to_dev(b)
            specs.append(dict(kind=2, side=side, uplo=uplo, ta=ta, m=m, n=n, a=a, b=b, A=A, C=Bd, c0=Bd.clone()))
            ops.append(g.GbxOp(kind=2, side=side.encode(), uplo=uplo.encode(), transa=ta.encode(), diag=b"N",
                               m=m, n=n, alpha=0.75, A=A.data_ptr(), lda=order, C=Bd.data_ptr(), ldc=m))

    def reset():
        for sp in specs:
            sp["C"].copy_(sp["c0"])
        torch.cuda.synchronize()

    def outputs():
        torch.cuda.synchronize()
        return [sp["C"].cpu().numpy().copy() for sp in specs]
    return specs, ops, reset, outputs


def test_loop_results_and_counters(orc, dev, lib):
    import libgpublas_gb300 as g
    specs, ops, reset, outputs = ops_for(g, orc, 41)
    srv = loop_server(g, 4)
    try:
        enabled, calls0, _ = srv.loop_stats()
        assert enabled
        reset()
        for op in ops:
            st, _ = srv.call(op)
            assert st == 0
        got = outputs()
        enabled, calls1, launches = srv.loop_stats()
        assert calls1 - calls0 == len(ops) and launches >= 1
    finally:
        srv.close()
    # the stream path on the same requests
    reset()
    for sp in specs:
        if sp["kind"] == 1:
            dev.dgemm_checked(sp["ta"], sp["tb"], sp["m"], sp["n"], sp["k"], 1.25, sp["A"], sp["a"].shape[0],
                              sp["B"], sp["b"].shape[0], -0.5, sp["C"], sp["m"])
        elif sp["kind"] == 3:
            dev.dsyrk(sp["uplo"], sp["tr"], sp["n"], sp["k"], -1.0, sp["A"], sp["a"].shape[0], 1.0, sp["C"], sp["n"])
    dev.sync()
    want = outputs()
    for sp, a, w in zip(specs, got, want):
        if sp["kind"] in (1, 3):
            assert np.array_equal(a, w), sp["kind"]
        else:
            x = np.asfortranarray(a.reshape(sp["m"], sp["n"], order="F"))
            r = orc.dtrsm_residual(sp["side"], sp["uplo"], sp["ta"], "N", sp["m"], sp["n"], 0.75, sp["a"],
                                   sp["b"], x)
            assert r <= 1e-14, r


def test_loop_restarts_after_leaving_idle(orc, lib):
    import libgpublas_gb300 as g
    specs, ops, reset, outputs = ops_for(g, orc, 42)
    srv = loop_server(g, 2)
    try:
        reset()
        assert srv.call(ops[0])[0] == 0
        first = outputs()[0]
        _, _, l1 = srv.loop_stats()
        time.sleep(0.2)                 # the resident kernel leaves after 20 ms without work
        reset()
        assert srv.call(ops[0])[0] == 0
        _, _, l2 = srv.loop_stats()
        assert l2 > l1
        assert np.array_equal(outputs()[0], first)
    finally:
        srv.close()


def test_loop_sixteen_threads_equal_alone(orc, lib):
    import libgpublas_gb300 as g
    specs, ops, reset, outputs = ops_for(g, orc, 43)
    srv = loop_server(g, 8)
    try:
        reset()
        for op in ops:
            assert srv.call(op)[0] == 0
        alone = outputs()
        reset()
        errors = []

        def worker(t):
            for j in range(t, len(ops), 16):
                st, _ = srv.call(ops[j])
                if st:
                    errors.append((j, st))
        threads = [threading.Thread(target=worker, args=(t,)) for t in range(16)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        assert not errors
        for a, m in zip(alone, outputs()):
            assert np.array_equal(a, m)
    finally:
        srv.close()


def test_loop_off_runs_on_slot_streams(orc, lib):
    import libgpublas_gb300 as g
    specs, ops, reset, outputs = ops_for(g, orc, 44)
    old = os.environ.pop("GBX_SERVE_LOOP", None)
    try:
        srv = g.Server(0, slots=4)
    finally:
        if old is not None:
            os.environ["GBX_SERVE_LOOP"] = old
    try:
        enabled, calls, _ = srv.loop_stats()
        assert not enabled
        reset()
        for op in ops:
            assert srv.call(op)[0] == 0
        assert srv.loop_stats()[1] == 0
        got = outputs()
    finally:
        srv.close()
    for sp, a in zip(specs, got):
        if sp["kind"] == 1:
            want = orc.dgemm_dd(sp["ta"], sp["tb"], sp["m"], sp["n"], sp["k"], 1.25, sp["a"], sp["b"], -0.5,
                                sp["c"])
            assert np.linalg.norm(a.reshape(sp["m"], sp["n"], order="F") - want) <= 1e-13 * np.linalg.norm(want)
