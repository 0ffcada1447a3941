"""The serving loop: calls from 16 host threads, continuously batched.

* Each result is bit-identical whether the call was served alone (one call
  in flight) or in a mix with all the others submitted concurrently from 16
  threads, and matches the oracle (relative error <= 1e-13; DTRSM residual
  <= 1e-14; DDOT/DNRM2 within 2*n*u of the double-double value).
* A call runs inline on a free slot when nothing waits to be grouped with
  it; small calls that queue up behind busy slots are grouped into one
  launch (fewer device batches than calls).
* Admission by memory: a reservation larger than the budget is refused; two
  reservations that do not fit together are serialised.
"""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def loguni(rng, lo, hi):
    return int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))


class Calls:
    def __init__(self, orc, count, seed):
        import torch
        import libgpublas_gb300 as g
        rng = np.random.default_rng(seed)
        chunks, self.specs, off = [], [], 0

        def place(a):
            nonlocal off
            a = np.asfortranarray(a)
            chunks.append(a.ravel(order="F"))
            pad = -a.size % 4
            if pad:
                chunks.append(np.zeros(pad))
            start = off
            off += a.size + pad
            return start

        s = seed
        for i in range(count):
            kind = [1, 1, 1, 2, 3, 4, 1, 2][i % 8]
            if kind == 1:
                big = i % 16 == 0
                m, n, k = ((loguni(rng, 600, 1200),) * 3 if big else
                           (loguni(rng, 8, 300), loguni(rng, 8, 300), loguni(rng, 8, 300)))
                a, s = orc.matrix(m, k, s)
                b, s = orc.matrix(k, n, s)
                c, s = orc.matrix(m, n, s)
                self.specs.append(dict(kind=1, m=m, n=n, k=k, a=a, b=b, c=c, oa=place(a), ob=place(b),
                                       oc=place(c)))
            elif kind == 2:
                order = loguni(rng, 8, 256) if i % 3 else loguni(rng, 300, 600)
                a, s = orc.trsm_matrix(order, s)
                b, s = orc.matrix(order, 16, s)
                self.specs.append(dict(kind=2, m=order, n=16, a=a, b=b, oa=place(a), ob=place(b)))
            elif kind == 3:
                n, k = loguni(rng, 64, 700), loguni(rng, 16, 300)
                a, s = orc.matrix(n, k, s)
                c, s = orc.matrix(n, n, s)
                self.specs.append(dict(kind=3, n=n, k=k, a=a, c=c, oa=place(a), oc=place(c)))
            else:
                n = loguni(rng, 100, 200000)
                x, s = orc.uniform(n, s)
                y, s = orc.uniform(n, s)
                self.specs.append(dict(kind=4, n=n, x=x, y=y, ox=place(x), oy=place(y),
                                       ores=place(np.zeros(1))))
        self.host = np.concatenate(chunks)
        self.dev = torch.from_numpy(self.host).cuda()
        base = self.dev.data_ptr()
        self.ops = []
        for sp in self.specs:
            if sp["kind"] == 1:
                op = g.GbxOp(kind=1, transa=b"N", transb=b"N", m=sp["m"], n=sp["n"], k=sp["k"],
                             alpha=1.0, beta=0.5, A=base + 8 * sp["oa"], lda=sp["m"],
                             B=base + 8 * sp["ob"], ldb=sp["k"], C=base + 8 * sp["oc"], ldc=sp["m"])
            elif sp["kind"] == 2:
                op = g.GbxOp(kind=2, transa=b"N", side=b"L", uplo=b"L", diag=b"N", m=sp["m"], n=16,
                             alpha=1.0, A=base + 8 * sp["oa"], lda=sp["m"], C=base + 8 * sp["ob"],
                             ldc=sp["m"])
            elif sp["kind"] == 3:
                op = g.GbxOp(kind=3, uplo=b"L", transa=b"N", n=sp["n"], k=sp["k"], alpha=-1.0,
                             beta=1.0, A=base + 8 * sp["oa"], lda=sp["n"], C=base + 8 * sp["oc"],
                             ldc=sp["n"])
            else:
                op = g.GbxOp(kind=4, n=sp["n"], A=base + 8 * sp["ox"], lda=1, B=base + 8 * sp["oy"],
                             ldb=1, C=base + 8 * sp["ores"])
            self.ops.append(op)

    def reset(self):
        import torch
        self.dev.copy_(torch.from_numpy(self.host))
        torch.cuda.synchronize()

    def outputs(self):
        h = self.dev.cpu().numpy()
        out = []
        for sp in self.specs:
            key = {1: "oc", 2: "ob", 3: "oc", 4: "ores"}[sp["kind"]]
            ref = {1: "c", 2: "b", 3: "c", 4: None}[sp["kind"]]
            size = 1 if ref is None else sp[ref].size
            shape = (1,) if ref is None else sp[ref].shape
            out.append(h[sp[key]: sp[key] + size].reshape(shape, order="F").copy())
        return out


@pytest.fixture(scope="module")
def server(lib):
    import libgpublas_gb300 as g
    s = g.Server(0, slots=8)
    yield s
    s.close()


def test_alone_equals_in_mix_and_oracle(orc, server):
    calls = Calls(orc, 96, seed=11)
    calls.reset()
    for op in calls.ops:
        st, _ = server.call(op)
        assert st == 0
    alone = calls.outputs()

    calls.reset()
    server.reset_stats()
    errors = []

    def worker(idx):
        for j in range(idx, len(calls.ops), 16):
            st, _ = server.call(calls.ops[j])
            if st != 0:
                errors.append((j, st))

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(16)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors
    mixed = calls.outputs()
    st = server.stats()
    assert st["completed"] == len(calls.ops)
    assert st["batches"] <= st["completed"]
    assert 0 < st["p50_us"] <= st["p99_us"]
    for sp, a, m in zip(calls.specs, alone, mixed):
        assert np.array_equal(a, m), sp["kind"]

    for sp, got in zip(calls.specs, mixed):
        if sp["kind"] == 1:
            want = sp["c"].copy(order="F")
            orc.dgemm("N", "N", sp["m"], sp["n"], sp["k"], 1.0, sp["a"], sp["b"], 0.5, want)
            assert np.linalg.norm(got - want) <= 1e-13 * np.linalg.norm(want)
        elif sp["kind"] == 2:
            r = orc.dtrsm_residual("L", "L", "N", "N", sp["m"], 16, 1.0, sp["a"], sp["b"],
                                   np.asfortranarray(got))
            assert r <= 1e-14
        elif sp["kind"] == 3:
            want = sp["c"].copy(order="F")
            orc.dsyrk("L", "N", sp["n"], sp["k"], -1.0, sp["a"], 1.0, want)
            assert np.linalg.norm(np.tril(got - want)) <= 1e-13 * np.linalg.norm(np.tril(want))
        else:
            ref = orc.ddot_dd(sp["n"], sp["x"], 1, sp["y"], 1)
            bound = 2 * sp["n"] * 2.0 ** -53 * float(np.abs(sp["x"]) @ np.abs(sp["y"]))
            assert abs(got[0] - ref) <= bound


def test_submit_many_then_wait(orc, server):
    calls = Calls(orc, 40, seed=12)
    calls.reset()
    tickets = [server.submit(op) for op in calls.ops]
    for t in reversed(tickets):
        st, lat = server.wait(t)
        assert st == 0 and lat > 0


def test_small_calls_queued_behind_a_busy_slot_are_grouped(orc, lib):
    # One slot, kept busy by a long DGEMM: the small calls submitted
    # meanwhile queue up and its worker takes them as one grouped launch;
    # their results equal the same calls served one at a time.
    import torch
    import libgpublas_gb300 as g
    srv = g.Server(0, slots=1)
    try:
        n = 3072
        big = [torch.rand(n * n, dtype=torch.float64, device="cuda") for _ in range(3)]
        torch.cuda.synchronize()
        long_op = g.GbxOp(kind=1, transa=b"N", transb=b"N", m=n, n=n, k=n, alpha=1.0, beta=0.0,
                          A=big[0].data_ptr(), lda=n, B=big[1].data_ptr(), ldb=n, C=big[2].data_ptr(), ldc=n)
        calls = Calls(orc, 24, seed=13)
        small = [op for op, sp in zip(calls.ops, calls.specs) if sp["kind"] in (1, 2)]
        kinds = [sp for sp in calls.specs if sp["kind"] in (1, 2)]
        calls.reset()
        for op in small:
            st, _ = srv.call(op)
            assert st == 0
        alone = [o for o, sp in zip(calls.outputs(), calls.specs) if sp["kind"] in (1, 2)]
        calls.reset()
        srv.reset_stats()
        t_long = srv.submit(long_op)          # about 45 ms of FP64 work
        tickets = [srv.submit(op) for op in small]
        assert srv.wait(t_long)[0] == 0
        for t in tickets:
            assert srv.wait(t)[0] == 0
        st = srv.stats()
        assert st["grouped_calls"] >= 2, st
        assert st["batches"] < st["completed"], st
        grouped = [o for o, sp in zip(calls.outputs(), calls.specs) if sp["kind"] in (1, 2)]
        for sp, a, b in zip(kinds, alone, grouped):
            assert np.array_equal(a, b), sp["kind"]
    finally:
        srv.close()


def test_memory_admission(lib):
    import libgpublas_gb300 as g
    s = g.Server(0, slots=2, mem_budget=1 << 20)
    try:
        assert s.admit(2 << 20) == 6        # GBX_ERR_ADMISSION: can never fit
        assert s.admit(600 << 10) == 0
        order = []

        def second():
            assert s.admit(600 << 10) == 0  # waits until the first is released
            order.append("second admitted")
            s.release(600 << 10)

        t = threading.Thread(target=second)
        t.start()
        time.sleep(0.2)
        order.append("first released")
        s.release(600 << 10)
        t.join(timeout=10)
        assert order == ["first released", "second admitted"]
        assert s.stats()["admission_waits"] >= 1
    finally:
        s.close()


def test_fortran_calls_through_the_serving_loop(orc):
    # BLAS2CUDA_OPTIONS=serve=on: dgemm_/dtrsm_/dsyrk_ from 8 threads on host
    # operands go through one serving loop; results match the oracle.
    import os
    import subprocess
    import sys
    import textwrap
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = textwrap.dedent("""
        import threading, numpy as np, oracle, libgpublas_gb300 as g
        orc = oracle.get(); f = g.F77(); errs = []
        def work(t):
            try:
                m, n, k = 100 + 37 * t, 90 + 11 * t, 120
                a, s = orc.matrix(m, k, t); b, s = orc.matrix(k, n, s); c, s = orc.matrix(m, n, s)
                want = orc.dgemm_dd('N', 'N', m, n, k, 1.0, a, b, 0.5, c)
                got = c.copy(order='F'); f.dgemm('N', 'N', m, n, k, 1.0, a, m, b, k, 0.5, got, m)
                assert np.linalg.norm(got - want) <= 1e-13 * np.linalg.norm(want)
                tri, s = orc.trsm_matrix(m, s + 1); rhs, s = orc.matrix(m, 16, s)
                x = rhs.copy(order='F'); f.dtrsm('L', 'L', 'N', 'N', m, 16, 1.0, tri, m, x, m)
                assert orc.dtrsm_residual('L', 'L', 'N', 'N', m, 16, 1.0, tri, rhs, x) <= 1e-14
                cs, s = orc.matrix(m, m, s); want = cs.copy(order='F')
                orc.dsyrk('L', 'N', m, k, -1.0, a, 1.0, want)
                gs = cs.copy(order='F'); f.dsyrk('L', 'N', m, k, -1.0, a, m, 1.0, gs, m)
                assert np.linalg.norm(np.tril(gs - want)) <= 1e-13 * np.linalg.norm(np.tril(want))
            except Exception as e:
                errs.append(repr(e))
        th = [threading.Thread(target=work, args=(t,)) for t in range(8)]
        [x.start() for x in th]; [x.join() for x in th]
        print('ERRS', errs)
    """)
    env = dict(os.environ, PYTHONPATH=root, BLAS2CUDA_OPTIONS="serve=on;errors=return")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, cwd=root,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "ERRS []" in r.stdout, r.stdout + r.stderr[-2000:]


@pytest.mark.parametrize("mode", ["plain", "served", "ozaki"])
def test_native_cholesky_trace(lib, mode):
    # the serving benchmark's native driver: 3 threads factorise SPD matrices
    # through the serving loop (or plain dispatch); each factor L must
    # reproduce A = L L^T on the lower triangle
    import torch
    import libgpublas_gb300 as g
    sizes, nbs = [300, 517, 256], [128, 256, 128]
    gen = torch.Generator(device="cuda")
    gen.manual_seed(21)
    mats, origs = [], []
    for n in sizes:
        G = torch.empty(n, n, dtype=torch.float64, device="cuda").uniform_(-1.0, 1.0, generator=gen)
        A = (G @ G.T + n * torch.eye(n, dtype=torch.float64, device="cuda")).T.contiguous()
        origs.append(A.clone())
        mats.append(A)
    info = torch.zeros(len(sizes), dtype=torch.int32, device="cuda")
    # the library's streams do not order with torch's: the operands must be
    # complete before the calls start
    torch.cuda.synchronize()
    server = g.Server(0, slots=4) if mode != "plain" else None
    try:
        r = g.cholesky_trace(server, 0, sizes, nbs, [m.data_ptr() for m in mats], info.data_ptr(),
                             mode == "ozaki")
    finally:
        if server:
            server.close()
    assert r["first_error"] == 0
    assert int((info != 0).sum()) == 0
    expect = 0
    for n, nb in zip(sizes, nbs):
        steps = (n + nb - 1) // nb
        for s in range(steps):
            rest = steps - s - 1
            expect += 1 + (1 if rest else 0) + rest + max(rest - 1, 0)
    assert r["calls"] == expect
    assert len(r["thread_finish_s"]) == len(sizes) and max(r["thread_finish_s"]) <= r["wall_s"] + 1e-3
    for n, A, A0 in zip(sizes, mats, origs):
        # column-major storage: the lower triangle of the n x n matrix is the
        # upper triangle of the row-major view
        Lm = torch.tril(A.T)
        R = torch.tril(Lm @ Lm.T - A0.T)
        assert float(R.norm() / torch.tril(A0.T).norm()) <= (1e-14 if mode != "ozaki" else 1e-13)
