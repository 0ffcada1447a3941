"""Grouped execution (one persistent kernel for many small uneven calls).

A mix of DGEMMs (M, N, K log-uniform in [8, 300], all transposition pairs,
alpha/beta) and DTRSMs (order log-uniform in [8, 256], 16 right-hand sides,
all side/uplo/trans/diag) runs as one plan, directly and as a replayed CUDA
graph.  Every operation's result must match the oracle (relative error
<= 1e-13) and the same operation issued alone through gbx_dgemm/gbx_dtrsm;
each TRSM also has a backward residual <= 1e-14.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def loguni(rng, lo, hi):
    return int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))


class Mix:
    def __init__(self, orc, ngemm, ntrsm, seed):
        import torch
        import libgpublas_gb300 as g
        rng = np.random.default_rng(seed)
        self.specs = []
        host_chunks = []
        off = 0

        def place(a):
            nonlocal off
            a = np.asfortranarray(a)
            host_chunks.append(a.ravel(order="F"))
            start = off
            off += a.size + (-a.size % 4)   # keep 32-byte alignment
            if a.size % 4:
                host_chunks.append(np.zeros(-a.size % 4))
            return start

        s = seed
        for i in range(ngemm + ntrsm):
            if i % 5 == 4 and ntrsm:
                order, nrhs = loguni(rng, 8, 256), 16
                side = "LR"[rng.integers(2)]
                uplo, ta, diag = "LU"[rng.integers(2)], "NT"[rng.integers(2)], "NU"[rng.integers(2)]
                m, n = (order, nrhs) if side == "L" else (nrhs, order)
                a, s = orc.trsm_matrix(order, s)
                b, s = orc.matrix(m, n, s)
                self.specs.append(dict(kind=2, side=side, uplo=uplo, ta=ta, diag=diag, m=m, n=n,
                                       alpha=1.25, a=a, b=b, oa=place(a), ob=place(b)))
            else:
                m, n, k = loguni(rng, 8, 300), loguni(rng, 8, 300), loguni(rng, 8, 300)
                ta, tb = "NT"[rng.integers(2)], "NT"[rng.integers(2)]
                ra, ca = (m, k) if ta == "N" else (k, m)
                rb, cb = (k, n) if tb == "N" else (n, k)
                a, s = orc.matrix(ra, ca, s)
                b, s = orc.matrix(rb, cb, s)
                c, s = orc.matrix(m, n, s)
                beta = [0.0, 0.5, 1.0][rng.integers(3)]
                self.specs.append(dict(kind=1, ta=ta, tb=tb, m=m, n=n, k=k, alpha=-0.75, beta=beta,
                                       a=a, b=b, c=c, oa=place(a), ob=place(b), oc=place(c)))
        self.host = np.concatenate(host_chunks)
        self.dev = torch.from_numpy(self.host).cuda()
        base = self.dev.data_ptr()
        self.ops = []
        for sp in self.specs:
            if sp["kind"] == 1:
                self.ops.append(g.GbxOp(kind=1, transa=sp["ta"].encode(), transb=sp["tb"].encode(),
                                        m=sp["m"], n=sp["n"], k=sp["k"], alpha=sp["alpha"],
                                        beta=sp["beta"], A=base + 8 * sp["oa"], lda=sp["a"].shape[0],
                                        B=base + 8 * sp["ob"], ldb=sp["b"].shape[0],
                                        C=base + 8 * sp["oc"], ldc=sp["c"].shape[0]))
            else:
                self.ops.append(g.GbxOp(kind=2, transa=sp["ta"].encode(), side=sp["side"].encode(),
                                        uplo=sp["uplo"].encode(), diag=sp["diag"].encode(),
                                        m=sp["m"], n=sp["n"], alpha=sp["alpha"],
                                        A=base + 8 * sp["oa"], lda=sp["a"].shape[0],
                                        C=base + 8 * sp["ob"], ldc=sp["b"].shape[0]))

    def reset(self):
        import torch
        self.dev.copy_(torch.from_numpy(self.host))
        torch.cuda.synchronize()

    def result(self, sp):
        h = self.dev.cpu().numpy()
        if sp["kind"] == 1:
            return h[sp["oc"]: sp["oc"] + sp["c"].size].reshape(sp["c"].shape, order="F")
        return h[sp["ob"]: sp["ob"] + sp["b"].size].reshape(sp["b"].shape, order="F")


def check(orc, mix, results):
    for sp, got in zip(mix.specs, results):
        if sp["kind"] == 1:
            want = sp["c"].copy(order="F")
            orc.dgemm(sp["ta"], sp["tb"], sp["m"], sp["n"], sp["k"], sp["alpha"], sp["a"], sp["b"],
                      sp["beta"], want)
        else:
            want = sp["b"].copy(order="F")
            orc.dtrsm(sp["side"], sp["uplo"], sp["ta"], sp["diag"], sp["m"], sp["n"], sp["alpha"],
                      sp["a"], want)
            res = orc.dtrsm_residual(sp["side"], sp["uplo"], sp["ta"], sp["diag"], sp["m"], sp["n"],
                                     sp["alpha"], sp["a"], sp["b"], np.asfortranarray(got))
            assert res <= 1e-14, sp
        err = np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-300)
        assert err <= 1e-13, (sp["kind"], sp.get("m"), sp.get("n"), err)


def test_grouped_plan_matches_oracle(orc, dev):
    mix = Mix(orc, ngemm=200, ntrsm=60, seed=7)
    plan = dev.plan_create(mix.ops)
    try:
        items, flops = dev.plan_info(plan)
        assert items >= len(mix.ops) and flops > 0
        for graph in (False, True, True):
            mix.reset()
            dev.plan_launch(plan, graph=graph)
            dev.sync()
            h = mix.dev.cpu().numpy()
            mix.host_result = h
            check(orc, mix, [mix.result(sp) for sp in mix.specs])
    finally:
        dev.plan_destroy(plan)


def test_grouped_plan_equals_per_call(orc, dev):
    mix = Mix(orc, ngemm=60, ntrsm=20, seed=8)
    plan = dev.plan_create(mix.ops)
    mix.reset()
    dev.plan_launch(plan)
    dev.sync()
    grouped = [mix.result(sp).copy() for sp in mix.specs]
    dev.plan_destroy(plan)
    mix.reset()
    for op in mix.ops:
        if op.kind == 1:
            dev.dgemm_checked(op.transa, op.transb, op.m, op.n, op.k, op.alpha, op.A, op.lda, op.B,
                              op.ldb, op.beta, op.C, op.ldc)
        else:
            dev.dtrsm(op.side, op.uplo, op.transa, op.diag, op.m, op.n, op.alpha, op.A, op.lda, op.C,
                      op.ldc)
    dev.sync()
    for sp, g in zip(mix.specs, grouped):
        single = mix.result(sp)
        assert np.linalg.norm(g - single) <= 1e-13 * max(np.linalg.norm(single), 1e-300)


def test_grouped_plan_rejects_bad_ops(dev):
    import libgpublas_gb300 as g
    with pytest.raises(g.GbxError, match="parameter 8"):
        dev.plan_create([g.GbxOp(kind=1, transa=b"N", transb=b"N", m=10, n=10, k=10, alpha=1.0,
                                 A=1 << 20, lda=5, B=1 << 20, ldb=10, C=1 << 20, ldc=10)])
    with pytest.raises(g.GbxError, match="order"):
        dev.plan_create([g.GbxOp(kind=2, transa=b"N", side=b"L", uplo=b"L", diag=b"N", m=300, n=4,
                                 alpha=1.0, A=1 << 20, lda=300, C=1 << 20, ldc=300)])
