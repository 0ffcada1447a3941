"""Generate tests/golden/blas_golden.npz from the CPU BLAS.

The reference's runnable BLAS path ends in the CPU BLAS it reaches with
dlsym(RTLD_NEXT) (runtime-blas.c:60-69, gemm.cc:129-141).  This script runs
that CPU BLAS (SciPy's bundled OpenBLAS, LP64) on seeded inputs and stores
its outputs.  Inputs are NOT stored: they are regenerated from the seeds with
the oracle's SplitMix64 generator, and a checksum of each input set is stored
so a generator change is detected.

Run:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import cpublas  # noqa: E402

OUT = os.path.join(HERE, "blas_golden.npz")


def checksum(*arrays):
    return float(sum(np.sum(np.abs(a) * (1 + np.arange(a.size).reshape(a.shape, order="F") % 7))
                     for a in arrays))


def cases():
    """Yield (name, dict of arrays/scalars) -- also used by the tests."""
    orc = oracle.get()
    out = []

    # DGEMM, small, all transposition pairs
    m, n, k = 13, 11, 17
    for ta in "NT":
        for tb in "NT":
            ra, ca = (m, k) if ta == "N" else (k, m)
            rb, cb = (k, n) if tb == "N" else (n, k)
            a, s = orc.matrix(ra, ca, 1001)
            b, s = orc.matrix(rb, cb, s)
            c, s = orc.matrix(m, n, s)
            out.append((f"dgemm_{ta}{tb}", dict(kind="dgemm", ta=ta, tb=tb, m=m, n=n, k=k,
                                                  alpha=1.5, beta=0.5, seed=1001, a=a, b=b, c=c)))
    # DGEMM config 1: 512^3 NN alpha=1 beta=0.5 seed 0 (stored as samples)
    out.append(("dgemm_cfg1", dict(kind="dgemm_cfg1", seed=0)))
    # ZGEMM
    for ta, tb in (("N", "N"), ("C", "N"), ("T", "C")):
        m, n, k = 7, 6, 5
        ra, ca = (m, k) if ta == "N" else (k, m)
        rb, cb = (k, n) if tb == "N" else (n, k)
        ar, s = orc.matrix(ra, ca, 2001)
        ai, s = orc.matrix(ra, ca, s)
        br, s = orc.matrix(rb, cb, s)
        bi, s = orc.matrix(rb, cb, s)
        cr, s = orc.matrix(m, n, s)
        ci, s = orc.matrix(m, n, s)
        out.append((f"zgemm_{ta}{tb}", dict(kind="zgemm", ta=ta, tb=tb, m=m, n=n, k=k,
                                              alpha=0.5 - 1.25j, beta=0.25 + 0.5j, seed=2001,
                                              a=np.asfortranarray(ar + 1j * ai),
                                              b=np.asfortranarray(br + 1j * bi),
                                              c=np.asfortranarray(cr + 1j * ci))))
    # DSYRK
    for uplo in "LU":
        for trans in "NT":
            n, k = 12, 9
            ra, ca = (n, k) if trans == "N" else (k, n)
            a, s = orc.matrix(ra, ca, 3001)
            c, s = orc.matrix(n, n, s)
            out.append((f"dsyrk_{uplo}{trans}", dict(kind="dsyrk", uplo=uplo, trans=trans, n=n,
                                                      k=k, alpha=-0.75, beta=1.25, seed=3001,
                                                      a=a, c=c)))
    # DTRSM / DTRMM, all 16 option combinations
    for kind in ("dtrsm", "dtrmm"):
        for side in "LR":
            for uplo in "LU":
                for ta in "NT":
                    for diag in "NU":
                        m, n = 9, 7
                        na = m if side == "L" else n
                        a, s = orc.trsm_matrix(na, 4001)
                        b, s = orc.matrix(m, n, s)
                        out.append((f"{kind}_{side}{uplo}{ta}{diag}",
                                    dict(kind=kind, side=side, uplo=uplo, ta=ta, diag=diag, m=m,
                                         n=n, alpha=1.5, seed=4001, a=a, b=b)))
    # DGEMV
    for trans in "NT":
        for incx, incy in ((1, 1), (2, -1)):
            m, n = 10, 8
            a, s = orc.matrix(m, n, 5001)
            lx, ly = (n, m) if trans == "N" else (m, n)
            x, s = orc.uniform(lx * abs(incx), s)
            y, s = orc.uniform(ly * abs(incy), s)
            out.append((f"dgemv_{trans}_{incx}_{incy}",
                        dict(kind="dgemv", trans=trans, m=m, n=n, alpha=0.75, beta=-0.5,
                             incx=incx, incy=incy, seed=5001, a=a, x=x, y=y)))
    # Level 1
    for incx, incy in ((1, 1), (3, -2)):
        n = 100
        x, s = orc.uniform(n * abs(incx), 6001)
        y, s = orc.uniform(n * abs(incy), s)
        out.append((f"daxpy_{incx}_{incy}", dict(kind="daxpy", n=n, alpha=-1.5, incx=incx,
                                                  incy=incy, seed=6001, x=x, y=y)))
        out.append((f"ddot_{incx}_{incy}", dict(kind="ddot", n=n, incx=incx, incy=incy,
                                                 seed=6001, x=x, y=y)))
    for scale in (1.0, 1e300, 1e-300):
        x, _ = orc.uniform(257, 7001)
        out.append((f"dnrm2_{scale:g}", dict(kind="dnrm2", n=257, incx=1, seed=7001,
                                              scale=scale, x=x * scale)))
    # i?amax: config 1 (n = 2^20, duplicate maximum) and a coarse tie-heavy vector
    n = 1 << 20
    x, _ = orc.uniform(n, 0)
    x[123457], x[987654] = 1.5, -1.5
    out.append(("idamax_cfg1", dict(kind="iamax", n=n, incx=1, seed=0, x=x)))
    x, _ = orc.uniform(4000, 8001)
    out.append(("iamax_ties", dict(kind="iamax", n=2000, incx=2, seed=8001,
                                   x=np.round(x * 16) / 16)))
    return out


def run_cpu(cb, name, d):
    """Outputs of the CPU BLAS for one case."""
    kind = d["kind"]
    if kind == "dgemm":
        c = d["c"].copy(order="F")
        cb.dgemm(d["ta"], d["tb"], d["m"], d["n"], d["k"], d["alpha"], d["a"], d["b"], d["beta"], c)
        return {"out": c}
    if kind == "dgemm_cfg1":
        orc = oracle.get()
        a, s = orc.matrix(512, 512, 0)
        b, s = orc.matrix(512, 512, s)
        c, s = orc.matrix(512, 512, s)
        cb.dgemm("N", "N", 512, 512, 512, 1.0, a, b, 0.5, c)
        rows = (np.arange(256) * 2654435761) % 512
        cols = (np.arange(256) * 40503) % 512
        return {"colsum": c.sum(axis=0), "sample": c[rows, cols], "rows": rows, "cols": cols,
                "fro": np.linalg.norm(c)}
    if kind == "zgemm":
        c = d["c"].copy(order="F")
        cb.zgemm(d["ta"], d["tb"], d["m"], d["n"], d["k"], d["alpha"], d["a"], d["b"], d["beta"], c)
        return {"out": c}
    if kind == "dsyrk":
        c = d["c"].copy(order="F")
        cb.dsyrk(d["uplo"], d["trans"], d["n"], d["k"], d["alpha"], d["a"], d["beta"], c)
        return {"out": c}
    if kind in ("dtrsm", "dtrmm"):
        b = d["b"].copy(order="F")
        getattr(cb, kind)(d["side"], d["uplo"], d["ta"], d["diag"], d["m"], d["n"], d["alpha"],
                          d["a"], b)
        return {"out": b}
    if kind == "dgemv":
        y = d["y"].copy()
        cb.dgemv(d["trans"], d["m"], d["n"], d["alpha"], d["a"], d["x"], d["incx"], d["beta"], y,
                 d["incy"])
        return {"out": y}
    if kind == "daxpy":
        y = d["y"].copy()
        cb.daxpy(d["n"], d["alpha"], d["x"], d["incx"], y, d["incy"])
        return {"out": y}
    if kind == "ddot":
        return {"out": np.array(cb.ddot(d["n"], d["x"], d["incx"], d["y"], d["incy"]))}
    if kind == "dnrm2":
        return {"out": np.array(cb.dnrm2(d["n"], d["x"], d["incx"]))}
    if kind == "iamax":
        return {"amax": np.array(cb.idamax(d["n"], d["x"], d["incx"])),
                "amin": np.array(cb.idamin(d["n"], d["x"], d["incx"]))}
    raise ValueError(kind)


def input_checksum(d):
    arrs = [v for v in d.values() if isinstance(v, np.ndarray)]
    return checksum(*arrs) if arrs else 0.0


def main():
    cb = cpublas.get()
    store = {"_blas": np.array(cb.config)}
    for name, d in cases():
        res = run_cpu(cb, name, d)
        for key, val in res.items():
            store[f"{name}/{key}"] = np.asarray(val)
        store[f"{name}/input_checksum"] = np.array(input_checksum(d))
    np.savez_compressed(OUT, **store)
    print(f"wrote {OUT}: {len(store)} arrays from {cb.config}")


if __name__ == "__main__":
    main()
