"""Cases for the Level-3 routines beyond D/Z GEMM, DSYRK, DTRSM, DTRMM:
S/C GEMM, xSYMM, xHEMM, xSYRK, xHERK, xSYR2K, xHER2K, xTRMM and xTRSM in the
precisions the reference exports (blas_level3/*.cc, prototypes
blas.h:202-314).

One case = routine family, precision prefix, option letters, sizes and
scalars.  ``inputs`` draws seeded operands; ``run_f77`` calls our Fortran
symbol on host arrays; ``run_oracle`` evaluates the complex-double
restatement in oracle/oracle.c; ``run_cpu`` calls the CPU BLAS (the library
the reference forwards to) through its Fortran symbol.
"""
import ctypes as C
import itertools

import numpy as np

DT = {"s": np.float32, "d": np.float64, "c": np.complex64, "z": np.complex128}
# relative Frobenius tolerance against the complex-double oracle
TOL = {"s": 2e-5, "d": 1e-13, "c": 2e-5, "z": 1e-13}
TR_N, TR_T, TR_C = 1, 2, 4


def allowed(routine, p):
    if routine in ("herk", "her2k"):
        return TR_N | TR_C
    if p in "cz":
        return TR_N | TR_T
    return TR_N | TR_T | TR_C


def letter_set(mask):
    return [ch for ch, bit in (("N", TR_N), ("T", TR_T), ("C", TR_C)) if mask & bit]


def scalars(p, herm_real=False):
    if p in "sd" or herm_real:
        return [(1.5, 0.5), (-0.75, 0.0), (0.0, 2.0), (1.0, 1.0)]
    return [(1.5 - 0.5j, 0.5 + 1.0j), (-0.75 + 0.25j, 0.0), (0.0, 2.0 - 1.0j), (1.0, 1.0)]


def cases():
    out = []
    for p in "sc":
        for ta, tb in itertools.product("NTC", "NTC"):
            out.append(dict(r="gemm", p=p, ta=ta, tb=tb, m=37, n=29, k=41, ab=scalars(p)[0]))
        for ab in scalars(p)[1:]:
            out.append(dict(r="gemm", p=p, ta="N", tb="N", m=65, n=70, k=33, ab=ab))
    for p in "sdcz":
        routines = ["symm"] + (["hemm"] if p in "cz" else [])
        for r, side, uplo in itertools.product(routines, "LR", "UL"):
            out.append(dict(r=r, p=p, side=side, uplo=uplo, m=33, n=47, ab=scalars(p)[0]))
        out.append(dict(r="symm", p=p, side="L", uplo="L", m=20, n=24, ab=scalars(p)[2]))
        for r in ["syrk", "syr2k"] + (["herk", "her2k"] if p in "cz" else []):
            herm = r in ("herk", "her2k")
            for uplo, tr in itertools.product("UL", letter_set(allowed(r, p))):
                ab = scalars(p, herm_real=(r == "herk"))[0]
                if r == "her2k":
                    ab = (scalars(p)[0][0], 0.5)
                out.append(dict(r=r, p=p, uplo=uplo, trans=tr, n=45, k=31, ab=ab))
            ab = scalars(p, herm_real=herm)[2]
            out.append(dict(r=r, p=p, uplo="L", trans="N", n=30, k=0 if r.endswith("k") else 0, ab=ab))
        for r in ("trmm", "trsm"):
            if p == "d":
                continue
            for side, uplo, ta, diag in itertools.product("LR", "UL", "NTC", "NU"):
                out.append(dict(r=r, p=p, side=side, uplo=uplo, ta=ta, diag=diag, m=37, n=29,
                                ab=(scalars(p)[0][0], None)))
    for p in "sdcz":
        out.append(dict(r="symm", p=p, side="R", uplo="U", m=0, n=5, ab=scalars(p)[0]))
        out.append(dict(r="syr2k", p=p, uplo="U", trans="N", n=0, k=3, ab=scalars(p)[0]))
    return out


def case_id(c):
    keys = [c["r"], c["p"]] + [str(c[k]) for k in ("side", "uplo", "ta", "tb", "trans", "diag") if k in c]
    return "-".join(keys) + f"-{c.get('m', c.get('n'))}"


def _rand(rng, shape, p):
    a = rng.uniform(-1, 1, shape)
    if p in "cz":
        a = a + 1j * rng.uniform(-1, 1, shape)
    return np.asfortranarray(a.astype(DT[p]))


def inputs(c, seed=0):
    """Seeded operands (Fortran order, the routine's dtype) with padded ld."""
    rng = np.random.default_rng(seed)
    p, r = c["p"], c["r"]
    d = {}
    if r == "gemm":
        m, n, k = c["m"], c["n"], c["k"]
        ar, ac = (m, k) if c["ta"] == "N" else (k, m)
        br, bc = (k, n) if c["tb"] == "N" else (n, k)
        d["a"] = _rand(rng, (ar + 3, ac), p)
        d["b"] = _rand(rng, (br + 2, bc), p)
        d["c"] = _rand(rng, (m + 1, n), p)
    elif r in ("symm", "hemm"):
        m, n = c["m"], c["n"]
        na = m if c["side"] == "L" else n
        d["a"] = _rand(rng, (na + 2, na), p)
        d["b"] = _rand(rng, (m + 1, n), p)
        d["c"] = _rand(rng, (m + 3, n), p)
    elif r in ("syrk", "herk", "syr2k", "her2k"):
        n, k = c["n"], c["k"]
        ar, ac = (n, k) if c["trans"] == "N" else (k, n)
        d["a"] = _rand(rng, (max(ar, 1) + 2, ac), p)
        if r.endswith("2k"):
            d["b"] = _rand(rng, (max(ar, 1) + 1, ac), p)
        d["c"] = _rand(rng, (n + 2, n), p)
    else:   # trmm / trsm
        m, n = c["m"], c["n"]
        na = m if c["side"] == "L" else n
        a = _rand(rng, (na + 1, na), p) / na
        for i in range(na):   # well conditioned: diagonal of modulus in [1, 2]
            a[i, i] = rng.uniform(1, 2) * (1 if p in "sd" else np.exp(1j * rng.uniform(0, 6.28)))
        d["a"] = np.asfortranarray(a.astype(DT[p]))
        d["b"] = _rand(rng, (m + 2, n), p)
    return d


def out_key(c):
    return "b" if c["r"] in ("trmm", "trsm") else "c"


def run_f77(f77, c, d):
    p, r = c["p"], c["r"]
    al, be = c["ab"]
    a = d["a"]
    if r == "gemm":
        f77.gemm(p, c["ta"], c["tb"], c["m"], c["n"], c["k"], al, a, a.shape[0], d["b"], d["b"].shape[0], be,
                 d["c"], d["c"].shape[0])
    elif r in ("symm", "hemm"):
        f77.symm(p, c["side"], c["uplo"], c["m"], c["n"], al, a, a.shape[0], d["b"], d["b"].shape[0], be,
                 d["c"], d["c"].shape[0], herm=(r == "hemm"))
    elif r in ("syrk", "herk"):
        f77.syrk(p, c["uplo"], c["trans"], c["n"], c["k"], al, a, a.shape[0], be, d["c"], d["c"].shape[0],
                 herm=(r == "herk"))
    elif r in ("syr2k", "her2k"):
        f77.syr2k(p, c["uplo"], c["trans"], c["n"], c["k"], al, a, a.shape[0], d["b"], d["b"].shape[0], be,
                  d["c"], d["c"].shape[0], herm=(r == "her2k"))
    else:
        f77.trxm(p, r, c["side"], c["uplo"], c["ta"], c["diag"], c["m"], c["n"], al, a, a.shape[0], d["b"],
                 d["b"].shape[0])


def run_oracle(orc, c, d):
    """Returns the oracle's output array (complex128)."""
    p, r = c["p"], c["r"]
    al, be = c["ab"]
    z = {k: orc.z(v) for k, v in d.items()}
    if r == "gemm":
        orc.zgemm(c["ta"], c["tb"], c["m"], c["n"], c["k"], al, z["a"], z["b"], be, z["c"])
    elif r in ("symm", "hemm"):
        orc.zsymm(c["side"], c["uplo"], c["m"], c["n"], al, z["a"], z["b"], be, z["c"], herm=(r == "hemm"))
    elif r in ("syrk", "herk"):
        orc.zsyrk(c["uplo"], c["trans"], allowed(r, p), c["n"], c["k"], al, z["a"], be, z["c"],
                  herm=(r == "herk"))
    elif r in ("syr2k", "her2k"):
        orc.zsyr2k(c["uplo"], c["trans"], allowed(r, p), c["n"], c["k"], al, z["a"], z["b"], be, z["c"],
                   herm=(r == "her2k"))
    elif r == "trmm":
        orc.ztrmm(c["side"], c["uplo"], c["ta"], c["diag"], c["m"], c["n"], al, z["a"], z["b"])
    else:
        orc.ztrsm(c["side"], c["uplo"], c["ta"], c["diag"], c["m"], c["n"], al, z["a"], z["b"])
    return z[out_key(c)]


def rel_err(got, ref):
    got = np.asarray(got, dtype=np.complex128)
    den = np.linalg.norm(ref)
    return np.linalg.norm(got - ref) / (den if den > 0 else 1.0)


# ---- the CPU BLAS through its Fortran symbols ------------------------------
def _cptr(x):
    return x.ctypes.data_as(C.c_void_p)


def run_cpu(cpu, c, d):
    """Calls the CPU BLAS's Fortran symbol (prefixed scipy_ in SciPy's
    OpenBLAS) on the same operands, in place."""
    p, r = c["p"], c["r"]
    al, be = c["ab"]
    herm_real = r in ("herk",)
    sdt = DT[p] if not (herm_real or p in "sd") else (np.float32 if p in "sc" else np.float64)
    al_a = np.array([al], dtype=sdt if r != "her2k" else DT[p])
    be_dt = sdt if r not in ("her2k",) else (np.float32 if p == "c" else np.float64)
    be_a = np.array([be if be is not None else 0], dtype=be_dt)
    ch = lambda s: C.c_char_p(s.encode())   # noqa: E731
    ii = lambda v: C.byref(C.c_int(int(v)))   # noqa: E731
    f = cpu._f(p + r + "_")
    a = d["a"]
    if r == "gemm":
        f(ch(c["ta"]), ch(c["tb"]), ii(c["m"]), ii(c["n"]), ii(c["k"]), _cptr(al_a), _cptr(a), ii(a.shape[0]),
          _cptr(d["b"]), ii(d["b"].shape[0]), _cptr(be_a), _cptr(d["c"]), ii(d["c"].shape[0]))
    elif r in ("symm", "hemm"):
        f(ch(c["side"]), ch(c["uplo"]), ii(c["m"]), ii(c["n"]), _cptr(al_a), _cptr(a), ii(a.shape[0]),
          _cptr(d["b"]), ii(d["b"].shape[0]), _cptr(be_a), _cptr(d["c"]), ii(d["c"].shape[0]))
    elif r in ("syrk", "herk"):
        f(ch(c["uplo"]), ch(c["trans"]), ii(c["n"]), ii(c["k"]), _cptr(al_a), _cptr(a), ii(a.shape[0]),
          _cptr(be_a), _cptr(d["c"]), ii(d["c"].shape[0]))
    elif r in ("syr2k", "her2k"):
        f(ch(c["uplo"]), ch(c["trans"]), ii(c["n"]), ii(c["k"]), _cptr(al_a), _cptr(a), ii(a.shape[0]),
          _cptr(d["b"]), ii(d["b"].shape[0]), _cptr(be_a), _cptr(d["c"]), ii(d["c"].shape[0]))
    else:
        f(ch(c["side"]), ch(c["uplo"]), ch(c["ta"]), ch(c["diag"]), ii(c["m"]), ii(c["n"]), _cptr(al_a),
          _cptr(a), ii(a.shape[0]), _cptr(d["b"]), ii(d["b"].shape[0]))
    return d[out_key(c)]
