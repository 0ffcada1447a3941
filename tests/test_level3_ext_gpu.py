"""GPU parity of the Level-3 set beyond D/Z GEMM, DSYRK, DTRSM, DTRMM: S/C
GEMM, xSYMM, xHEMM, xSYRK, xHERK, xSYR2K, xHER2K and S/C/Z TRMM, TRSM,
through the Fortran symbols on host arrays (staged) and on device memory
(in place), against the complex-double oracle.  Tolerances: relative
Frobenius error 1e-13 (D, Z) and 2e-5 (S, C).  Entries of C outside the
updated triangle must come back unchanged (bit for bit).
"""
import ctypes as C

import numpy as np
import pytest

from tests import l3cases as L3

pytestmark = pytest.mark.gpu
CASES = L3.cases()


@pytest.mark.parametrize("case", CASES, ids=[L3.case_id(c) for c in CASES])
def test_fortran_symbols_match_oracle(orc, f77, case):
    d = L3.inputs(case, seed=11)
    ref = L3.run_oracle(orc, case, {k: v.copy(order="F") for k, v in d.items()})
    got = {k: v.copy(order="F") for k, v in d.items()}
    L3.run_f77(f77, case, got)
    key = L3.out_key(case)
    err = L3.rel_err(got[key], ref)
    assert err <= L3.TOL[case["p"]], (L3.case_id(case), err)
    if case["r"] in ("syrk", "herk", "syr2k", "her2k") and case["n"] > 0:
        n = case["n"]
        other = np.triu(np.ones((n, n), bool), 1) if case["uplo"] == "L" else np.tril(np.ones((n, n), bool), -1)
        assert np.array_equal(got["c"][:n, :n][other], d["c"][:n, :n][other])
    # rows of the leading dimension below the matrix are never written
    m = case.get("m", case.get("n"))
    assert np.array_equal(got[key][m:], d[key][m:])


@pytest.mark.parametrize("p", "sdcz")
def test_device_resident_operands(orc, f77, p):
    import torch
    # symm on device memory: the Fortran symbol uses the operands in place
    c = dict(r="symm", p=p, side="R", uplo="L", m=130, n=70, ab=L3.scalars(p)[0])
    d = L3.inputs(c, seed=5)
    ref = L3.run_oracle(orc, c, {k: v.copy(order="F") for k, v in d.items()})
    tdt = {"s": torch.float32, "d": torch.float64, "c": torch.complex64, "z": torch.complex128}[p]
    dev = {k: torch.from_numpy(np.ascontiguousarray(v.T)).to("cuda", tdt) for k, v in d.items()}
    f77.symm(p, "R", "L", 130, 70, c["ab"][0], dev["a"].data_ptr(), d["a"].shape[0], dev["b"].data_ptr(),
             d["b"].shape[0], c["ab"][1], dev["c"].data_ptr(), d["c"].shape[0])
    torch.cuda.synchronize()
    got = dev["c"].cpu().numpy().T
    assert L3.rel_err(got, ref) <= L3.TOL[p]


@pytest.mark.parametrize("p", "sdcz")
def test_large_rank_k_update(orc, f77, p):
    # multi-tile triangular grid (n = 300 spans several 128/64 tiles)
    r = "herk" if p in "cz" else "syrk"
    c = dict(r=r, p=p, uplo="U", trans="N", n=300, k=200, ab=(0.5, 2.0))
    d = L3.inputs(c, seed=9)
    ref = L3.run_oracle(orc, c, {k: v.copy(order="F") for k, v in d.items()})
    L3.run_f77(f77, c, d)
    assert L3.rel_err(d["c"], ref) <= L3.TOL[p] * 4


@pytest.mark.parametrize("p", "scz")
def test_large_trsm(orc, f77, p):
    # recursion over several 64-blocks, both sides
    for side in "LR":
        c = dict(r="trsm", p=p, side=side, uplo="L", ta="C" if p in "cz" else "T", diag="N", m=300, n=190,
                 ab=(L3.scalars(p)[0][0], None))
        d = L3.inputs(c, seed=13)
        ref = L3.run_oracle(orc, c, {k: v.copy(order="F") for k, v in d.items()})
        L3.run_f77(f77, c, d)
        assert L3.rel_err(d["b"], ref) <= L3.TOL[p] * 10, (p, side)


def _cb(lib, name):
    return getattr(lib, "cblas_" + name)


@pytest.mark.parametrize("p", "sdcz")
def test_cblas_row_major_equals_column_major(lib, f77, p):
    """Row-major CBLAS = the column-major routine on the transposed problem."""
    rng = np.random.default_rng(21)
    dt = L3.DT[p]
    cplx = p in "cz"

    def rnd(*shape):
        a = rng.uniform(-1, 1, shape)
        if cplx:
            a = a + 1j * rng.uniform(-1, 1, shape)
        return a.astype(dt)

    def sc(v, real=False):
        if p in "sd" or real:
            return (C.c_float if p in "sc" else C.c_double)(v.real if isinstance(v, complex) else v)
        return np.array([v], dtype=dt).ctypes.data_as(C.c_void_p)

    keep = []

    def ptr(a):
        keep.append(a)
        return a.ctypes.data_as(C.c_void_p)

    al, be = (1.25 - 0.5j, 0.5 + 0.25j) if cplx else (1.25, 0.5)
    tol = L3.TOL[p] * 10
    # symm: row-major C (m x n) = A (m x m, symmetric, lower stored row-major) B
    m, n = 23, 17
    A, B, C0 = rnd(m, m), rnd(m, n), rnd(m, n)
    name = ("hemm" if cplx else "symm")
    Ar = np.ascontiguousarray(A)
    Cr = np.ascontiguousarray(C0.copy())
    _cb(lib, p + name)(101, 141, 122, m, n, sc(al), ptr(Ar), m, ptr(np.ascontiguousarray(B)), n, sc(be), ptr(Cr), n)
    Af = np.asfortranarray(A)
    Cf = np.asfortranarray(C0.copy())
    f77.symm(p, "L", "L", m, n, al, Af, m, np.asfortranarray(B), m, be, Cf, m, herm=cplx)
    assert np.linalg.norm(Cr - Cf) <= tol * np.linalg.norm(Cf)
    # syrk / herk: row-major C = A A^T (A n x k row-major), upper
    n, k = 19, 11
    A, C0 = rnd(n, k), rnd(n, n)
    name = "herk" if cplx else "syrk"
    alr, ber = (0.75, 1.5)
    Cr = np.ascontiguousarray(C0.copy())
    _cb(lib, p + name)(101, 121, 111, n, k, sc(alr, True) if cplx else sc(alr), ptr(np.ascontiguousarray(A)), k,
                       sc(ber, True) if cplx else sc(ber), ptr(Cr), n)
    Cf = np.asfortranarray(C0.copy())
    f77.syrk(p, "U", "N", n, k, alr, np.asfortranarray(A), n, ber, Cf, n, herm=cplx)
    iu = np.triu_indices(n)
    assert np.linalg.norm(Cr[iu] - Cf[iu]) <= tol * np.linalg.norm(Cf[iu])
    # trsm: row-major B (m x n) := alpha * inv(A) B, A lower m x m
    m, n = 21, 9
    A = (rnd(m, m) / m + np.eye(m) * 2).astype(dt)
    B0 = rnd(m, n)
    Br = np.ascontiguousarray(B0.copy())
    _cb(lib, p + "trsm")(101, 141, 122, 111, 131, m, n, sc(al), ptr(np.ascontiguousarray(A)), m, ptr(Br), n)
    Bf = np.asfortranarray(B0.copy())
    f77.trxm(p, "trsm", "L", "L", "N", "N", m, n, al, np.asfortranarray(A), m, Bf, m)
    assert np.linalg.norm(Br - Bf) <= tol * np.linalg.norm(Bf)
