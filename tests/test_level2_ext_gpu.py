"""GPU parity of DGER, DSYMV and DTRSV (Fortran symbols on host arrays, and
the device C ABI in place) against the oracle.  Tolerances: DGER 1e-15
absolute on entries of size ~1 (one FMA per element), DSYMV 1e-13 relative,
DTRSV residual ||op(A) x - b|| / (||A|| ||x||) <= 1e-14 plus 1e-12 relative
to the oracle on well-conditioned triangles (diagonal in [1, 2],
off-diagonal uniform / n)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def vec(rng, n, inc):
    return rng.uniform(-1, 1, 1 + (n - 1) * abs(inc))


def tri_matrix(rng, n, ld):
    a = np.asfortranarray(rng.uniform(-1, 1, (ld, n)) / n)
    for i in range(n):
        a[i, i] = rng.uniform(1, 2)
    return a


@pytest.mark.parametrize("m,n", [(1, 1), (37, 23), (1000, 333), (4099, 70)])
@pytest.mark.parametrize("inc", [(1, 1), (2, -3)])
def test_dger(orc, f77, m, n, inc):
    rng = np.random.default_rng(m + n)
    x, y = vec(rng, m, inc[0]), vec(rng, n, inc[1])
    if n > 2:
        y[2 * abs(inc[1])] = 0.0
    a = np.asfortranarray(rng.uniform(-1, 1, (m + 1, n)))
    if n > 2:   # a column whose y_j is 0 keeps its contents even where x is inf
        x[0] = np.inf
    ref, got = a.copy(order="F"), a.copy(order="F")
    orc.dger(m, n, -0.5, x, inc[0], y, inc[1], ref)
    f77.dger(m, n, -0.5, x, inc[0], y, inc[1], got, m + 1)
    assert np.array_equal(np.isfinite(got), np.isfinite(ref))
    fin = np.isfinite(ref)
    assert np.max(np.abs(got[fin] - ref[fin])) <= 1e-15 * 4


@pytest.mark.parametrize("n", [1, 63, 64, 65, 300, 2049])
@pytest.mark.parametrize("uplo", "UL")
def test_dsymv(orc, f77, n, uplo):
    rng = np.random.default_rng(n)
    a = np.asfortranarray(rng.uniform(-1, 1, (n + 3, n)))
    for incx, incy in [(1, 1), (-2, 3)]:
        x, y = vec(rng, n, incx), vec(rng, n, incy)
        for al, be in [(1.25, 0.5), (0.0, 2.0), (1.0, 0.0)]:
            ref, got = y.copy(), y.copy()
            orc.dsymv(uplo, n, al, a, x, incx, be, ref, incy)
            f77.dsymv(uplo, n, al, a, n + 3, x, incx, be, got, incy)
            assert np.linalg.norm(got - ref) <= 1e-13 * max(1.0, np.linalg.norm(ref)), (incx, al, be)


@pytest.mark.parametrize("n", [1, 64, 129, 1000])
@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("trans", "NT")
@pytest.mark.parametrize("diag", "NU")
def test_dtrsv(orc, f77, n, uplo, trans, diag):
    rng = np.random.default_rng(n * 7 + ord(uplo))
    a = tri_matrix(rng, n, n + 2)
    for inc in (1, -2):
        b = vec(rng, n, inc)
        ref, got = b.copy(), b.copy()
        orc.dtrsv(uplo, trans, diag, n, a, ref, inc)
        f77.dtrsv(uplo, trans, diag, n, a, n + 2, got, inc)
        assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref), inc
        if inc < 0:   # stride gaps untouched
            gaps = np.ones(b.size, bool)
            gaps[::abs(inc)] = False
            assert np.array_equal(got[gaps], b[gaps])


def test_dtrsv_large_residual(f77):
    # 64-row steps across n = 6000: backward error of the blocked substitution
    rng = np.random.default_rng(99)
    n = 6000
    a = tri_matrix(rng, n, n)
    b = rng.uniform(-1, 1, n)
    for uplo, trans in [("L", "N"), ("U", "T"), ("U", "N"), ("L", "T")]:
        x = b.copy()
        f77.dtrsv(uplo, trans, "N", n, a, n, x, 1)
        t = np.tril(a) if uplo == "L" else np.triu(a)
        if trans == "T":
            t = t.T
        res = np.linalg.norm(t @ x - b) / (np.linalg.norm(t) * np.linalg.norm(x))
        assert res <= 1e-14, (uplo, trans, res)


def test_device_abi_in_place(orc, dev):
    import torch
    rng = np.random.default_rng(4)
    n = 777
    a = tri_matrix(rng, n, n)
    b = rng.uniform(-1, 1, n)
    ref = b.copy()
    orc.dtrsv("L", "N", "N", n, a, ref, 1)
    A = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
    X = torch.from_numpy(b.copy()).cuda()
    st = dev.L.gbx_dtrsv(dev.ctx, b"L", b"N", b"N", n, C.c_void_p(A.data_ptr()), n, C.c_void_p(X.data_ptr()), 1)
    assert st == 0
    dev.sync()
    assert np.linalg.norm(X.cpu().numpy() - ref) <= 1e-12 * np.linalg.norm(ref)


def test_cblas_row_major(lib, f77):
    rng = np.random.default_rng(8)
    m, n = 19, 13
    x, y = rng.uniform(-1, 1, m), rng.uniform(-1, 1, n)
    a = rng.uniform(-1, 1, (m, n))
    ar = np.ascontiguousarray(a.copy())
    lib.cblas_dger(101, m, n, C.c_double(0.5), x.ctypes.data_as(C.c_void_p), 1, y.ctypes.data_as(C.c_void_p), 1,
                   ar.ctypes.data_as(C.c_void_p), n)
    assert np.allclose(ar, a + 0.5 * np.outer(x, y), rtol=1e-14, atol=1e-15)
    s = rng.uniform(-1, 1, (n, n))
    sym = np.tril(s) + np.tril(s, -1).T
    xv, yv = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    sr = np.ascontiguousarray(s)
    out = yv.copy()
    lib.cblas_dsymv(101, 122, n, C.c_double(1.5), sr.ctypes.data_as(C.c_void_p), n, xv.ctypes.data_as(C.c_void_p),
                    1, C.c_double(0.25), out.ctypes.data_as(C.c_void_p), 1)
    assert np.allclose(out, 1.5 * sym @ xv + 0.25 * yv, rtol=1e-13)
    t = tri_matrix(rng, n, n)
    tr = np.ascontiguousarray(t)
    xb = rng.uniform(-1, 1, n)
    xs = xb.copy()
    lib.cblas_dtrsv(101, 122, 112, 131, n, tr.ctypes.data_as(C.c_void_p), n, xs.ctypes.data_as(C.c_void_p), 1)
    assert np.allclose(np.tril(t).T @ xs, xb, rtol=1e-12, atol=1e-13)
