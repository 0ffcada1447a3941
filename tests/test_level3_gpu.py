"""Level-2/3 parity on the GPU through the Fortran ABI (host operands).

Stated tolerance for the plain FP64 routines: relative Frobenius error
<= 1e-13 against the double-double oracle (DGEMM/ZGEMM/DSYRK/DTRMM/DGEMV),
and a normwise backward residual <= 1e-14 for DTRSM.  Every operand lives
inside a larger buffer whose padding rows hold a sentinel that must survive
the call unchanged.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13
SENT = 12345.678


def padded(orc, rows, cols, seed, pad=3):
    ld = rows + pad
    a, s = orc.matrix(rows, cols, seed, ld=ld)
    a[rows:, :] = SENT
    return a, s


def rel(x, ref):
    d = np.linalg.norm(ref)
    return np.linalg.norm(x - ref) / (d if d > 0 else 1.0)


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T"), ("C", "n")])
@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (7, 33, 129), (129, 7, 33), (257, 130, 64),
                                   (300, 200, 517)])
def test_dgemm_shapes(orc, f77, ta, tb, m, n, k):
    ra, ca = (m, k) if ta.upper() == "N" else (k, m)
    rb, cb = (k, n) if tb.upper() == "N" else (n, k)
    a, s = padded(orc, ra, ca, 100 + m + n + k)
    b, s = padded(orc, rb, cb, s)
    c, s = padded(orc, m, n, s)
    for alpha, beta in [(1.0, 0.0), (1.5, 0.5), (-0.75, 1.0)]:
        ref = orc.dgemm_dd(ta, tb, m, n, k, alpha, a, b, beta, c)
        got = c.copy(order="F")
        f77.dgemm(ta, tb, m, n, k, alpha, a, a.shape[0], b, b.shape[0], beta, got, got.shape[0])
        assert rel(got[:m], ref[:m]) <= TOL
        assert np.all(got[m:] == SENT)


def test_dgemm_config1(orc, cpublas, f77):
    # dgemm_('N','N') M=N=K=512, ld=512, alpha=1, beta=0.5; A, B, C from seed 0
    n = 512
    a, s = orc.matrix(n, n, 0)
    b, s = orc.matrix(n, n, s)
    c, s = orc.matrix(n, n, s)
    ref = orc.dgemm_dd("N", "N", n, n, n, 1.0, a, b, 0.5, c)
    got = c.copy(order="F")
    f77.dgemm("N", "N", n, n, n, 1.0, a, n, b, n, 0.5, got, n)
    cpu = c.copy(order="F")
    cpublas.dgemm("N", "N", n, n, n, 1.0, a, b, 0.5, cpu)
    assert rel(got, ref) <= TOL
    assert rel(cpu, ref) <= TOL
    assert rel(got, cpu) <= 2 * TOL


def test_dgemm_beta_zero_clears_nan_and_quick_returns(orc, f77):
    m, n, k = 40, 30, 20
    a, s = orc.matrix(m, k, 3)
    b, s = orc.matrix(k, n, s)
    c = np.full((m, n), np.nan, order="F")
    f77.dgemm("N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c, m)
    assert np.all(np.isfinite(c))
    # alpha = 0, beta = 0 -> C = 0 (even NaN); alpha = 0, beta = 2 -> C *= 2
    c = np.full((m, n), np.nan, order="F")
    f77.dgemm("N", "N", m, n, k, 0.0, a, m, b, k, 0.0, c, m)
    assert np.all(c == 0.0)
    c2, _ = orc.matrix(m, n, 9)
    want = 2.0 * c2
    f77.dgemm("N", "N", m, n, 0, 1.0, a, m, b, 1, 2.0, c2, m)
    assert np.array_equal(c2, want)
    # beta = 1 with alpha = 0: untouched; m = 0: untouched
    c3, _ = orc.matrix(m, n, 10)
    keep = c3.copy()
    f77.dgemm("N", "N", m, n, k, 0.0, a, m, b, k, 1.0, c3, m)
    f77.dgemm("N", "N", 0, n, k, 1.0, a, m, b, k, 0.0, c3, m)
    assert np.array_equal(c3, keep)


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("C", "N"), ("N", "C"), ("T", "C"), ("C", "T")])
def test_zgemm(orc, f77, ta, tb):
    m, n, k = 67, 45, 91
    ra, ca = (m, k) if ta == "N" else (k, m)
    rb, cb = (k, n) if tb == "N" else (n, k)
    rng = np.random.default_rng(5)
    a = np.asfortranarray(rng.uniform(-1, 1, (ra, ca)) + 1j * rng.uniform(-1, 1, (ra, ca)))
    b = np.asfortranarray(rng.uniform(-1, 1, (rb, cb)) + 1j * rng.uniform(-1, 1, (rb, cb)))
    c = np.asfortranarray(rng.uniform(-1, 1, (m, n)) + 1j * rng.uniform(-1, 1, (m, n)))
    alpha, beta = 0.5 - 1.25j, 0.25 + 0.5j
    want = c.copy(order="F")
    orc.zgemm(ta, tb, m, n, k, alpha, a, b, beta, want)
    got = c.copy(order="F")
    f77.zgemm(ta, tb, m, n, k, alpha, a, ra, b, rb, beta, got, m)
    assert rel(got, want) <= TOL


@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("n,k", [(1, 5), (77, 33), (300, 129)])
def test_dsyrk(orc, f77, uplo, trans, n, k):
    ra, ca = (n, k) if trans == "N" else (k, n)
    a, s = padded(orc, ra, ca, 300 + n + k)
    c, _ = padded(orc, n, n, s)
    for alpha, beta in [(1.0, 0.0), (-0.5, 0.75)]:
        want = c.copy(order="F")
        orc.dsyrk(uplo, trans, n, k, alpha, a, beta, want)
        got = c.copy(order="F")
        f77.dsyrk(uplo, trans, n, k, alpha, a, a.shape[0], beta, got, got.shape[0])
        tri = np.tril if uplo == "L" else np.triu
        assert rel(tri(got[:n]), tri(want[:n])) <= TOL
        other = np.triu(np.ones((n, n)), 1) if uplo == "L" else np.tril(np.ones((n, n)), -1)
        assert np.array_equal(got[:n][other == 1], c[:n][other == 1])
        assert np.all(got[n:] == SENT)


SIDES = [(s, u, t, d) for s in "LR" for u in "LU" for t in "NT" for d in "NU"]


@pytest.mark.parametrize("side,uplo,ta,diag", SIDES)
def test_dtrmm(orc, f77, side, uplo, ta, diag):
    m, n = 150, 71
    na = m if side == "L" else n
    a, s = orc.trsm_matrix(na, 400 + ord(side) + ord(uplo))
    a = np.asfortranarray(a * 4.0)
    b, _ = padded(orc, m, n, s)
    want = b.copy(order="F")
    orc.dtrmm(side, uplo, ta, diag, m, n, 0.5, a, want)
    got = b.copy(order="F")
    f77.dtrmm(side, uplo, ta, diag, m, n, 0.5, a, na, got, got.shape[0])
    assert rel(got[:m], want[:m]) <= TOL
    assert np.all(got[m:] == SENT)


@pytest.mark.parametrize("side,uplo,ta,diag", SIDES)
@pytest.mark.parametrize("m,n", [(1, 3), (70, 33), (200, 130)])
def test_dtrsm(orc, f77, side, uplo, ta, diag, m, n):
    na = m if side == "L" else n
    a, s = orc.trsm_matrix(na, 500 + m + n + ord(side))
    b, _ = padded(orc, m, n, s)
    alpha = 1.5
    got = b.copy(order="F")
    f77.dtrsm(side, uplo, ta, diag, m, n, alpha, a, na, got, got.shape[0])
    resid = orc.dtrsm_residual(side, uplo, ta, diag, m, n, alpha, a, b, got)
    assert resid <= 1e-14
    want = b.copy(order="F")
    orc.dtrsm(side, uplo, ta, diag, m, n, alpha, a, want)
    assert rel(got[:m], want[:m]) <= TOL
    assert np.all(got[m:] == SENT)


def test_dtrsm_alpha_zero_and_errors(orc, f77, capfd):
    a, s = orc.trsm_matrix(20, 1)
    b = np.full((20, 5), np.nan, order="F")
    f77.dtrsm("L", "L", "N", "N", 20, 5, 0.0, a, 20, b, 20)
    assert np.all(b == 0.0)
    # invalid side -> xerbla with parameter 1, B untouched
    b2 = np.ones((20, 5), order="F")
    f77.dtrsm("X", "L", "N", "N", 20, 5, 1.0, a, 20, b2, 20)
    f77.dtrsm("L", "L", "N", "N", 20, 5, 1.0, a, 10, b2, 20)
    err = capfd.readouterr().err
    assert "DTRSM" in err and "parameter number  1" in err and "parameter number  9" in err
    assert np.all(b2 == 1.0)


@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("m,n", [(1, 1), (513, 77), (77, 1025), (1000, 1000)])
@pytest.mark.parametrize("incx,incy", [(1, 1), (2, -1)])
def test_dgemv(orc, f77, trans, m, n, incx, incy):
    a, s = padded(orc, m, n, 600 + m + n)
    lenx, leny = (n, m) if trans == "N" else (m, n)
    x, s = orc.uniform(lenx * abs(incx), s)
    y, _ = orc.uniform(leny * abs(incy), s + 1)
    for alpha, beta in [(1.0, 0.0), (0.5, -2.0)]:
        want = y.copy()
        orc.dgemv(trans, m, n, alpha, a, x, incx, beta, want, incy)
        got = y.copy()
        f77.dgemv(trans, m, n, alpha, a, a.shape[0], x, incx, beta, got, incy)
        assert rel(got, want) <= TOL


def test_xerbla_codes_match_oracle(orc, f77, capfd):
    a = np.zeros((4, 4), order="F")
    cases = [("Q", "N", 2, 2, 2, 2, 2, 2), ("N", "Q", 2, 2, 2, 2, 2, 2), ("N", "N", -1, 2, 2, 2, 2, 2),
             ("N", "N", 2, -1, 2, 2, 2, 2), ("N", "N", 2, 2, -1, 2, 2, 2), ("N", "N", 3, 2, 2, 2, 2, 3),
             ("N", "N", 2, 2, 3, 2, 2, 2), ("N", "N", 3, 2, 2, 3, 2, 2)]
    for ta, tb, m, n, k, lda, ldb, ldc in cases:
        info = orc.check_dgemm(ta, tb, m, n, k, lda, ldb, ldc)
        assert info > 0
        f77.dgemm(ta, tb, m, n, k, 1.0, a, lda, a, ldb, 0.0, a, ldc)
        err = capfd.readouterr().err
        assert f"DGEMM parameter number {info:2d}" in err, (err, info)
