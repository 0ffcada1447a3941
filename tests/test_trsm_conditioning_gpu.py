"""DTRSM on ill-conditioned triangles, plain FP64 and Ozaki.

The plain DTRSM applies inverted 64 x 64 diagonal blocks (FP64) and updates
the rest with the FP64 GEMM core; the Ozaki DTRSM forms op(A)^-1 in FP64 and
applies it as one Ozaki product.  Solves through an inverse are not backward
stable in general, so both are checked on triangles with condition numbers
of about 1e8 to 1e10, where that would show:

  * "unscaled": diagonal uniform[1,2], off-diagonal uniform[-1,1] (not
    divided by n); cond ~ 8e8 at order 256;
  * "graded": rows scaled by 10^(-8 i/n) of a config-2 triangle (diagonal
    uniform[1,2], off-diagonal uniform[-1,1]/n); cond ~ 1e8.

Measures, against the double-double oracle:
  * normwise backward error ||op(A) X - alpha B|| / (||A|| ||X|| + |alpha| ||B||)
    <= 1e-14 for both paths;
  * componentwise backward error max |op(A) X - alpha B| / (|op(A)| |X| +
    |alpha| |B|): for the plain path <= 1e-14, or 10x what the oracle's
    substitution reaches on the same triangle if that is larger (2e-16 on
    "unscaled", up to 4e-15 on "graded" at order 1000); for the Ozaki path the product's
    error is relative to |op(A)^-1| |B|, which cancellation can make much
    larger than |X|, so its bound is 1e-12 (tol 1e-14 times the observed
    amplification, below 100 on these triangles).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [(s, u, t) for s, u, t in [("L", "L", "N"), ("L", "U", "T"), ("R", "L", "T"), ("R", "U", "N")]]


def to_dev(a):
    # the library's context stream does not order with torch's stream: the
    # copy is complete before the call is issued
    import torch
    t = torch.from_numpy(np.asfortranarray(a).ravel(order="F").copy()).cuda()
    torch.cuda.synchronize()
    return t


def from_dev(t, rows, cols):
    return t.cpu().numpy().reshape(rows, cols, order="F")


def triangle(kind, n, seed, uplo):
    rng = np.random.default_rng(seed)
    if kind == "unscaled":
        low = np.tril(rng.uniform(-1, 1, (n, n)), -1) + np.diag(rng.uniform(1, 2, n))
    else:
        low = np.tril(rng.uniform(-1, 1, (n, n)) / n, -1) + np.diag(rng.uniform(1, 2, n))
        low = np.diag(10.0 ** (-8.0 * np.arange(n) / n)) @ low
    a = low if uplo == "L" else low.T
    # the unused triangle holds values that must be ignored
    junk = rng.uniform(-1e3, 1e3, (n, n))
    a = np.where(np.tril(np.ones((n, n), bool)) if uplo == "L" else np.triu(np.ones((n, n), bool)), a, junk)
    return np.asfortranarray(a)


def solve_and_measure(orc, dev, run, kind, na, side, uplo, ta, nrhs=48):
    a = triangle(kind, na, 8000 + na + ord(side) + ord(uplo), uplo)
    m, n = (na, nrhs) if side == "L" else (nrhs, na)
    b = np.asfortranarray(np.random.default_rng(8100 + na).uniform(-1, 1, (m, n)))
    alpha = 1.5
    B = to_dev(b)
    run(side, uplo, ta, m, n, alpha, to_dev(a), na, B, m)
    dev.sync()
    x = np.asfortranarray(from_dev(B, m, n))
    assert np.all(np.isfinite(x))
    nw = orc.dtrsm_residual(side, uplo, ta, "N", m, n, alpha, a, b, x)
    cw = orc.dtrsm_residual_cw(side, uplo, ta, "N", m, n, alpha, a, b, x)
    ref = b.copy(order="F")
    orc.dtrsm(side, uplo, ta, "N", m, n, alpha, a, ref)
    cw_subst = orc.dtrsm_residual_cw(side, uplo, ta, "N", m, n, alpha, a, b, ref)
    return nw, cw, cw_subst, np.linalg.cond(np.tril(a) if uplo == "L" else np.triu(a))


@pytest.mark.parametrize("kind,na", [("unscaled", 256), ("graded", 256), ("graded", 1000)])
@pytest.mark.parametrize("side,uplo,ta", CASES)
def test_plain_dtrsm_ill_conditioned(orc, dev, kind, na, side, uplo, ta):
    def run(side, uplo, ta, m, n, alpha, A, lda, B, ldb):
        dev.dtrsm(side, uplo, ta, "N", m, n, alpha, A, lda, B, ldb)
    nw, cw, cw_subst, cond = solve_and_measure(orc, dev, run, kind, na, side, uplo, ta)
    print(f"plain {kind} n={na} {side}{uplo}{ta}: cond {cond:.1e} normwise {nw:.2e} "
          f"componentwise {cw:.2e} (substitution {cw_subst:.2e})")
    assert cond > 1e7
    assert nw <= 1e-14
    assert cw <= max(1e-14, 10 * cw_subst)


@pytest.mark.parametrize("kind,na", [("unscaled", 256), ("graded", 256)])
@pytest.mark.parametrize("side,uplo,ta", CASES)
def test_ozaki_dtrsm_ill_conditioned(orc, dev, kind, na, side, uplo, ta):
    def run(side, uplo, ta, m, n, alpha, A, lda, B, ldb):
        dev.dtrsm_ozaki(side, uplo, ta, "N", m, n, alpha, A, lda, B, ldb)
    nw, cw, cw_subst, cond = solve_and_measure(orc, dev, run, kind, na, side, uplo, ta)
    print(f"ozaki {kind} n={na} {side}{uplo}{ta}: cond {cond:.1e} normwise {nw:.2e} "
          f"componentwise {cw:.2e} (substitution {cw_subst:.2e})")
    assert nw <= 1e-14
    assert cw <= 1e-12
