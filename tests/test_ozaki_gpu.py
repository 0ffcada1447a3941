"""Ozaki split-precision products on the tcgen05 FP8 path.

* Exactness of the tensor-core FP32 accumulation: with one forced slice and
  operands whose single digit represents them exactly, the result must equal
  the exact integer product bit for bit (partial sums up to ~2^23.8).
* Accuracy: relative Frobenius error <= 1e-14 against the double-double
  oracle at the default target (tol = 1e-14), for uniform inputs and inputs
  with exponent spread s in {0, 8, 24} (entries u * 2^e, e uniform in
  [-s, s]); the error decreases with the slice count.
* Semantics: all transposition pairs, edge tiles, alpha/beta, beta = 0
  clearing NaN, DSYRK triangles, ZGEMM conjugation, determinism.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-14


def rel(x, ref):
    d = np.linalg.norm(ref)
    return float(np.linalg.norm(x - ref) / (d if d > 0 else 1.0))


def to_dev(a):
    import torch
    return torch.from_numpy(np.asfortranarray(a).ravel(order="F")).cuda()


def from_dev(t, rows, cols):
    return t.cpu().numpy().reshape(rows, cols, order="F")


@pytest.mark.parametrize("K", [1024, 4096, 65536])
def test_fp8_accumulation_is_exact(dev, K):
    # K = 1024 runs the small-K kernel (all diagonals resident in TMEM), the
    # others the wide-tile kernel
    # Rows/columns hold even integers with |x| <= 30 and a 30 in every row and
    # column: e = 5, one digit d = x/2 (|d| <= 15) represents x exactly, so
    # slices=1 makes the result exactly 4 * sum d_a d_b.
    rng = np.random.default_rng(K)
    M, N = 128, 256
    da = rng.integers(-15, 16, (M, K))
    db = rng.integers(-15, 16, (K, N))
    da[:, 0] = 15
    db[0, :] = 15
    # a block of same-sign maxima drives partial sums toward 225 * K
    da[:8, :] = 15
    db[:, :8] = 15
    a = (2 * da).astype(np.float64)
    b = (2 * db).astype(np.float64)
    exact = 4 * (da.astype(np.int64) @ db.astype(np.int64))
    A, B = to_dev(a), to_dev(b)
    C = to_dev(np.zeros((M, N)))
    used = dev.dgemm_ozaki("N", "N", M, N, K, 1.0, A, M, B, K, 0.0, C, M, 0.0, 1)
    assert used == 1
    got = from_dev(C, M, N)
    assert np.abs(exact).max() < 2 ** 53
    assert np.array_equal(got, exact.astype(np.float64)), np.abs(got - exact).max()


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (130, 70, 200), (257, 300, 129)])
def test_dgemm_ozaki_shapes(orc, dev, ta, tb, m, n, k):
    ra, ca = (m, k) if ta == "N" else (k, m)
    rb, cb = (k, n) if tb == "N" else (n, k)
    a, s = orc.matrix(ra, ca, 900 + m + k)
    b, s = orc.matrix(rb, cb, s)
    c, s = orc.matrix(m, n, s)
    for alpha, beta in [(1.0, 0.0), (-1.5, 0.5)]:
        ref = orc.dgemm_dd(ta, tb, m, n, k, alpha, a, b, beta, c)
        C = to_dev(c)
        used = dev.dgemm_ozaki(ta, tb, m, n, k, alpha, to_dev(a), ra, to_dev(b), rb, beta, C, m)
        assert 1 <= used <= 14
        assert rel(from_dev(C, m, n), ref) <= TOL


@pytest.mark.parametrize("spread", [0, 8, 24])
def test_dgemm_ozaki_spread_accuracy(orc, dev, spread):
    m = n = 384
    k = 1000
    a, s = orc.spread((m, k), spread, 31 + spread)
    b, s = orc.spread((k, n), spread, s)
    c = np.zeros((m, n), order="F")
    ref = orc.dgemm_dd("N", "N", m, n, k, 1.0, a, b, 0.0, c)
    errs = {}
    for S in (4, 7, 10):
        C = to_dev(c)
        dev.dgemm_ozaki("N", "N", m, n, k, 1.0, to_dev(a), m, to_dev(b), k, 0.0, C, m, 0.0, S)
        errs[S] = rel(from_dev(C, m, n), ref)
    assert errs[4] > errs[7] > errs[10] or errs[10] <= 1e-15
    C = to_dev(c)
    used = dev.dgemm_ozaki("N", "N", m, n, k, 1.0, to_dev(a), m, to_dev(b), k, 0.0, C, m, TOL, 0)
    err = rel(from_dev(C, m, n), ref)
    assert err <= TOL, (spread, used, err, errs)


def test_dgemm_ozaki_tolerance_controls_slices(orc, dev):
    m = n = k = 256
    a, s = orc.matrix(m, k, 5)
    b, s = orc.matrix(k, n, s)
    c = np.zeros((m, n), order="F")
    ref = orc.dgemm_dd("N", "N", m, n, k, 1.0, a, b, 0.0, c)
    used = {}
    for tol in (1e-6, 1e-10, 1e-14):
        C = to_dev(c)
        used[tol] = dev.dgemm_ozaki("N", "N", m, n, k, 1.0, to_dev(a), m, to_dev(b), k, 0.0, C, m, tol, 0)
        assert rel(from_dev(C, m, n), ref) <= tol
    assert used[1e-6] < used[1e-10] < used[1e-14]


def test_dgemm_ozaki_beta0_nan_and_determinism(orc, dev):
    m, n, k = 200, 100, 300
    a, s = orc.matrix(m, k, 8)
    b, s = orc.matrix(k, n, s)
    A, B = to_dev(a), to_dev(b)
    outs = []
    for _ in range(3):
        C = to_dev(np.full((m, n), np.nan))
        dev.dgemm_ozaki("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, C, m)
        outs.append(from_dev(C, m, n))
    assert np.all(np.isfinite(outs[0]))
    assert all(np.array_equal(outs[0], o) for o in outs[1:])


@pytest.mark.parametrize("k", [128, 2048])        # small-K kernel, wide-tile kernel
@pytest.mark.parametrize("bad", [np.inf, np.nan])
def test_nonfinite_operand_is_reported_and_context_recovers(orc, dev, k, bad):
    # the preparation flags the operand, the product kernel skips, the sync
    # reports it; the next call on the same context runs normally
    from libgpublas_gb300._lib import GbxError
    m, n = 256, 128
    a, s = orc.matrix(m, k, 3)
    b, s = orc.matrix(k, n, s)
    c, s = orc.matrix(m, n, s)
    a_bad = a.copy()
    a_bad[5, 7] = bad
    with pytest.raises(GbxError, match="non-finite"):
        dev.dgemm_ozaki("N", "N", m, n, k, 1.0, to_dev(a_bad), m, to_dev(b), k, 0.5, to_dev(c), m)
    C = to_dev(c)
    dev.dgemm_ozaki("N", "N", m, n, k, 1.0, to_dev(a), m, to_dev(b), k, 0.5, C, m)
    ref = orc.dgemm_dd("N", "N", m, n, k, 1.0, a, b, 0.5, c)
    assert rel(from_dev(C, m, n), ref) <= TOL


@pytest.mark.parametrize("k", [64, 2048])         # small-K kernel, wide-tile kernel
@pytest.mark.parametrize("alpha,beta", [(1.0, 0.0), (-0.75, 0.0)])
def test_results_near_the_underflow_threshold(orc, dev, k, alpha, beta):
    # operands scaled by 2^-512: the products are near 2^-1020, so the low
    # part of each element's two-part conversion leaves the normal range and
    # the 128-bit route converts it; the reference is the unscaled product
    # scaled by the same power of two
    m, n = 96, 80
    a, s = orc.matrix(m, k, 77 + k)
    b, s = orc.matrix(k, n, s)
    c = np.zeros((m, n), order="F")
    ref = np.ldexp(orc.dgemm_dd("N", "N", m, n, k, alpha, a, b, beta, c), -1024)
    C = to_dev(c)
    dev.dgemm_ozaki("N", "N", m, n, k, alpha, to_dev(np.ldexp(a, -512)), m, to_dev(np.ldexp(b, -512)), k, beta,
                    C, m)
    got = from_dev(C, m, n)
    assert np.all(np.isfinite(got))
    assert rel(got, ref) <= TOL


@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "T"])
def test_dsyrk_ozaki(orc, dev, uplo, trans):
    n, k = 300, 170
    ra, ca = (n, k) if trans == "N" else (k, n)
    a, s = orc.matrix(ra, ca, 77)
    c, _ = orc.matrix(n, n, s)
    want = c.copy(order="F")
    orc.dsyrk(uplo, trans, n, k, 0.75, a, 0.5, want)
    C = to_dev(c)
    dev.dsyrk_ozaki(uplo, trans, n, k, 0.75, to_dev(a), ra, 0.5, C, n)
    got = from_dev(C, n, n)
    tri = np.tril if uplo == "L" else np.triu
    assert rel(tri(got), tri(want)) <= TOL
    other = np.triu(np.ones((n, n)), 1) if uplo == "L" else np.tril(np.ones((n, n)), -1)
    assert np.array_equal(got[other == 1], c[other == 1])


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("C", "N"), ("N", "T"), ("T", "C")])
def test_zgemm_ozaki(orc, dev, ta, tb):
    m, n, k = 150, 90, 130
    rng = np.random.default_rng(3)
    ra, ca = (m, k) if ta == "N" else (k, m)
    rb, cb = (k, n) if tb == "N" else (n, k)
    a = np.asfortranarray(rng.uniform(-1, 1, (ra, ca)) + 1j * rng.uniform(-1, 1, (ra, ca)))
    b = np.asfortranarray(rng.uniform(-1, 1, (rb, cb)) + 1j * rng.uniform(-1, 1, (rb, cb)))
    c = np.asfortranarray(rng.uniform(-1, 1, (m, n)) + 1j * rng.uniform(-1, 1, (m, n)))
    alpha, beta = 0.5 - 1.25j, 0.25 + 0.5j
    rows = rng.integers(0, m, 500)
    cols = rng.integers(0, n, 500)
    ref = orc.zgemm_dd_sample(ta, tb, k, alpha, a, b, beta, c, rows, cols)
    import torch
    C = torch.from_numpy(c.ravel(order="F").view(np.float64).copy()).cuda()
    A = torch.from_numpy(a.ravel(order="F").view(np.float64).copy()).cuda()
    B = torch.from_numpy(b.ravel(order="F").view(np.float64).copy()).cuda()
    dev.zgemm_ozaki(ta, tb, m, n, k, alpha, A, ra, B, rb, beta, C, m)
    got = C.cpu().numpy().view(np.complex128).reshape(m, n, order="F")
    assert rel(got[rows, cols], ref) <= TOL


@pytest.mark.parametrize("side", "LR")
@pytest.mark.parametrize("uplo", "LU")
@pytest.mark.parametrize("ta", "NT")
@pytest.mark.parametrize("diag", "NU")
def test_dtrsm_ozaki(orc, dev, side, uplo, ta, diag):
    # op(A)^-1 formed in FP64, applied as one Ozaki product; well-conditioned
    # triangles (diagonal uniform[1,2], off-diagonal uniform[-1,1]/n)
    m, n = 300, 190
    na = m if side == "L" else n
    a, s = orc.trsm_matrix(na, 40 + na)
    b, _ = orc.matrix(m, n, s)
    want = b.copy(order="F")
    orc.dtrsm(side, uplo, ta, diag, m, n, -0.75, a, want)
    B = to_dev(b)
    used = dev.dtrsm_ozaki(side, uplo, ta, diag, m, n, -0.75, to_dev(a), na, B, m)
    assert 1 <= used <= 14
    assert rel(from_dev(B, m, n), want) <= 1e-13


@pytest.mark.parametrize("m,n,k", [(1500, 128, 128), (700, 256, 256), (4100, 96, 64)])
def test_trailing_update_shapes(orc, dev, m, n, k):
    # the rank-nb updates of a blocked Cholesky: C -= A B^T with operands that
    # are sub-blocks of one larger matrix (leading dimension > rows)
    ld = m + n + 37
    big, s = orc.matrix(ld, k, 321 + m)
    a = np.asfortranarray(big[:m])
    b = np.asfortranarray(big[m:m + n])
    c, _ = orc.matrix(m, n, s)
    ref = orc.dgemm_dd("N", "T", m, n, k, -1.0, a, b, 1.0, c)
    BIG = to_dev(big)
    C = to_dev(c)
    dev.dgemm_ozaki("N", "T", m, n, k, -1.0, BIG, ld, BIG[m:], ld, 1.0, C, m)
    assert rel(from_dev(C, m, n), ref) <= TOL
    # the diagonal block: symmetric rank-k on the first n rows
    cs, _ = orc.matrix(n, n, 5)
    want = cs.copy(order="F")
    orc.dsyrk("L", "N", n, k, -1.0, np.asfortranarray(big[:n]), 1.0, want)
    CS = to_dev(cs)
    dev.dsyrk_ozaki("L", "N", n, k, -1.0, BIG, ld, 1.0, CS, n)
    got = from_dev(CS, n, n)
    assert rel(np.tril(got), np.tril(want)) <= TOL
    assert np.array_equal(np.triu(got, 1), np.triu(cs, 1))


@pytest.mark.skipif(__import__("os").environ.get("GBX_OZAKI_SMALLK") == "0",
                    reason="already running without the small-K kernel")
def test_wide_tile_kernel_for_small_k():
    # the small-K kernel is the default for K <= 1024; rerun the small-K tests
    # with the wide-tile kernel selected
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, GBX_OZAKI_SMALLK="0", PYTHONPATH=root)
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider",
                        os.path.abspath(__file__), "-k", "shapes or spread or syrk or zgemm or tolerance"],
                       capture_output=True, text=True, env=env, cwd=root, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]


@pytest.mark.skipif(__import__("os").environ.get("GBX_OZAKI_PAIR") == "1",
                    reason="already running with the CTA-pair kernel")
def test_cta_pair_kernel_variant():
    # The CTA-pair (tcgen05 cta_group::2) kernel is chosen by size (mid-size
    # products with K > 1024); rerun the kernel tests in a child process with
    # it forced for every product with more than one 128-row tile, small K
    # included.
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, GBX_OZAKI_PAIR="1", PYTHONPATH=root)
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider",
                        os.path.abspath(__file__), "-k", "exact or shapes or spread or syrk or zgemm"],
                       capture_output=True, text=True, env=env, cwd=root, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]


def test_f77_precision_option_routes_to_ozaki(orc):
    # BLAS2CUDA_OPTIONS=precision=ozaki sends dgemm_ through the split path;
    # checked in a child process because options are read once per process.
    import os
    import subprocess
    import sys
    import textwrap
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = textwrap.dedent("""
        import numpy as np, oracle, libgpublas_gb300 as g
        orc = oracle.get(); f = g.F77()
        a, s = orc.matrix(300, 300, 1); b, s = orc.matrix(300, 300, s); c = np.zeros((300, 300), order='F')
        ref = orc.dgemm_dd('N', 'N', 300, 300, 300, 1.0, a, b, 0.0, c)
        f.dgemm('N', 'N', 300, 300, 300, 1.0, a, 300, b, 300, 0.0, c, 300)
        print('ERR', np.linalg.norm(c - ref) / np.linalg.norm(ref))
    """)
    env = dict(os.environ, PYTHONPATH=root, BLAS2CUDA_OPTIONS="precision=ozaki;errors=return")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, cwd=root,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    err = float(r.stdout.split("ERR")[1])
    assert err <= TOL
