"""Parity at the shapes that select the large tiles, i.e. the kernels the
benchmarks time.

The GEMM core picks its FP64 block tile (64 x 64, 32 x 32 or 16 x 16) by
how well the last wave of tiles fills the SMs, and the 64 x 64 complex tile
once every SM gets two tiles; the Ozaki product takes its 128 x 256 tile
once 152 such tiles exist (about 2560 x 2560) with K > 1024.  The cases
here are sized to select the tiles the benchmarks time: 64 x 64 for DGEMM
(2040 x 1210 and 1287 x 1287, as at 8192), 32 x 32 for DSYRK (n = 3201, as
at 8192 / 2048), 16 x 16 for large ragged products (2311 x 2305, as in the
DTRSM updates), with ragged edges (sizes that are not multiples of the
tile), odd leading dimensions whose padding rows hold a sentinel, and
beta != 0.

Checks, each with the tolerance stated:
  * sampled entries (random plus the last rows and columns, where the edge
    tiles are) against the double-double oracle: relative error <= 1e-13 for
    the FP64 routines, <= 1e-14 for the Ozaki products (their default target);
  * every entry against an FP64 host product (numpy): relative Frobenius
    difference <= 1e-13, so a wrong tile anywhere is caught;
  * padding rows and the untouched triangle are bit-identical afterwards.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13
TOL_OZ = 1e-14
SENT = 12345.678


def rel(x, ref):
    d = np.linalg.norm(ref)
    return float(np.linalg.norm(x - ref) / (d if d > 0 else 1.0))


def padded(orc, rows, cols, seed, pad=3):
    a, s = orc.matrix(rows, cols, seed, ld=rows + pad)
    a[rows:, :] = SENT
    return a, s


def to_dev(a):
    # the library's context stream does not order with torch's stream: the
    # copy is complete before the call is issued
    import torch
    t = torch.from_numpy(np.asfortranarray(a).ravel(order="F").copy()).cuda()
    torch.cuda.synchronize()
    return t


def from_dev(t, rows, cols):
    return t.cpu().numpy().reshape(rows, cols, order="F")


def samples(m, n, count, seed, lower=None):
    """Random (row, col) pairs plus the last rows and columns (edge tiles);
    lower=True/False keeps only the lower/upper triangle."""
    rng = np.random.default_rng(seed)
    r = np.concatenate([rng.integers(0, m, count), np.full(64, m - 1), rng.integers(0, m, 64),
                        m - 1 - np.arange(64) % m])
    c = np.concatenate([rng.integers(0, n, count), rng.integers(0, n, 64), np.full(64, n - 1),
                        n - 1 - np.arange(64) % n])
    if lower is not None:
        keep = (r >= c) if lower else (r <= c)
        r, c = r[keep], c[keep]
    return r.astype(np.int32), c.astype(np.int32)


def op(x, t):
    return x if t == "N" else x.T


# ------------------------------------------------------------ FP64 DGEMM, 64 x 64 and 16 x 16 tiles
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
@pytest.mark.parametrize("m,n,k", [(2040, 1210, 129), (1287, 1287, 512), (2311, 2305, 129)])
def test_dgemm_large_tile(orc, dev, ta, tb, m, n, k):
    # 2040 x 1210: 32 x 19 = 608 tiles of 64 (four per SM); 1287^2: 21 x 21
    # tiles of 64; 2311 x 2305: 145 x 145 tiles of 16
    if (m, n, k) == (1287, 1287, 512) and tb == "T":
        pytest.skip("the square case runs NN and TN (the benchmarked forms)")
    ra, ca = (m, k) if ta == "N" else (k, m)
    rb, cb = (k, n) if tb == "N" else (n, k)
    a, s = padded(orc, ra, ca, 7000 + m + k)
    b, s = padded(orc, rb, cb, s)
    c, s = padded(orc, m, n, s)
    A, B = to_dev(a), to_dev(b)
    rows, cols = samples(m, n, 2048, m + n + k)
    for alpha, beta in [(1.5, 0.5), (1.0, 0.0)]:
        cin = c.copy(order="F")
        if beta == 0.0:
            cin[:m] = np.nan          # beta = 0 must overwrite, not scale
        C = to_dev(cin)
        dev.dgemm_checked(ta, tb, m, n, k, alpha, A, a.shape[0], B, b.shape[0], beta, C, c.shape[0])
        dev.sync()
        got = from_dev(C, c.shape[0], n)
        assert np.all(got[m:] == SENT)
        ref = orc.dgemm_dd_sample(ta, tb, k, alpha, a, b, beta, c, rows, cols)
        assert rel(got[rows, cols], ref) <= TOL
        full = alpha * (op(a[:ra], ta) @ op(b[:rb], tb)) + (beta * c[:m] if beta else 0.0)
        assert rel(got[:m], full) <= TOL


def test_dgemm_large_tile_through_fortran_symbol(orc, f77):
    # the drop-in path: host operands with an odd leading dimension, staged
    m, n, k = 2400, 2333, 300
    a, s = padded(orc, m, k, 71)
    b, s = padded(orc, k, n, s)
    c, s = padded(orc, m, n, s)
    got = c.copy(order="F")
    f77.dgemm("N", "N", m, n, k, -0.5, a, a.shape[0], b, b.shape[0], 0.25, got, got.shape[0])
    assert np.all(got[m:] == SENT)
    rows, cols = samples(m, n, 2048, 72)
    ref = orc.dgemm_dd_sample("N", "N", k, -0.5, a, b, 0.25, c, rows, cols)
    assert rel(got[rows, cols], ref) <= TOL
    assert rel(got[:m], -0.5 * (a[:m] @ b[:k]) + 0.25 * c[:m]) <= TOL


# ------------------------------------------------------------ FP64 DSYRK, 32 x 32 tile
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "T"])
def test_dsyrk_large_tile(orc, dev, uplo, trans):
    # 101 x 102 / 2 = 5151 triangular tiles of 32 (34 per SM)
    n, k = 3201, 300
    ra, ca = (n, k) if trans == "N" else (k, n)
    a, s = padded(orc, ra, ca, 7100 + ord(uplo) + ord(trans))
    c, _ = padded(orc, n, n, s)
    C = to_dev(c)
    dev.dsyrk(uplo, trans, n, k, -0.75, to_dev(a), a.shape[0], 0.5, C, c.shape[0])
    dev.sync()
    got = from_dev(C, c.shape[0], n)
    assert np.all(got[n:] == SENT)
    lower = uplo == "L"
    rows, cols = samples(n, n, 2048, 7101, lower=lower)
    ta, tb = ("N", "T") if trans == "N" else ("T", "N")
    ref = orc.dgemm_dd_sample(ta, tb, k, -0.75, a, a, 0.5, c, rows, cols)
    assert rel(got[rows, cols], ref) <= TOL
    x = a[:ra]
    full = -0.75 * (x @ x.T if trans == "N" else x.T @ x) + 0.5 * c[:n]
    tri = np.tril if lower else np.triu
    assert rel(tri(got[:n]), tri(full)) <= TOL
    untouched = np.triu(np.ones((n, n), bool), 1) if lower else np.tril(np.ones((n, n), bool), -1)
    assert np.array_equal(got[:n][untouched], c[:n][untouched])


# ------------------------------------------------------------ FP64 DTRMM, 16 x 16 tile
@pytest.mark.parametrize("side,uplo,ta", [("L", "L", "N"), ("R", "U", "T")])
def test_dtrmm_large_tile(orc, dev, side, uplo, ta):
    m, n = 2311, 2305
    na = m if side == "L" else n
    a, s = orc.trsm_matrix(na, 7200 + ord(side))
    b, _ = padded(orc, m, n, s)
    B = to_dev(b)
    dev.dtrmm(side, uplo, ta, "N", m, n, 0.5, to_dev(a), na, B, b.shape[0])
    dev.sync()
    got = from_dev(B, b.shape[0], n)
    assert np.all(got[m:] == SENT)
    t = np.tril(a) if uplo == "L" else np.triu(a)
    t = t if ta == "N" else t.T
    full = 0.5 * (t @ b[:m] if side == "L" else b[:m] @ t)
    assert rel(got[:m], full) <= TOL


# ------------------------------------------------------------ FP64 ZGEMM, 64 x 64 complex tile
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("C", "N"), ("N", "T")])
def test_zgemm_64_tile(orc, dev, ta, tb):
    # 19 x 19 = 361 complex tiles of 64
    m, n, k = 1201, 1153, 200
    rng = np.random.default_rng(7300 + ord(ta))
    ra, ca = (m, k) if ta == "N" else (k, m)
    rb, cb = (k, n) if tb == "N" else (n, k)
    a = np.asfortranarray(rng.uniform(-1, 1, (ra, ca)) + 1j * rng.uniform(-1, 1, (ra, ca)))
    b = np.asfortranarray(rng.uniform(-1, 1, (rb, cb)) + 1j * rng.uniform(-1, 1, (rb, cb)))
    c = np.asfortranarray(rng.uniform(-1, 1, (m, n)) + 1j * rng.uniform(-1, 1, (m, n)))
    alpha, beta = 0.5 - 1.25j, 0.25 + 0.5j
    A = to_dev(a.ravel(order="F").view(np.float64))
    B = to_dev(b.ravel(order="F").view(np.float64))
    C = to_dev(c.ravel(order="F").view(np.float64))
    dev.zgemm(ta, tb, m, n, k, alpha, A, ra, B, rb, beta, C, m)
    dev.sync()
    got = C.cpu().numpy().view(np.complex128).reshape(m, n, order="F")
    rows, cols = samples(m, n, 1024, 7301)
    ref = orc.zgemm_dd_sample(ta, tb, k, alpha, a, b, beta, c, rows, cols)
    assert rel(got[rows, cols], ref) <= TOL

    def zop(x, t):
        return x if t == "N" else (x.T if t == "T" else x.conj().T)
    assert rel(got, alpha * (zop(a, ta) @ zop(b, tb)) + beta * c) <= TOL


# ------------------------------------------------------------ Ozaki, 128 x 256 tile (K > 1024)
@pytest.mark.parametrize("spread", [0, 8, 24])
def test_dgemm_ozaki_wide_256_tile(orc, dev, spread):
    # 20 x 10 = 200 tiles of 128 x 256 (>= one per SM), K = 2048
    m = n = 2560
    k = 2048
    a, s = orc.spread((m, k), spread, 7400 + spread)
    b, s = orc.spread((k, n), spread, s)
    c, _ = orc.matrix(m, n, s)
    C = to_dev(c)
    used = dev.dgemm_ozaki("N", "N", m, n, k, 1.0, to_dev(a), m, to_dev(b), k, 0.5, C, m)
    assert 1 <= used <= 14
    got = from_dev(C, m, n)
    rows, cols = samples(m, n, 2048, 7401 + spread)
    ref = orc.dgemm_dd_sample("N", "N", k, 1.0, a, b, 0.5, c, rows, cols)
    assert rel(got[rows, cols], ref) <= TOL_OZ, (spread, used)


@pytest.mark.parametrize("ta,tb", [("T", "N"), ("N", "T")])
def test_dgemm_ozaki_wide_256_tile_ragged(orc, dev, ta, tb):
    # ragged edges in every dimension: 21 x 11 = 231 tiles, K = 2100
    m, n, k = 2600, 2590, 2100
    ra, ca = (m, k) if ta == "N" else (k, m)
    rb, cb = (k, n) if tb == "N" else (n, k)
    a, s = padded(orc, ra, ca, 7500)
    b, s = padded(orc, rb, cb, s)
    c, _ = padded(orc, m, n, s)
    C = to_dev(c)
    dev.dgemm_ozaki(ta, tb, m, n, k, -1.25, to_dev(a), a.shape[0], to_dev(b), b.shape[0], 0.75, C,
                    c.shape[0])
    got = from_dev(C, c.shape[0], n)
    assert np.all(got[m:] == SENT)
    rows, cols = samples(m, n, 2048, 7501)
    ref = orc.dgemm_dd_sample(ta, tb, k, -1.25, a, b, 0.75, c, rows, cols)
    assert rel(got[rows, cols], ref) <= TOL_OZ
    full = -1.25 * (op(a[:ra], ta) @ op(b[:rb], tb)) + 0.75 * c[:m]
    assert rel(got[:m], full) <= TOL


# ------------------------------------------------------------ Ozaki, half tiles in the last wave
@pytest.mark.parametrize("m,n,k", [(4000, 2500, 1500), (2048, 1536, 1100)])
def test_dgemm_ozaki_half_tile_tail(orc, dev, m, n, k):
    # A last wave that would fill at most half the SMs runs as half-width
    # tiles: 4000 x 2500 is 32 x 10 = 320 tiles of 128 x 256, the 16 left
    # after two waves of 152 run as 32 tiles of 128 x 128 (ragged in M and
    # N); 2048 x 1536 takes 128-wide tiles (16 x 12 = 192), the 40 left run
    # as 80 tiles of 128 x 64.  Every entry against an FP64 host product,
    # sampled entries (edges included) against the double-double oracle.
    a, s = orc.matrix(m, k, 7450 + n)
    b, s = orc.matrix(k, n, s)
    c, _ = orc.matrix(m, n, s)
    C = to_dev(c)
    dev.dgemm_ozaki("N", "N", m, n, k, 0.75, to_dev(a), m, to_dev(b), k, -0.5, C, m)
    dev.sync()
    got = from_dev(C, m, n)
    assert rel(got, 0.75 * (a @ b) - 0.5 * c) <= TOL
    rows, cols = samples(m, n, 2048, 7451 + n)
    ref = orc.dgemm_dd_sample("N", "N", k, 0.75, a, b, -0.5, c, rows, cols)
    assert rel(got[rows, cols], ref) <= TOL_OZ


# ------------------------------------------------------------ Ozaki, B tiles multicast in cluster pairs
@pytest.mark.parametrize("m,n,k,ta,tb", [(4050, 2600, 2100, "T", "N"), (4096, 4096, 2048, "N", "T")])
def test_dgemm_ozaki_multicast_pairs(orc, dev, m, n, k, ta, tb):
    # Products with an even number of 128-row tiles and at least two tiles
    # per SM run in clusters of two CTAs on vertically adjacent tiles, each
    # loading half of the shared B tile for both: 4050 x 2600 is 16 x 11
    # tile pairs (ragged in every dimension, the 24 pairs of the last wave
    # as half tiles), 4096 x 4096 is 16 x 16 pairs (28 left as half tiles).
    ra, ca = (m, k) if ta == "N" else (k, m)
    rb, cb = (k, n) if tb == "N" else (n, k)
    a, s = padded(orc, ra, ca, 7460 + m)
    b, s = padded(orc, rb, cb, s)
    c, _ = padded(orc, m, n, s)
    C = to_dev(c)
    dev.dgemm_ozaki(ta, tb, m, n, k, -0.75, to_dev(a), a.shape[0], to_dev(b), b.shape[0], 1.5, C, c.shape[0])
    dev.sync()
    got = from_dev(C, c.shape[0], n)
    assert np.all(got[m:] == SENT)
    full = -0.75 * (op(a[:ra], ta) @ op(b[:rb], tb)) + 1.5 * c[:m]
    assert rel(got[:m], full) <= TOL
    rows, cols = samples(m, n, 2048, 7461 + m)
    ref = orc.dgemm_dd_sample(ta, tb, k, -0.75, a, b, 1.5, c, rows, cols)
    assert rel(got[rows, cols], ref) <= TOL_OZ


def test_zgemm_ozaki_multicast_pairs(orc, dev):
    # complex K = 600 is a real product of K = 1200 on the wide tile, in
    # cluster pairs (4000 x 2500: 16 x 10 tile pairs)
    m, n, k = 4000, 2500, 600
    ar, s = orc.matrix(m, k, 7620)
    ai, s = orc.matrix(m, k, s)
    br, s = orc.matrix(k, n, s)
    bi, s = orc.matrix(k, n, s)
    cr, s = orc.matrix(m, n, s)
    a = np.asfortranarray(ar + 1j * ai)
    b = np.asfortranarray(br + 1j * bi)
    c = np.asfortranarray(cr + 0.5j * cr)
    alpha, beta = 0.75 + 0.5j, -0.5 + 0.25j
    A = to_dev(a.ravel(order="F").view(np.float64))
    B = to_dev(b.ravel(order="F").view(np.float64))
    C = to_dev(c.ravel(order="F").view(np.float64))
    dev.zgemm_ozaki("N", "N", m, n, k, alpha, A, m, B, k, beta, C, m)
    dev.sync()
    got = C.cpu().numpy().view(np.complex128).reshape(m, n, order="F")
    assert rel(got, alpha * (a @ b) + beta * c) <= TOL
    rows, cols = samples(m, n, 1024, 7621)
    ref = orc.zgemm_dd_sample("N", "N", k, alpha, a, b, beta, c, rows, cols)
    assert rel(got[rows, cols], ref) <= TOL_OZ


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_dsyrk_ozaki_half_tile_tail(orc, dev, uplo):
    # 18 x 9 = 162 tiles of 128 x 256 over the whole square; the 10 left
    # after one wave run as half tiles, those outside the triangle skipped
    n, k = 2304, 1536
    a, s = orc.matrix(n, k, 7720 + ord(uplo))
    c, _ = orc.matrix(n, n, s)
    C = to_dev(c)
    dev.dsyrk_ozaki(uplo, "N", n, k, -1.0, to_dev(a), n, 1.0, C, n)
    dev.sync()
    got = from_dev(C, n, n)
    lower = uplo == "L"
    keep = np.tril(np.ones((n, n), bool)) if lower else np.triu(np.ones((n, n), bool))
    full = -(a @ a.T) + c
    assert rel(got[keep], full[keep]) <= TOL
    assert np.array_equal(got[~keep], c[~keep])
    rows, cols = samples(n, n, 2048, 7721, lower=lower)
    ref = orc.dgemm_dd_sample("N", "T", k, -1.0, a, a, 1.0, c, rows, cols)
    assert rel(got[rows, cols], ref) <= TOL_OZ


@pytest.mark.parametrize("spread", [0, 8])
def test_zgemm_ozaki_wide_256_tile(orc, dev, spread):
    # complex K = 1024 is a real product of K = 2048 on the wide tile
    m = n = 2560
    k = 1024
    ar, s = orc.spread((m, k), spread, 7600 + spread)
    ai, s = orc.spread((m, k), spread, s)
    br, s = orc.spread((k, n), spread, s)
    bi, s = orc.spread((k, n), spread, s)
    a = np.asfortranarray(ar + 1j * ai)
    b = np.asfortranarray(br + 1j * bi)
    c = np.zeros((m, n), dtype=np.complex128, order="F")
    alpha = 0.75 + 0.5j
    A = to_dev(a.ravel(order="F").view(np.float64))
    B = to_dev(b.ravel(order="F").view(np.float64))
    C = to_dev(c.ravel(order="F").view(np.float64))
    dev.zgemm_ozaki("N", "N", m, n, k, alpha, A, m, B, k, 0.0, C, m)
    got = C.cpu().numpy().view(np.complex128).reshape(m, n, order="F")
    rows, cols = samples(m, n, 1024, 7601)
    ref = orc.zgemm_dd_sample("N", "N", k, alpha, a, b, 0.0, c, rows, cols)
    assert rel(got[rows, cols], ref) <= TOL_OZ


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_dsyrk_ozaki_wide(orc, dev, uplo):
    n, k = 2600, 2048
    a, s = orc.matrix(n, k, 7700 + ord(uplo))
    c, _ = orc.matrix(n, n, s)
    C = to_dev(c)
    dev.dsyrk_ozaki(uplo, "N", n, k, -1.0, to_dev(a), n, 1.0, C, n)
    got = from_dev(C, n, n)
    lower = uplo == "L"
    rows, cols = samples(n, n, 2048, 7701, lower=lower)
    ref = orc.dgemm_dd_sample("N", "T", k, -1.0, a, a, 1.0, c, rows, cols)
    assert rel(got[rows, cols], ref) <= TOL_OZ
    untouched = np.triu(np.ones((n, n), bool), 1) if lower else np.tril(np.ones((n, n), bool), -1)
    assert np.array_equal(got[untouched], c[untouched])


# ------------------------------------------------------------ DTRSM with 32 / 16-tile updates
def test_dtrsm_large_left_lower(orc, dev):
    # config-2 distribution (diagonal uniform[1,2], off-diagonal
    # uniform[-1,1]/m); the recursive updates run on 32 x 32 and 16 x 16
    # tiles.
    # Backward residual of 16 sampled right-hand sides against the
    # double-double oracle, forward error of the same columns against the
    # oracle's substitution.
    m, n = 4096, 512
    a, s = orc.trsm_matrix(m, 7800)
    b, _ = orc.matrix(m, n, s)
    B = to_dev(b)
    dev.dtrsm("L", "L", "N", "N", m, n, 1.0, to_dev(a), m, B, m)
    dev.sync()
    got = from_dev(B, m, n)
    cols = np.sort(np.random.default_rng(7801).choice(n, 16, replace=False))
    cols[-1] = n - 1
    xs = np.asfortranarray(got[:, cols])
    bs = np.asfortranarray(b[:, cols])
    assert orc.dtrsm_residual("L", "L", "N", "N", m, len(cols), 1.0, a, bs, xs) <= 1e-14
    want = bs.copy(order="F")
    orc.dtrsm("L", "L", "N", "N", m, len(cols), 1.0, a, want)
    assert rel(xs, want) <= TOL


# ------------------------------------------------------------ dgemm_ on host operands, pipelined copies
@pytest.mark.parametrize("ta,tb,beta", [("N", "N", 0.5), ("T", "N", 0.0), ("N", "T", -1.0)])
def test_fortran_dgemm_pipelined_copies_match_device_path(orc, f77, dev, ta, tb, beta):
    # large enough for the Fortran symbol to cut C into blocks whose copies
    # overlap the block products (2 x 3 blocks here); the result must be
    # bit-identical to the same product on device operands (same kernel,
    # same K order), padding rows untouched
    import libgpublas_gb300 as g
    m, n, k = 8300, 6200, 300
    ra, ca = (m, k) if ta == "N" else (k, m)
    rb, cb = (k, n) if tb == "N" else (n, k)
    a, s = padded(orc, ra, ca, 7900)
    b, s = padded(orc, rb, cb, s)
    c, _ = padded(orc, m, n, s)
    cin = c.copy(order="F")
    if beta == 0.0:
        cin[:m] = np.nan
    C = to_dev(cin)
    dev.dgemm_checked(ta, tb, m, n, k, 1.25, to_dev(a), a.shape[0], to_dev(b), b.shape[0], beta, C, c.shape[0])
    dev.sync()
    want = from_dev(C, c.shape[0], n)
    s0 = g.stats()
    got = cin.copy(order="F")
    f77.dgemm(ta, tb, m, n, k, 1.25, a, a.shape[0], b, b.shape[0], beta, got, got.shape[0])
    s1 = g.stats()
    moved = (ra * ca + rb * cb + (m * n if beta != 0.0 else 0)) * 8
    assert s1["bytes_h2d"] - s0["bytes_h2d"] == moved
    assert s1["bytes_d2h"] - s0["bytes_d2h"] == m * n * 8
    assert np.all(got[m:] == SENT)
    assert np.array_equal(got, want)
    rows, cols = samples(m, n, 1024, 7901)
    ref = orc.dgemm_dd_sample(ta, tb, k, 1.25, a, b, beta, c, rows, cols)
    assert rel(got[rows, cols], ref) <= TOL


@pytest.mark.skipif(__import__("os").environ.get("GBX_OZAKI_PAIR") == "0",
                    reason="already running with the one-CTA kernel")
def test_one_cta_ozaki_kernel_variant():
    # Products of at most four waves of 256 x 256 tiles take the CTA-pair
    # kernel by default, so the Ozaki cases above run on it; rerun them in a
    # child process with GBX_OZAKI_PAIR=0, on the one-CTA kernel that the
    # larger products (the 8192 benchmark) use, with and without B multicast.
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, GBX_OZAKI_PAIR="0", PYTHONPATH=root)
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider", "-m", "gpu",
                        os.path.abspath(__file__), "-k", "ozaki and not variant"],
                       capture_output=True, text=True, env=env, cwd=root, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
