"""Level-1 parity on the GPU through the Fortran ABI and the device C ABI.

Tolerances (FP64): daxpy elementwise |err| <= 2 ulp of max(|y|, |a*x|);
ddot |err| <= 2*n*u*sum|x*y| against the double-double dot; dnrm2 relative
error <= 1e-14 against the double-double two-pass norm.  idamax/idamin are
bit-exact against the oracle (netlib rules, first index wins ties) and, for
NaN-free input, against the CPU BLAS.
"""
import numpy as np
import pytest

U = 2.0 ** -53

pytestmark = pytest.mark.gpu


def _vec(orc, n, seed):
    x, _ = orc.uniform(max(n, 1), seed)
    return x[:n].copy() if n else np.zeros(1)


def test_idamax_config1_duplicate_maximum(orc, cpublas, f77):
    # n = 2^20 uniform[-1,1] from seed 0; |x| = 1.5 injected at two indices
    # of opposite signs: the first must win (1-based i1 + 1).
    n = 1 << 20
    x, _ = orc.uniform(n, 0)
    i1, i2 = 123457, 987654
    x[i1], x[i2] = 1.5, -1.5
    want = i1 + 1
    assert orc.idamax(n, x, 1) == want
    assert f77.idamax(n, x, 1) == want
    # The CPU BLAS must at least find a maximal element.  (Multi-threaded
    # OpenBLAS on aarch64 returns the LAST of the two tied maxima here, which
    # breaks the BLAS first-index rule; on x86-64 it returns the first.)
    assert abs(x[cpublas.idamax(n, x, 1) - 1]) == 1.5


@pytest.mark.parametrize("n", [1, 2, 3, 31, 32, 33, 1000, 4097, 1 << 16, 1000003])
@pytest.mark.parametrize("incx", [1, 2, 3])
def test_idamax_idamin_random(orc, cpublas, f77, n, incx):
    x, _ = orc.uniform(n * incx, 1000 + n + incx)
    # coarse values create many exact ties
    xq = np.round(x * 64) / 64
    for v in (x, xq):
        assert f77.idamax(n, v, incx) == orc.idamax(n, v, incx)
        assert f77.idamin(n, v, incx) == orc.idamin(n, v, incx)
        # the CPU BLAS agrees on the extreme value; on tie-free data also on
        # the index (see test_idamax_config1_duplicate_maximum for ties)
        seen = np.abs(v[: n * incx: incx])
        assert seen[cpublas.idamax(n, v, incx) - 1] == seen.max()
        assert seen[cpublas.idamin(n, v, incx) - 1] == seen.min()
    assert cpublas.idamax(n, x, incx) == orc.idamax(n, x, incx)


def test_iamax_edge_cases(orc, f77):
    x = np.array([3.0, -3.0, 1.0, 3.0])
    assert f77.idamax(4, x, 1) == 1
    assert f77.idamax(0, x, 1) == 0
    assert f77.idamax(4, x, 0) == 0
    assert f77.idamax(4, x, -1) == 0
    assert f77.idamin(0, x, 1) == 0
    assert f77.idamin(2, x, -2) == 0
    z = np.zeros(1000)
    assert f77.idamax(1000, z, 1) == 1
    assert f77.idamin(1000, z, 1) == 1
    # -0.0 and +0.0 have the same magnitude
    x = np.array([0.5, -0.0, 0.0, -0.5])
    assert f77.idamin(4, x, 1) == 2
    assert f77.idamax(4, x, 1) == 1


def test_iamax_nan_follows_netlib(orc, f77):
    # netlib: a NaN never compares greater/smaller, except x(1) = NaN -> 1.
    cases = [[np.nan, 1, 2, 3], [1, np.nan, 5, 2], [1, 2, np.nan, 0.5] + [0.1] * 40,
             [1, 2, np.inf, np.nan, 3], [np.nan] * 5, [1, 5, np.nan] + [2] * 100 + [5, 7]]
    for c in cases:
        x = np.array(c, dtype=np.float64)
        n = len(x)
        assert f77.idamax(n, x, 1) == orc.idamax(n, x, 1), c
        assert f77.idamin(n, x, 1) == orc.idamin(n, x, 1), c
    big = np.full(1 << 18, 0.25)
    big[5000] = np.nan
    big[200000] = -0.75
    assert f77.idamax(big.size, big, 1) == 200001
    assert f77.idamin(big.size, big, 1) == 1


@pytest.mark.parametrize("n", [0, 1, 2, 7, 1024, 100003, 1 << 20])
@pytest.mark.parametrize("incx,incy", [(1, 1), (2, 1), (1, -1), (-2, 3), (0, 1)])
def test_daxpy(orc, f77, n, incx, incy):
    x, s = orc.uniform(max(1, n * max(1, abs(incx))), 7 + n)
    y, _ = orc.uniform(max(1, n * abs(incy)), s)
    if incx == 0:
        x = x[:1].copy()
    want = y.copy()
    orc.daxpy(n, 0.75, x, incx, want, incy)
    got = y.copy()
    f77.daxpy(n, 0.75, x, incx, got, incy)
    tol = 4 * U * np.maximum(np.abs(want), 1.0)
    assert np.all(np.abs(got - want) <= tol)


def test_daxpy_misaligned_and_alpha0(orc, f77):
    n = 100001
    buf_x, s = orc.uniform(n + 1, 11)
    buf_y, _ = orc.uniform(n + 2, s)
    for ox, oy in [(1, 0), (0, 1), (1, 1), (1, 2)]:
        x = buf_x[ox:ox + n]
        y = buf_y.copy()
        want = y.copy()
        orc.daxpy(n, -1.25, x.copy(), 1, want[oy:oy + n], 1)
        yv = y[oy:oy + n]
        f77.daxpy(n, -1.25, x, 1, yv, 1)
        assert np.all(np.abs(y - want) <= 4 * U * np.maximum(np.abs(want), 1.0))
    y0 = buf_y.copy()
    f77.daxpy(n, 0.0, buf_x, 1, y0, 1)
    assert np.array_equal(y0, buf_y)


@pytest.mark.parametrize("n", [0, 1, 3, 1000, 65537, 1 << 20])
@pytest.mark.parametrize("incx,incy", [(1, 1), (3, 2), (-1, 1), (1, -2)])
def test_ddot(orc, cpublas, f77, n, incx, incy):
    x, s = orc.uniform(max(1, n * abs(incx)), 21 + n)
    y, _ = orc.uniform(max(1, n * abs(incy)), s)
    ref = orc.ddot_dd(n, x, incx, y, incy)
    got = f77.ddot(n, x, incx, y, incy)
    bound = 2 * max(n, 1) * U * (np.abs(x[: n * abs(incx): abs(incx)]) @ np.abs(y[: n * abs(incy): abs(incy)]) if n else 0.0)
    assert abs(got - ref) <= bound + 1e-300
    assert abs(cpublas.ddot(n, x, incx, y, incy) - ref) <= bound + 1e-300


def test_ddot_deterministic(orc, f77):
    n = (1 << 22) + 5
    x, s = orc.uniform(n, 5)
    y, _ = orc.uniform(n, s)
    vals = {f77.ddot(n, x, 1, y, 1) for _ in range(5)}
    assert len(vals) == 1


@pytest.mark.parametrize("n", [1, 2, 17, 1000, 1 << 20])
@pytest.mark.parametrize("incx", [1, 2])
@pytest.mark.parametrize("scale", [1.0, 1e300, 1e-300, 1e-160])
def test_dnrm2(orc, cpublas, f77, n, incx, scale):
    x, _ = orc.uniform(n * incx, 31 + n)
    x = x * scale
    ref = orc.dnrm2(n, x, incx)
    got = f77.dnrm2(n, x, incx)
    assert np.isfinite(got)
    assert abs(got - ref) <= 1e-14 * ref
    assert abs(cpublas.dnrm2(n, x, incx) - ref) <= 1e-13 * ref


def test_dnrm2_edges(f77):
    x = np.array([3.0, 4.0, np.nan])
    assert f77.dnrm2(0, x, 1) == 0.0
    assert f77.dnrm2(2, x, 0) == 0.0
    assert f77.dnrm2(2, x, -1) == 0.0
    assert f77.dnrm2(2, x, 1) == 5.0
    assert np.isnan(f77.dnrm2(3, x, 1))
    mixed = np.array([1e200, 1e-200, 3.0, 1e200])
    assert abs(f77.dnrm2(4, mixed, 1) - np.sqrt(2) * 1e200) <= 1e-14 * np.sqrt(2) * 1e200


@pytest.mark.parametrize("edge", [486, -511])
def test_dnrm2_range_thresholds(orc, f77, edge):
    # elements on both sides of the scaling thresholds 2^486 and 2^-511, with
    # zeros and subnormals, spread over many warps
    rng = np.random.default_rng(edge & 0xffff)
    t = np.ldexp(1.0, edge)
    pool = np.array([t, np.nextafter(t, 0), np.nextafter(t, np.inf), t * (1 + 2.0 ** -20),
                     t * (1 + 2.0 ** -21), t * 0.75, 0.0, -t, 5e-324, 2.2e-308, 1.0])
    for n in (37, 4096, 100003):
        x = rng.choice(pool, n) * rng.uniform(0.5, 1.0, n) ** (rng.integers(0, 2, n))
        ref = orc.dnrm2(n, x, 1)
        got = f77.dnrm2(n, x, 1)
        assert abs(got - ref) <= 1e-14 * ref, (n, got, ref)


def test_device_abi_level1(orc, dev):
    import torch
    n = 3 * (1 << 20) + 1
    xh, s = orc.uniform(n, 77)
    yh, _ = orc.uniform(n, s)
    x = torch.from_numpy(xh).cuda()
    y = torch.from_numpy(yh).cuda()
    res = torch.zeros(1, dtype=torch.float64, device="cuda")
    ires = torch.zeros(1, dtype=torch.int32, device="cuda")
    dev.ddot(n, x, 1, y, 1, res)
    dev.idamax(n, x, 1, ires)
    dev.sync()
    assert abs(res.item() - orc.ddot_dd(n, xh, 1, yh, 1)) <= 2 * n * U * float(np.abs(xh) @ np.abs(yh))
    assert ires.item() == orc.idamax(n, xh, 1)
    dev.daxpy(n, 2.0, x, 1, y, 1)
    dev.sync()
    want = yh.copy()
    orc.daxpy(n, 2.0, xh, 1, want, 1)
    assert np.max(np.abs(y.cpu().numpy() - want)) <= 8 * U
