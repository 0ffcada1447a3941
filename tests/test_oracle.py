"""Pin the oracle (CPU, no GPU): against the golden vectors produced by the
CPU BLAS that the reference's runnable path ends in, and against that CPU BLAS
run live on fresh inputs.

Tolerance: relative Frobenius error <= 1e-14 for floating-point outputs
(different but correctly rounded summation orders), bit-exact for indices.
"""
import os

import numpy as np
import pytest

from tests.golden import make_golden as mg

GOLD = os.path.join(os.path.dirname(__file__), "golden", "blas_golden.npz")
RTOL = 1e-14


def rel(x, ref):
    d = np.linalg.norm(ref)
    return np.linalg.norm(np.asarray(x) - ref) / (d if d > 0 else 1.0)


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def test_splitmix64_known_values(orc):
    # SplitMix64 from state 0: published first outputs of the generator
    import ctypes
    s = ctypes.c_uint64(0)
    got = [orc.lib.orc_splitmix64_next(ctypes.byref(s)) for _ in range(3)]
    assert got == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]
    x, _ = orc.uniform(5, 0)
    assert np.all((x >= -1) & (x < 1))
    assert x[0] == 2.0 * ((0xE220A8397B1DCDAF >> 11) * 2.0 ** -53) - 1.0


CASES = mg.cases()


@pytest.mark.parametrize("name,d", CASES, ids=[c[0] for c in CASES])
def test_oracle_matches_golden(orc, gold, name, d):
    assert float(gold[f"{name}/input_checksum"]) == pytest.approx(mg.input_checksum(d), rel=1e-15)
    kind = d["kind"]
    if kind == "dgemm":
        c = d["c"].copy(order="F")
        orc.dgemm(d["ta"], d["tb"], d["m"], d["n"], d["k"], d["alpha"], d["a"], d["b"], d["beta"], c)
        assert rel(c, gold[f"{name}/out"]) <= RTOL
    elif kind == "dgemm_cfg1":
        a, s = orc.matrix(512, 512, 0)
        b, s = orc.matrix(512, 512, s)
        c, s = orc.matrix(512, 512, s)
        orc.dgemm("N", "N", 512, 512, 512, 1.0, a, b, 0.5, c)
        assert rel(c.sum(axis=0), gold[f"{name}/colsum"]) <= 1e-13
        r, q = gold[f"{name}/rows"], gold[f"{name}/cols"]
        assert rel(c[r, q], gold[f"{name}/sample"]) <= RTOL
        assert abs(np.linalg.norm(c) - float(gold[f"{name}/fro"])) <= 1e-13 * np.linalg.norm(c)
    elif kind == "zgemm":
        c = d["c"].copy(order="F")
        orc.zgemm(d["ta"], d["tb"], d["m"], d["n"], d["k"], d["alpha"], d["a"], d["b"], d["beta"], c)
        assert rel(c, gold[f"{name}/out"]) <= RTOL
    elif kind == "dsyrk":
        c = d["c"].copy(order="F")
        orc.dsyrk(d["uplo"], d["trans"], d["n"], d["k"], d["alpha"], d["a"], d["beta"], c)
        assert rel(c, gold[f"{name}/out"]) <= RTOL
    elif kind in ("dtrsm", "dtrmm"):
        b = d["b"].copy(order="F")
        getattr(orc, kind)(d["side"], d["uplo"], d["ta"], d["diag"], d["m"], d["n"], d["alpha"],
                           d["a"], b)
        assert rel(b, gold[f"{name}/out"]) <= RTOL
    elif kind == "dgemv":
        y = d["y"].copy()
        orc.dgemv(d["trans"], d["m"], d["n"], d["alpha"], d["a"], d["x"], d["incx"], d["beta"], y,
                  d["incy"])
        assert rel(y, gold[f"{name}/out"]) <= RTOL
    elif kind == "daxpy":
        y = d["y"].copy()
        orc.daxpy(d["n"], d["alpha"], d["x"], d["incx"], y, d["incy"])
        assert rel(y, gold[f"{name}/out"]) <= RTOL
    elif kind == "ddot":
        v = orc.ddot(d["n"], d["x"], d["incx"], d["y"], d["incy"])
        assert abs(v - float(gold[f"{name}/out"])) <= 1e-13
    elif kind == "dnrm2":
        v = orc.dnrm2(d["n"], d["x"], d["incx"])
        g = float(gold[f"{name}/out"])
        assert abs(v - g) <= RTOL * g
    elif kind == "iamax":
        # fixtures come from x86-64 OpenBLAS, which keeps the first index on
        # ties (its multi-threaded aarch64 build does not; see test_l1_gpu)
        assert orc.idamax(d["n"], d["x"], d["incx"]) == int(gold[f"{name}/amax"])
        assert orc.idamin(d["n"], d["x"], d["incx"]) == int(gold[f"{name}/amin"])
    else:
        raise AssertionError(kind)


def test_config1_idamax_is_first_of_duplicate(gold):
    assert int(gold["idamax_cfg1/amax"]) == 123457 + 1


@pytest.mark.parametrize("seed", [11, 12, 13])
def test_oracle_vs_cpublas_live(orc, cpublas, seed):
    rng = np.random.default_rng(seed)
    m, n, k = (int(v) for v in rng.integers(1, 60, 3))
    for ta in "NT":
        for tb in "NT":
            a, s = orc.matrix(m if ta == "N" else k, k if ta == "N" else m, seed)
            b, s = orc.matrix(k if tb == "N" else n, n if tb == "N" else k, s)
            c, s = orc.matrix(m, n, s)
            c1, c2 = c.copy(order="F"), c.copy(order="F")
            orc.dgemm(ta, tb, m, n, k, 0.7, a, b, -1.3, c1)
            cpublas.dgemm(ta, tb, m, n, k, 0.7, a, b, -1.3, c2)
            assert rel(c1, c2) <= 1e-14
    a, s = orc.trsm_matrix(m, seed)
    b, s = orc.matrix(m, n, s)
    for side, uplo, t, dg in [("L", "L", "N", "N"), ("R", "U", "T", "U"), ("L", "U", "T", "N")]:
        na = m if side == "L" else n
        aa, _ = orc.trsm_matrix(na, seed + 1)
        b1, b2 = b.copy(order="F"), b.copy(order="F")
        orc.dtrsm(side, uplo, t, dg, m, n, 2.0, aa, b1)
        cpublas.dtrsm(side, uplo, t, dg, m, n, 2.0, aa, b2)
        assert rel(b1, b2) <= 1e-14


def test_dd_checker_is_more_accurate_than_plain(orc):
    # cancellation-heavy dot: the dd result equals the exact rational value
    x = np.array([1e16, 1.0, -1e16, 1.0])
    y = np.ones(4)
    assert orc.ddot_dd(4, x, 1, y, 1) == 2.0
    assert orc.ddot(4, x, 1, y, 1) != 2.0


def test_argument_checks_follow_netlib(orc):
    assert orc.check_dgemm("X", "N", 1, 1, 1, 1, 1, 1) == 1
    assert orc.check_dgemm("N", "N", 4, 1, 1, 3, 1, 4) == 8
    assert orc.check_dgemm("N", "T", 4, 5, 2, 4, 4, 4) == 10
    assert orc.check_dgemm("N", "N", 4, 5, 2, 4, 2, 3) == 13
    assert orc.check_dtrsm("L", "L", "N", "N", 5, 3, 4, 5) == 9
    assert orc.check_dtrsm("R", "L", "N", "N", 5, 3, 3, 4) == 11
    assert orc.check_dsyrk("L", "T", 5, 7, 6, 5) == 7
    assert orc.check_dgemv("N", 5, 3, 5, 0, 1) == 8


def test_componentwise_trsm_residual(orc):
    # The oracle's substitution solve has a componentwise backward error near
    # n*u even on a triangle with condition number ~1e9; a solution perturbed
    # by 1e-12 relative (a planted mistake, on the CPU) is flagged.
    rng = np.random.default_rng(4)
    n, nrhs = 200, 8
    t = np.asfortranarray(np.tril(rng.uniform(-1, 1, (n, n)), -1) + np.diag(rng.uniform(1, 2, n)))
    assert np.linalg.cond(np.tril(t)) > 1e6
    b = np.asfortranarray(rng.uniform(-1, 1, (n, nrhs)))
    x = b.copy(order="F")
    orc.dtrsm("L", "L", "N", "N", n, nrhs, 1.0, t, x)
    cw = orc.dtrsm_residual_cw("L", "L", "N", "N", n, nrhs, 1.0, t, b, x)
    assert cw <= 1e-15
    bad = np.asfortranarray(x * (1.0 + 1e-12 * rng.choice([-1.0, 1.0], x.shape)))
    assert orc.dtrsm_residual_cw("L", "L", "N", "N", n, nrhs, 1.0, t, b, bad) > 1e-13
    # side R, upper, transposed: X op(A) = alpha B
    xr = np.asfortranarray(rng.uniform(-1, 1, (nrhs, n)))
    br = xr.copy(order="F")
    orc.dtrsm("R", "U", "T", "N", nrhs, n, 2.0, np.asfortranarray(t.T), br)
    # br now holds the solution of X op(A) = 2 xr
    assert orc.dtrsm_residual_cw("R", "U", "T", "N", nrhs, n, 2.0, np.asfortranarray(t.T), xr, br) <= 1e-15
