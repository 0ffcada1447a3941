"""GPU results through the Fortran ABI against the committed golden vectors
(outputs of the CPU BLAS on the same seeded inputs).

Tolerance: relative Frobenius error <= 1e-13 for floating point; indices
bit-exact.
"""
import os

import numpy as np
import pytest

from tests.golden import make_golden as mg

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "blas_golden.npz")
CASES = mg.cases()


def rel(x, ref):
    d = np.linalg.norm(ref)
    return np.linalg.norm(np.asarray(x) - ref) / (d if d > 0 else 1.0)


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.mark.parametrize("name,d", CASES, ids=[c[0] for c in CASES])
def test_gpu_matches_golden(f77, orc, gold, name, d):
    kind = d["kind"]
    tol = 1e-13
    if kind == "dgemm":
        c = d["c"].copy(order="F")
        f77.dgemm(d["ta"], d["tb"], d["m"], d["n"], d["k"], d["alpha"], d["a"], d["a"].shape[0],
                  d["b"], d["b"].shape[0], d["beta"], c, c.shape[0])
        assert rel(c, gold[f"{name}/out"]) <= tol
    elif kind == "dgemm_cfg1":
        a, s = orc.matrix(512, 512, 0)
        b, s = orc.matrix(512, 512, s)
        c, s = orc.matrix(512, 512, s)
        f77.dgemm("N", "N", 512, 512, 512, 1.0, a, 512, b, 512, 0.5, c, 512)
        r, q = gold[f"{name}/rows"], gold[f"{name}/cols"]
        assert rel(c[r, q], gold[f"{name}/sample"]) <= tol
        assert rel(c.sum(axis=0), gold[f"{name}/colsum"]) <= tol
    elif kind == "zgemm":
        c = d["c"].copy(order="F")
        f77.zgemm(d["ta"], d["tb"], d["m"], d["n"], d["k"], d["alpha"], d["a"], d["a"].shape[0],
                  d["b"], d["b"].shape[0], d["beta"], c, c.shape[0])
        assert rel(c, gold[f"{name}/out"]) <= tol
    elif kind == "dsyrk":
        c = d["c"].copy(order="F")
        f77.dsyrk(d["uplo"], d["trans"], d["n"], d["k"], d["alpha"], d["a"], d["a"].shape[0],
                  d["beta"], c, c.shape[0])
        assert rel(c, gold[f"{name}/out"]) <= tol
    elif kind in ("dtrsm", "dtrmm"):
        b = d["b"].copy(order="F")
        getattr(f77, kind)(d["side"], d["uplo"], d["ta"], d["diag"], d["m"], d["n"], d["alpha"],
                           d["a"], d["a"].shape[0], b, b.shape[0])
        assert rel(b, gold[f"{name}/out"]) <= tol
    elif kind == "dgemv":
        y = d["y"].copy()
        f77.dgemv(d["trans"], d["m"], d["n"], d["alpha"], d["a"], d["a"].shape[0], d["x"],
                  d["incx"], d["beta"], y, d["incy"])
        assert rel(y, gold[f"{name}/out"]) <= tol
    elif kind == "daxpy":
        y = d["y"].copy()
        f77.daxpy(d["n"], d["alpha"], d["x"], d["incx"], y, d["incy"])
        assert rel(y, gold[f"{name}/out"]) <= tol
    elif kind == "ddot":
        v = f77.ddot(d["n"], d["x"], d["incx"], d["y"], d["incy"])
        assert abs(v - float(gold[f"{name}/out"])) <= 1e-13
    elif kind == "dnrm2":
        v = f77.dnrm2(d["n"], d["x"], d["incx"])
        g = float(gold[f"{name}/out"])
        assert abs(v - g) <= 1e-14 * g
    elif kind == "iamax":
        assert f77.idamax(d["n"], d["x"], d["incx"]) == int(gold[f"{name}/amax"])
        assert f77.idamin(d["n"], d["x"], d["incx"]) == int(gold[f"{name}/amin"])
