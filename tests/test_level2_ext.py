"""DGER, DSYMV and DTRSV: the oracle restatements pinned against the CPU BLAS
the reference forwards to (Fortran symbols of SciPy's OpenBLAS), the
library's argument checks against the oracle's, and xerbla_ reporting
without a GPU.  The GPU parity tests are in test_level2_ext_gpu.py."""
import ctypes as C
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _i(v):
    return C.byref(C.c_int(int(v)))


def _d(v):
    return C.byref(C.c_double(float(v)))


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _c(s):
    return C.c_char_p(s.encode())


def vec(rng, n, inc):
    return rng.uniform(-1, 1, 1 + (n - 1) * abs(inc) if n > 0 else 1)


def tri_matrix(rng, n, ld):
    a = np.asfortranarray(rng.uniform(-1, 1, (ld, n)) / max(n, 1))
    for i in range(n):
        a[i, i] = rng.uniform(1, 2)
    return a


@pytest.mark.parametrize("inc", [(1, 1), (2, -3), (-1, 2)])
def test_dger_oracle_matches_cpu_blas(orc, cpublas, inc):
    rng = np.random.default_rng(1)
    m, n = 37, 23
    x, y = vec(rng, m, inc[0]), vec(rng, n, inc[1])
    y[1 * abs(inc[1])] = 0.0   # netlib skips zero y_j
    a = np.asfortranarray(rng.uniform(-1, 1, (m + 3, n)))
    ref, got = a.copy(order="F"), a.copy(order="F")
    orc.dger(m, n, 0.75, x, inc[0], y, inc[1], ref)
    cpublas._f("dger_")(_i(m), _i(n), _d(0.75), _p(x), _i(inc[0]), _p(y), _i(inc[1]), _p(got), _i(m + 3))
    assert np.allclose(got, ref, rtol=1e-14, atol=1e-15)


@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("ab", [(1.5, 0.5), (0.0, 2.0), (1.0, 0.0)])
def test_dsymv_oracle_matches_cpu_blas(orc, cpublas, uplo, ab):
    rng = np.random.default_rng(2)
    n = 45
    a = np.asfortranarray(rng.uniform(-1, 1, (n + 2, n)))
    x, y = vec(rng, n, -2), vec(rng, n, 3)
    ref, got = y.copy(), y.copy()
    orc.dsymv(uplo, n, ab[0], a, x, -2, ab[1], ref, 3)
    cpublas._f("dsymv_")(_c(uplo), _i(n), _d(ab[0]), _p(a), _i(n + 2), _p(x), _i(-2), _d(ab[1]), _p(got), _i(3))
    assert np.allclose(got, ref, rtol=1e-13, atol=1e-14)


@pytest.mark.parametrize("uplo", "UL")
@pytest.mark.parametrize("trans", "NTC")
@pytest.mark.parametrize("diag", "NU")
def test_dtrsv_oracle_matches_cpu_blas(orc, cpublas, uplo, trans, diag):
    rng = np.random.default_rng(3)
    n = 57
    a = tri_matrix(rng, n, n + 1)
    x = vec(rng, n, 2)
    ref, got = x.copy(), x.copy()
    orc.dtrsv(uplo, trans, diag, n, a, ref, 2)
    cpublas._f("dtrsv_")(_c(uplo), _c(trans), _c(diag), _i(n), _p(a), _i(n + 1), _p(got), _i(2))
    assert np.allclose(got, ref, rtol=1e-12, atol=1e-13)


@pytest.mark.parametrize("seed", range(3))
def test_argument_checks_match_oracle(lib, orc, seed):
    rng = np.random.default_rng(200 + seed)
    lib.gbx_check_ger_args.argtypes = [C.c_int] * 5
    lib.gbx_check_symv_args.argtypes = [C.c_char] + [C.c_int] * 4
    lib.gbx_check_trsv_args.argtypes = [C.c_char] * 3 + [C.c_int] * 3
    chars = b"NTCnXLUlRru"
    for _ in range(400):
        c = [bytes([chars[i]]) for i in rng.integers(0, len(chars), 3)]
        v = [int(x) for x in rng.integers(-2, 6, 5)]
        assert lib.gbx_check_ger_args(*v) == orc.lib.orc_check_dger(*v)
        assert lib.gbx_check_symv_args(c[0], *v[:4]) == orc.lib.orc_check_dsymv(c[0], *v[:4])
        assert lib.gbx_check_trsv_args(c[0], c[1], c[2], *v[:3]) == \
            orc.lib.orc_check_dtrsv(c[0], c[1], c[2], *v[:3])


def test_invalid_arguments_call_xerbla_without_device(lib):
    code = """
        import numpy as np, libgpublas_gb300 as g
        f = g.F77(); a = np.zeros((8, 8), order='F'); v = np.zeros(16)
        f.dger(3, 2, 1.0, v, 1, v, 0, a, 3)               # incy -> 7
        f.dsymv('L', 3, 1.0, a, 2, v, 1, 0.0, v, 1)       # lda -> 5
        f.dtrsv('L', 'N', 'X', 2, a, 2, v, 1)             # diag -> 3
        f.dger(0, 2, 1.0, v, 1, v, 1, a, 1)               # quick return
        f.dtrsv('L', 'N', 'N', 0, a, 1, v, 1)             # quick return
        print('calls', g.stats()['calls'])
    """
    e = dict(os.environ, PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, "-c", textwrap.dedent(code)], capture_output=True, text=True, env=e,
                       cwd=ROOT, timeout=120)
    assert r.returncode == 0, r.stderr
    for name, pos in [("DGER", 7), ("DSYMV", 5), ("DTRSV", 3)]:
        assert f"On entry to {name} parameter number {pos:2d}" in r.stderr, r.stderr
    assert "calls 0" in r.stdout
