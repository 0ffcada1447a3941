"""CPU tests of the Level-3 set beyond D/Z GEMM, DSYRK, DTRSM, DTRMM.

* The complex-double oracle restatements (orc_zsymm, orc_zsyrk, orc_zsyr2k,
  orc_ztrmm, orc_ztrsm, used for every precision) are pinned against the CPU
  BLAS the reference forwards to (SciPy's OpenBLAS, through its Fortran
  symbols) on the same seeded operands.
* The library's netlib argument checks for the new routines match the
  oracle's, and invalid calls report through xerbla_ without a GPU.
"""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from tests import l3cases as L3

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = L3.cases()


@pytest.mark.parametrize("case", CASES, ids=[L3.case_id(c) for c in CASES])
def test_oracle_matches_cpu_blas(orc, cpublas, case):
    d = L3.inputs(case, seed=7)
    ref = L3.run_oracle(orc, case, {k: v.copy(order="F") for k, v in d.items()})
    got = L3.run_cpu(cpublas, case, {k: v.copy(order="F") for k, v in d.items()})
    tol = L3.TOL[case["p"]]
    assert L3.rel_err(got, ref) <= tol, (L3.case_id(case), L3.rel_err(got, ref))


def test_hermitian_results_have_real_diagonal(orc):
    c = dict(r="herk", p="z", uplo="L", trans="N", n=9, k=5, ab=(1.0, 1.0))
    d = L3.inputs(c, seed=3)
    out = L3.run_oracle(orc, c, d)
    assert np.all(np.diag(out[:9, :9]).imag == 0.0)


@pytest.mark.parametrize("seed", range(3))
def test_argument_checks_match_oracle(lib, orc, seed):
    import ctypes as C
    rng = np.random.default_rng(100 + seed)
    lib.gbx_check_symm_args.argtypes = [C.c_char, C.c_char] + [C.c_int] * 5
    lib.gbx_check_rank_k_args.argtypes = [C.c_char, C.c_char] + [C.c_int] * 5
    lib.gbx_check_rank_2k_args.argtypes = [C.c_char, C.c_char] + [C.c_int] * 6
    chars = b"NTCnXLUlRru"
    for _ in range(400):
        c = [bytes([chars[i]]) for i in rng.integers(0, len(chars), 2)]
        v = [int(x) for x in rng.integers(-2, 6, 6)]
        mask = int(rng.choice([7, 3, 5]))
        assert lib.gbx_check_symm_args(c[0], c[1], *v[:5]) == orc.check_symm(c[0], c[1], *v[:5])
        assert lib.gbx_check_rank_k_args(c[0], c[1], mask, *v[:4]) == \
            orc.check_rank_k(c[0], c[1], mask, *v[:4])
        assert lib.gbx_check_rank_2k_args(c[0], c[1], mask, *v[:5]) == \
            orc.check_rank_2k(c[0], c[1], mask, *v[:5])


def test_invalid_arguments_call_xerbla_without_device(lib):
    code = """
        import numpy as np, libgpublas_gb300 as g
        f = g.F77()
        a = np.zeros((8, 8), dtype=np.complex128, order='F')
        s = np.zeros((8, 8), dtype=np.float32, order='F')
        f.symm('s', 'X', 'L', 2, 2, 1.0, s, 2, s, 2, 0.0, s, 2)          # side -> 1
        f.symm('z', 'L', 'L', 3, 2, 1.0, a, 2, a, 3, 0.0, a, 3, True)    # lda -> 7
        f.syrk('c', 'L', 'C', 2, 2, 1.0, a, 2, 0.0, a, 2)                # CSYRK takes N, T -> 2
        f.syrk('z', 'L', 'T', 2, 2, 1.0, a, 2, 0.0, a, 2, True)          # ZHERK takes N, C -> 2
        f.syr2k('d', 'U', 'N', 3, 2, 1.0, s.astype(np.float64), 3, s.astype(np.float64), 2, 0.0,
                s.astype(np.float64), 3)                                 # ldb -> 9
        f.syr2k('z', 'U', 'N', 2, 2, 1.0, a, 2, a, 2, 0.0, a, 1, True)   # ldc -> 12
        f.trxm('c', 'trsm', 'L', 'L', 'N', 'N', 3, 2, 1.0, a, 2, a, 3)   # lda -> 9
        f.trxm('s', 'trmm', 'L', 'L', 'N', 'Q', 2, 2, 1.0, s, 2, s, 2)   # diag -> 4
        f.gemm('c', 'N', 'Q', 2, 2, 2, 1.0, a, 2, a, 2, 0.0, a, 2)       # transb -> 2
        f.symm('d', 'L', 'U', 0, 3, 1.0, s.astype(np.float64), 1, s.astype(np.float64), 1, 0.0,
               s.astype(np.float64), 1)                                  # quick return
        f.syrk('z', 'L', 'N', 3, 0, 1.0, a, 3, 1.0, a, 3, True)          # quick return (k = 0, beta = 1)
        print('calls', g.stats()['calls'])
    """
    e = dict(os.environ, PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, "-c", textwrap.dedent(code)], capture_output=True, text=True, env=e,
                       cwd=ROOT, timeout=120)
    assert r.returncode == 0, r.stderr
    err = r.stderr
    for name, pos in [("SSYMM", 1), ("ZHEMM", 7), ("CSYRK", 2), ("ZHERK", 2), ("DSYR2K", 9), ("ZHER2K", 12),
                      ("CTRSM", 9), ("STRMM", 4), ("CGEMM", 2)]:
        assert f"On entry to {name} parameter number {pos:2d}" in err, (name, err)
    assert "calls 0" in r.stdout
