"""The C-ABI library without a GPU: it builds for sm_103a, loads, exports every
symbol the public headers declare, and its host-side logic (argument checks,
xerbla, quick returns, option parsing, failure reporting) behaves as
specified.  No call here reaches a kernel.
"""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_exports_every_declared_symbol(lib):
    import libgpublas_gb300 as g
    names = g.declared_symbols()
    assert "dgemm_" in names and "gbx_dgemm" in names and "cblas_idamax" in names
    out = subprocess.run(["nm", "-D", "--defined-only", g.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in names if n not in exported]
    assert not missing, missing


def test_diag_library_exports_its_symbols(lib):
    # benchmark and failure-path diagnostics live in libgbxdiag.so, not in
    # the BLAS library an application loads
    import libgpublas_gb300 as g
    names = g.declared_symbols(g.DIAG_HEADERS)
    assert "gbx_diag_fp64_peak" in names and "gbx_diag_expire_wait" in names
    nm = lambda p: {ln.split()[-1] for ln in subprocess.run(  # noqa: E731
        ["nm", "-D", "--defined-only", p], capture_output=True, text=True, check=True).stdout.splitlines()
        if ln.strip()}
    diag, blas = nm(g.DIAG_LIB_PATH), nm(g.LIB_PATH)
    assert not [n for n in names if n not in diag]
    assert not [n for n in blas if n.startswith("gbx_diag")]
    g.load_diag()


def test_library_is_sm103a_only(lib):
    import libgpublas_gb300 as g
    out = subprocess.run(["cuobjdump", "--list-elf", g.LIB_PATH], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    arches = {ln.split(".")[-2] for ln in out.stdout.splitlines() if ".sm_" in ln}
    assert arches == {"sm_103a"}, arches


@pytest.mark.parametrize("seed", range(4))
def test_argument_checks_match_oracle(lib, orc, seed):
    import ctypes as C
    rng = np.random.default_rng(seed)
    L = lib
    L.gbx_check_gemm_args.argtypes = [C.c_char, C.c_char] + [C.c_int] * 6
    L.gbx_check_trxm_args.argtypes = [C.c_char] * 4 + [C.c_int] * 4
    L.gbx_check_syrk_args.argtypes = [C.c_char] * 2 + [C.c_int] * 4
    L.gbx_check_gemv_args.argtypes = [C.c_char] + [C.c_int] * 5
    chars = b"NTCnXLUlRru"
    for _ in range(400):
        c = [bytes([chars[i]]) for i in rng.integers(0, len(chars), 4)]
        v = [int(x) for x in rng.integers(-2, 6, 6)]
        assert L.gbx_check_gemm_args(c[0], c[1], *v) == orc.check_dgemm(c[0], c[1], *v)
        assert L.gbx_check_trxm_args(c[0], c[1], c[2], c[3], *v[:4]) == \
            orc.check_dtrsm(c[0], c[1], c[2], c[3], *v[:4])
        assert L.gbx_check_syrk_args(c[0], c[1], *v[:4]) == orc.check_dsyrk(c[0], c[1], *v[:4])
        assert L.gbx_check_gemv_args(c[0], *v[:5]) == orc.check_dgemv(c[0], *v[:5])


def _run_py(code, env=None):
    e = dict(os.environ)
    e.update(env or {})
    e["PYTHONPATH"] = ROOT
    return subprocess.run([sys.executable, "-c", textwrap.dedent(code)], capture_output=True,
                          text=True, env=e, cwd=ROOT, timeout=120)


def test_invalid_arguments_call_xerbla_without_device(lib):
    # invalid calls and quick returns never touch CUDA, so they run here
    r = _run_py("""
        import numpy as np, libgpublas_gb300 as g
        f = g.F77(); a = np.zeros((4, 4), order='F')
        f.dgemm('N', 'N', 3, 2, 2, 1.0, a, 2, a, 2, 0.0, a, 3)      # lda < m -> 8
        f.dtrsm('L', 'Q', 'N', 'N', 2, 2, 1.0, a, 2, a, 2)          # uplo -> 2
        f.dsyrk('L', 'N', 3, 2, 1.0, a, 2, 0.0, a, 3)                # lda -> 7
        f.dgemv('N', 2, 2, 1.0, a, 2, a, 0, 0.0, a, 1)               # incx -> 8
        f.dgemm('N', 'N', 0, 2, 2, 1.0, a, 1, a, 2, 0.0, a, 1)       # quick return
        print('idamax', f.idamax(0, a, 1), f.idamax(3, a, 0), f.idamax(1, a, 1))
        print('ddot', f.ddot(0, a, 1, a, 1), 'nrm2', f.dnrm2(0, a, 1))
        print('calls', g.stats()['calls'])
    """)
    assert r.returncode == 0, r.stderr
    err = r.stderr
    assert "On entry to DGEMM parameter number  8" in err
    assert "On entry to DTRSM parameter number  2" in err
    assert "On entry to DSYRK parameter number  7" in err
    assert "On entry to DGEMV parameter number  8" in err
    assert "idamax 0 0 1" in r.stdout
    assert "ddot 0.0 nrm2 0.0" in r.stdout
    assert "calls 0" in r.stdout


def test_device_failure_is_reported_not_silent(lib):
    # With no usable device the call must fail loudly; errors=return makes it
    # print and return instead of aborting (the reference always aborts).
    r = _run_py("""
        import numpy as np, libgpublas_gb300 as g, torch
        if torch.cuda.is_available():
            print('HAS_GPU'); raise SystemExit(0)
        f = g.F77(); a = np.ones((8, 8), order='F'); c = np.full((8, 8), 7.0, order='F')
        f.dgemm('N', 'N', 8, 8, 8, 1.0, a, 8, a, 8, 0.0, c, 8)
        print('after', float(c[0, 0]))
    """, env={"BLAS2CUDA_OPTIONS": "errors=return"})
    if "HAS_GPU" in r.stdout:
        pytest.skip("a GPU is present")
    assert r.returncode == 0, r.stderr
    assert "gbxblas: DGEMM failed" in r.stderr
    assert "after 7.0" in r.stdout
    r2 = _run_py("""
        import numpy as np, libgpublas_gb300 as g
        f = g.F77(); a = np.ones((8, 8), order='F')
        f.dgemm('N', 'N', 8, 8, 8, 1.0, a, 8, a, 8, 0.0, a, 8)
    """, env={"BLAS2CUDA_OPTIONS": ""})
    assert r2.returncode != 0 and "gbxblas: DGEMM failed" in r2.stderr


def test_options_parsing(lib):
    r = _run_py("""
        import ctypes as C, libgpublas_gb300 as g
        L = g.load()
        class Cfg(C.Structure):
            _fields_ = [('ozaki', C.c_int), ('tol', C.c_double), ('prefetch', C.c_int),
                        ('abort', C.c_int), ('trace', C.c_int), ('heuristic', C.c_int)]
        L.gbx_get_config.restype = C.POINTER(Cfg)
        c = L.gbx_get_config().contents
        print(c.ozaki, c.tol, c.prefetch, c.abort, c.heuristic)
    """, env={"BLAS2CUDA_OPTIONS": "help;precision=ozaki:1e-12;prefetch=off;errors=return;"
                                   "heuristic=true;bogus"})
    assert r.returncode == 0, r.stderr
    assert r.stdout.split() == ["1", "1e-12", "0", "0", "1"]
    assert "gbxblas options" in r.stderr and "unknown option 'bogus'" in r.stderr


@pytest.mark.parametrize("m,n,tri,tile", [
    (8192, 8192, 0, 64),    # the DGEMM headline: 16384 tiles of 64, 107.8 per SM
    (2040, 1210, 0, 64),    # 608 tiles of 64: exactly four per SM
    (1287, 1287, 0, 64),
    (4096, 1024, 0, 32),    # a DTRSM update: 1024 tiles of 64 would leave 0.74 of a wave
    (2048, 1024, 0, 16),    # 512 tiles of 64: four tile times for 3.37 tiles of work
    (1024, 1024, 0, 16),
    (2311, 2305, 0, 16),
    (64, 64, 0, 16),        # a small product: the most SMs
    (8192, 8192, 1, 32),    # DSYRK 8192: 32896 triangular tiles of 32
    (3201, 3201, 1, 32),
])
def test_fp64_tile_choice(lib, m, n, tri, tile):
    # The FP64 GEMM core's block tile for a 152-SM part: the best product
    # of the kernel's efficiency (64: 1.0, 32: 0.998, 16: 0.985, measured)
    # and the fill of the last wave of tiles.
    import ctypes as C
    f = lib.gbx_dgemm_tile_choice
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int]
    assert f(m, n, tri, 152) == tile
