"""The oracle: a CPU restatement of the netlib BLAS semantics on the
intercepted path, and a ctypes handle on the CPU BLAS the reference falls
back to.

TEST INFRASTRUCTURE ONLY.  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this package, always as the checker or
as the timed CPU baseline -- never as the thing measured on the GPU or shipped.

* ``Oracle``  -- ctypes wrapper over ``oracle/liboracle.so`` (oracle.c).
* ``cpublas`` -- the CPU BLAS the reference reaches through
  ``dlsym(RTLD_NEXT)`` (runtime-blas.c:60-69, gemm.cc:129-141); here that is
  SciPy's bundled OpenBLAS.

Arrays are numpy float64 (complex128 for Z routines) in Fortran order; the
leading dimension of a 2-D array is its first extent.
"""
import ctypes as C

import numpy as np

from .build import build_oracle

_c_int, _c_dbl, _c_char = C.c_int, C.c_double, C.c_char
_P = C.c_void_p


def _ptr(a):
    if a is None:
        return None
    assert a.flags.f_contiguous or a.ndim == 1, "oracle wants Fortran-ordered arrays"
    return a.ctypes.data_as(_P)


def _ch(c):
    return _c_char(c.encode() if isinstance(c, str) else c)


class Oracle:
    """Thin typed view of liboracle.so."""

    def __init__(self, path=None):
        self.lib = C.CDLL(path or build_oracle())
        L = self.lib
        L.orc_splitmix64_next.restype = C.c_uint64
        for f in ("orc_fill_uniform", "orc_fill_spread"):
            getattr(L, f).restype = C.c_uint64
        L.orc_fill_uniform.argtypes = [C.c_uint64, _P, C.c_size_t]
        L.orc_fill_spread.argtypes = [C.c_uint64, _P, C.c_size_t, _c_int]
        L.orc_fill_matrix.restype = C.c_uint64
        L.orc_fill_matrix.argtypes = [C.c_uint64, _P, _c_int, _c_int, _c_int]
        L.orc_fill_trsm_matrix.restype = C.c_uint64
        L.orc_fill_trsm_matrix.argtypes = [C.c_uint64, _P, _c_int, _c_int]
        L.orc_daxpy.argtypes = [_c_int, _c_dbl, _P, _c_int, _P, _c_int]
        L.orc_ddot.restype = _c_dbl
        L.orc_ddot.argtypes = [_c_int, _P, _c_int, _P, _c_int]
        L.orc_ddot_dd.restype = _c_dbl
        L.orc_ddot_dd.argtypes = [_c_int, _P, _c_int, _P, _c_int]
        L.orc_dnrm2.restype = _c_dbl
        L.orc_dnrm2.argtypes = [_c_int, _P, _c_int]
        L.orc_idamax.argtypes = [_c_int, _P, _c_int]
        L.orc_idamin.argtypes = [_c_int, _P, _c_int]
        L.orc_dgemv.argtypes = [_c_char, _c_int, _c_int, _c_dbl, _P, _c_int, _P, _c_int,
                                _c_dbl, _P, _c_int]
        L.orc_dgemm.argtypes = [_c_char, _c_char, _c_int, _c_int, _c_int, _c_dbl, _P, _c_int,
                                _P, _c_int, _c_dbl, _P, _c_int]
        L.orc_zgemm.argtypes = [_c_char, _c_char, _c_int, _c_int, _c_int, _P, _P, _c_int,
                                _P, _c_int, _P, _P, _c_int]
        L.orc_dsyrk.argtypes = [_c_char, _c_char, _c_int, _c_int, _c_dbl, _P, _c_int,
                                _c_dbl, _P, _c_int]
        for f in ("orc_dtrsm", "orc_dtrmm"):
            getattr(L, f).argtypes = [_c_char, _c_char, _c_char, _c_char, _c_int, _c_int,
                                      _c_dbl, _P, _c_int, _P, _c_int]
        L.orc_check_dgemm.argtypes = [_c_char, _c_char] + [_c_int] * 6
        L.orc_check_dtrsm.argtypes = [_c_char] * 4 + [_c_int] * 4
        L.orc_check_dsyrk.argtypes = [_c_char, _c_char] + [_c_int] * 4
        L.orc_check_dgemv.argtypes = [_c_char] + [_c_int] * 5
        L.orc_dgemm_dd.argtypes = [_c_char, _c_char, _c_int, _c_int, _c_int, _c_dbl, _P, _c_int,
                                   _P, _c_int, _c_dbl, _P, _c_int, _P, _c_int]
        L.orc_dgemm_dd_sample.argtypes = [_c_char, _c_char, _c_int, _c_dbl, _P, _c_int, _P,
                                          _c_int, _c_dbl, _P, _c_int, _c_int, _P, _P, _P]
        L.orc_zgemm_dd_sample.argtypes = [_c_char, _c_char, _c_int, _P, _P, _c_int, _P,
                                          _c_int, _P, _P, _c_int, _c_int, _P, _P, _P]
        L.orc_dtrsm_residual.restype = _c_dbl
        L.orc_dtrsm_residual.argtypes = [_c_char] * 4 + [_c_int, _c_int, _c_dbl, _P, _c_int,
                                                         _P, _c_int, _P, _c_int]
        L.orc_dtrsm_residual_cw.restype = _c_dbl
        L.orc_dtrsm_residual_cw.argtypes = L.orc_dtrsm_residual.argtypes
        L.orc_zsymm.argtypes = [_c_char, _c_char, _c_int, _c_int, _P, _P, _c_int, _P, _c_int, _P, _P,
                                _c_int, _c_int]
        L.orc_zsyrk.argtypes = [_c_char, _c_char, _c_int, _c_int, _c_int, _P, _P, _c_int, _P, _P, _c_int,
                                _c_int]
        L.orc_zsyr2k.argtypes = [_c_char, _c_char, _c_int, _c_int, _c_int, _P, _P, _c_int, _P, _c_int, _P,
                                 _P, _c_int, _c_int]
        for f in ("orc_ztrmm", "orc_ztrsm"):
            getattr(L, f).argtypes = [_c_char, _c_char, _c_char, _c_char, _c_int, _c_int, _P, _P, _c_int,
                                      _P, _c_int]
        L.orc_dger.argtypes = [_c_int, _c_int, _c_dbl, _P, _c_int, _P, _c_int, _P, _c_int]
        L.orc_dsymv.argtypes = [_c_char, _c_int, _c_dbl, _P, _c_int, _P, _c_int, _c_dbl, _P, _c_int]
        L.orc_dtrsv.argtypes = [_c_char, _c_char, _c_char, _c_int, _P, _c_int, _P, _c_int]
        L.orc_check_dger.argtypes = [_c_int] * 5
        L.orc_check_dsymv.argtypes = [_c_char] + [_c_int] * 4
        L.orc_check_dtrsv.argtypes = [_c_char] * 3 + [_c_int] * 3
        L.orc_check_symm.argtypes = [_c_char, _c_char] + [_c_int] * 5
        L.orc_check_rank_k.argtypes = [_c_char, _c_char] + [_c_int] * 5
        L.orc_check_rank_2k.argtypes = [_c_char, _c_char] + [_c_int] * 6
        L.orc_rel_fro.restype = _c_dbl
        L.orc_rel_fro.argtypes = [_c_int, _c_int, _P, _c_int, _P, _c_int]

    # ---- seeded inputs ----------------------------------------------------
    def uniform(self, n, state):
        out = np.empty(n, dtype=np.float64)
        state = self.lib.orc_fill_uniform(state, _ptr(out), n)
        return out, state

    def matrix(self, m, n, state, ld=None):
        ld = ld or max(1, m)
        a = np.empty((ld, n), dtype=np.float64, order="F")
        state = self.lib.orc_fill_matrix(state, _ptr(a), m, n, ld)
        return a, state

    def trsm_matrix(self, n, state, ld=None):
        ld = ld or max(1, n)
        a = np.empty((ld, n), dtype=np.float64, order="F")
        state = self.lib.orc_fill_trsm_matrix(state, _ptr(a), n, ld)
        return a, state

    def spread(self, shape, s, state):
        a = np.empty(shape, dtype=np.float64, order="F")
        state = self.lib.orc_fill_spread(state, _ptr(a), a.size, s)
        return a, state

    # ---- routines (in place on y / c / b, as BLAS does) ------------------
    def daxpy(self, n, alpha, x, incx, y, incy):
        self.lib.orc_daxpy(n, alpha, _ptr(x), incx, _ptr(y), incy)

    def ddot(self, n, x, incx, y, incy):
        return self.lib.orc_ddot(n, _ptr(x), incx, _ptr(y), incy)

    def ddot_dd(self, n, x, incx, y, incy):
        return self.lib.orc_ddot_dd(n, _ptr(x), incx, _ptr(y), incy)

    def dnrm2(self, n, x, incx):
        return self.lib.orc_dnrm2(n, _ptr(x), incx)

    def idamax(self, n, x, incx):
        return self.lib.orc_idamax(n, _ptr(x), incx)

    def idamin(self, n, x, incx):
        return self.lib.orc_idamin(n, _ptr(x), incx)

    def dgemv(self, trans, m, n, alpha, a, x, incx, beta, y, incy):
        self.lib.orc_dgemv(_ch(trans), m, n, alpha, _ptr(a), a.shape[0], _ptr(x), incx,
                           beta, _ptr(y), incy)

    def dgemm(self, ta, tb, m, n, k, alpha, a, b, beta, c):
        self.lib.orc_dgemm(_ch(ta), _ch(tb), m, n, k, alpha, _ptr(a), a.shape[0],
                           _ptr(b), b.shape[0], beta, _ptr(c), c.shape[0])

    def zgemm(self, ta, tb, m, n, k, alpha, a, b, beta, c):
        al = np.array([complex(alpha)], dtype=np.complex128)
        be = np.array([complex(beta)], dtype=np.complex128)
        self.lib.orc_zgemm(_ch(ta), _ch(tb), m, n, k, _ptr(al), _ptr(a), a.shape[0],
                           _ptr(b), b.shape[0], _ptr(be), _ptr(c), c.shape[0])

    def dsyrk(self, uplo, trans, n, k, alpha, a, beta, c):
        self.lib.orc_dsyrk(_ch(uplo), _ch(trans), n, k, alpha, _ptr(a), a.shape[0],
                           beta, _ptr(c), c.shape[0])

    def dtrsm(self, side, uplo, ta, diag, m, n, alpha, a, b):
        self.lib.orc_dtrsm(_ch(side), _ch(uplo), _ch(ta), _ch(diag), m, n, alpha,
                           _ptr(a), a.shape[0], _ptr(b), b.shape[0])

    def dtrmm(self, side, uplo, ta, diag, m, n, alpha, a, b):
        self.lib.orc_dtrmm(_ch(side), _ch(uplo), _ch(ta), _ch(diag), m, n, alpha,
                           _ptr(a), a.shape[0], _ptr(b), b.shape[0])

    # ---- argument checks ---------------------------------------------------
    # ---- DGER / DSYMV / DTRSV (in place, leading dimension = first extent)
    def dger(self, m, n, alpha, x, incx, y, incy, a):
        self.lib.orc_dger(m, n, alpha, _ptr(x), incx, _ptr(y), incy, _ptr(a), a.shape[0])

    def dsymv(self, uplo, n, alpha, a, x, incx, beta, y, incy):
        self.lib.orc_dsymv(_ch(uplo), n, alpha, _ptr(a), a.shape[0], _ptr(x), incx, beta, _ptr(y), incy)

    def dtrsv(self, uplo, trans, diag, n, a, x, incx):
        self.lib.orc_dtrsv(_ch(uplo), _ch(trans), _ch(diag), n, _ptr(a), a.shape[0], _ptr(x), incx)

    # ---- the rest of Level 3, on complex128 arrays (real or single-precision
    # inputs are widened by the caller; ``z`` promotes a copy) -------------
    @staticmethod
    def z(a):
        """Fortran-ordered complex128 copy of any numeric array."""
        return np.asfortranarray(np.asarray(a, dtype=np.complex128))

    def zsymm(self, side, uplo, m, n, alpha, a, b, beta, c, herm=False):
        al = np.array([complex(alpha)]); be = np.array([complex(beta)])
        self.lib.orc_zsymm(_ch(side), _ch(uplo), m, n, _ptr(al), _ptr(a), a.shape[0], _ptr(b), b.shape[0],
                           _ptr(be), _ptr(c), c.shape[0], int(herm))

    def zsyrk(self, uplo, trans, allowed, n, k, alpha, a, beta, c, herm=False):
        al = np.array([complex(alpha)]); be = np.array([complex(beta)])
        self.lib.orc_zsyrk(_ch(uplo), _ch(trans), allowed, n, k, _ptr(al), _ptr(a), a.shape[0], _ptr(be),
                           _ptr(c), c.shape[0], int(herm))

    def zsyr2k(self, uplo, trans, allowed, n, k, alpha, a, b, beta, c, herm=False):
        al = np.array([complex(alpha)]); be = np.array([complex(beta)])
        self.lib.orc_zsyr2k(_ch(uplo), _ch(trans), allowed, n, k, _ptr(al), _ptr(a), a.shape[0], _ptr(b),
                            b.shape[0], _ptr(be), _ptr(c), c.shape[0], int(herm))

    def ztrmm(self, side, uplo, ta, diag, m, n, alpha, a, b):
        al = np.array([complex(alpha)])
        self.lib.orc_ztrmm(_ch(side), _ch(uplo), _ch(ta), _ch(diag), m, n, _ptr(al), _ptr(a), a.shape[0],
                           _ptr(b), b.shape[0])

    def ztrsm(self, side, uplo, ta, diag, m, n, alpha, a, b):
        al = np.array([complex(alpha)])
        self.lib.orc_ztrsm(_ch(side), _ch(uplo), _ch(ta), _ch(diag), m, n, _ptr(al), _ptr(a), a.shape[0],
                           _ptr(b), b.shape[0])

    def check_symm(self, side, uplo, m, n, lda, ldb, ldc):
        return self.lib.orc_check_symm(_ch(side), _ch(uplo), m, n, lda, ldb, ldc)

    def check_rank_k(self, uplo, trans, allowed, n, k, lda, ldc):
        return self.lib.orc_check_rank_k(_ch(uplo), _ch(trans), allowed, n, k, lda, ldc)

    def check_rank_2k(self, uplo, trans, allowed, n, k, lda, ldb, ldc):
        return self.lib.orc_check_rank_2k(_ch(uplo), _ch(trans), allowed, n, k, lda, ldb, ldc)

    def check_dgemm(self, ta, tb, m, n, k, lda, ldb, ldc):
        return self.lib.orc_check_dgemm(_ch(ta), _ch(tb), m, n, k, lda, ldb, ldc)

    def check_dtrsm(self, side, uplo, ta, diag, m, n, lda, ldb):
        return self.lib.orc_check_dtrsm(_ch(side), _ch(uplo), _ch(ta), _ch(diag), m, n, lda, ldb)

    def check_dsyrk(self, uplo, trans, n, k, lda, ldc):
        return self.lib.orc_check_dsyrk(_ch(uplo), _ch(trans), n, k, lda, ldc)

    def check_dgemv(self, trans, m, n, lda, incx, incy):
        return self.lib.orc_check_dgemv(_ch(trans), m, n, lda, incx, incy)

    # ---- accuracy ------------------------------------------------------------
    def dgemm_dd(self, ta, tb, m, n, k, alpha, a, b, beta, c):
        out = np.empty((max(1, m), n), dtype=np.float64, order="F")
        self.lib.orc_dgemm_dd(_ch(ta), _ch(tb), m, n, k, alpha, _ptr(a), a.shape[0],
                              _ptr(b), b.shape[0], beta, _ptr(c), c.shape[0],
                              _ptr(out), out.shape[0])
        return out

    def dgemm_dd_sample(self, ta, tb, k, alpha, a, b, beta, c, rows, cols):
        rows = np.ascontiguousarray(rows, dtype=np.int32)
        cols = np.ascontiguousarray(cols, dtype=np.int32)
        out = np.empty(len(rows), dtype=np.float64)
        self.lib.orc_dgemm_dd_sample(_ch(ta), _ch(tb), k, alpha, _ptr(a), a.shape[0],
                                     _ptr(b), b.shape[0], beta, _ptr(c), c.shape[0],
                                     len(rows), _ptr(rows), _ptr(cols), _ptr(out))
        return out

    def zgemm_dd_sample(self, ta, tb, k, alpha, a, b, beta, c, rows, cols):
        rows = np.ascontiguousarray(rows, dtype=np.int32)
        cols = np.ascontiguousarray(cols, dtype=np.int32)
        al = np.array([complex(alpha)], dtype=np.complex128)
        be = np.array([complex(beta)], dtype=np.complex128)
        out = np.empty(len(rows), dtype=np.complex128)
        self.lib.orc_zgemm_dd_sample(_ch(ta), _ch(tb), k, _ptr(al), _ptr(a), a.shape[0],
                                     _ptr(b), b.shape[0], _ptr(be), _ptr(c), c.shape[0],
                                     len(rows), _ptr(rows), _ptr(cols), _ptr(out))
        return out

    def dtrsm_residual(self, side, uplo, ta, diag, m, n, alpha, a, b0, x):
        return self.lib.orc_dtrsm_residual(_ch(side), _ch(uplo), _ch(ta), _ch(diag), m, n,
                                           alpha, _ptr(a), a.shape[0], _ptr(b0), b0.shape[0],
                                           _ptr(x), x.shape[0])

    def dtrsm_residual_cw(self, side, uplo, ta, diag, m, n, alpha, a, b0, x):
        return self.lib.orc_dtrsm_residual_cw(_ch(side), _ch(uplo), _ch(ta), _ch(diag), m, n,
                                              alpha, _ptr(a), a.shape[0], _ptr(b0), b0.shape[0],
                                              _ptr(x), x.shape[0])

    def rel_fro(self, m, n, x, ref):
        return self.lib.orc_rel_fro(m, n, _ptr(x), x.shape[0], _ptr(ref), ref.shape[0])


_ORACLE = None


def get() -> Oracle:
    global _ORACLE
    if _ORACLE is None:
        _ORACLE = Oracle()
    return _ORACLE
