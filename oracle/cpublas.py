"""ctypes handle on the CPU BLAS that the reference's runnable path ends in.

TEST INFRASTRUCTURE / CPU BASELINE ONLY.

The reference forwards every call it does not (or cannot) run on the GPU to the
next ``dgemm_`` in the link order, found with ``dlsym(RTLD_NEXT, name)``
(runtime-blas.c:60-69; the size cutoff is gemm.cc:129-141).  Its build takes
whatever ``dependency('blas')`` resolves to (meson.build:100-104, unpinned).
This module binds SciPy's bundled OpenBLAS (LP64, 32-bit integers, the Fortran
default-integer ABI), which exports the Fortran symbols with a ``scipy_``
prefix.  The library is present on x86-64 and aarch64 SciPy wheels alike.
"""
import ctypes as C
import glob
import os

import numpy as np

_P = C.c_void_p
_I = C.POINTER(C.c_int)
_D = C.POINTER(C.c_double)


def find_openblas():
    """Path of SciPy's bundled OpenBLAS, or None."""
    try:
        import scipy
    except ImportError:
        return None
    root = os.path.dirname(os.path.dirname(os.path.abspath(scipy.__file__)))
    hits = sorted(glob.glob(os.path.join(root, "scipy.libs", "libscipy_openblas*.so*")))
    return hits[0] if hits else None


def _i(v):
    return C.byref(C.c_int(int(v)))


def _d(v):
    return C.byref(C.c_double(float(v)))


def _c(ch):
    return C.c_char_p(ch.encode() if isinstance(ch, str) else ch)


def _ptr(a):
    return a.ctypes.data_as(_P)


class CpuBlas:
    def __init__(self, path=None):
        path = path or find_openblas()
        if path is None:
            raise OSError("no CPU BLAS found (SciPy's bundled OpenBLAS is missing)")
        self.path = path
        self.lib = C.CDLL(path)
        pre = "scipy_" if hasattr(self.lib, "scipy_dgemm_") else ""
        self._f = lambda name: getattr(self.lib, pre + name)
        self._f("ddot_").restype = C.c_double
        self._f("dnrm2_").restype = C.c_double
        self._f("idamax_").restype = C.c_int
        self._f("idamin_").restype = C.c_int
        # raise xerbla to a Python-visible no-op: OpenBLAS's xerbla prints and
        # returns, which is what the tests expect from an invalid call.
        try:
            self._set_threads = self._f("openblas_set_num_threads")
            self._get_threads = self._f("openblas_get_num_threads")
            self._get_threads.restype = C.c_int
        except AttributeError:
            self._set_threads = self._get_threads = None
        try:
            cfg = self._f("openblas_get_config")
            cfg.restype = C.c_char_p
            self.config = cfg().decode()
        except AttributeError:
            self.config = "unknown"

    def set_threads(self, n):
        if self._set_threads is not None:
            self._set_threads(C.c_int(int(n)))

    def threads(self):
        return self._get_threads() if self._get_threads is not None else 1

    # ---- Fortran-ABI calls (arrays in Fortran order, ld = shape[0]) -------
    def dgemm(self, ta, tb, m, n, k, alpha, a, b, beta, c):
        self._f("dgemm_")(_c(ta), _c(tb), _i(m), _i(n), _i(k), _d(alpha), _ptr(a),
                          _i(a.shape[0]), _ptr(b), _i(b.shape[0]), _d(beta), _ptr(c),
                          _i(c.shape[0]))

    def dgemm_raw(self, ta, tb, m, n, k, alpha, pa, lda, pb, ldb, beta, pc, ldc):
        self._f("dgemm_")(_c(ta), _c(tb), _i(m), _i(n), _i(k), _d(alpha), pa, _i(lda),
                          pb, _i(ldb), _d(beta), pc, _i(ldc))

    def zgemm(self, ta, tb, m, n, k, alpha, a, b, beta, c):
        al = np.array([complex(alpha)], dtype=np.complex128)
        be = np.array([complex(beta)], dtype=np.complex128)
        self._f("zgemm_")(_c(ta), _c(tb), _i(m), _i(n), _i(k), _ptr(al), _ptr(a),
                          _i(a.shape[0]), _ptr(b), _i(b.shape[0]), _ptr(be), _ptr(c),
                          _i(c.shape[0]))

    def dsyrk(self, uplo, trans, n, k, alpha, a, beta, c):
        self._f("dsyrk_")(_c(uplo), _c(trans), _i(n), _i(k), _d(alpha), _ptr(a),
                          _i(a.shape[0]), _d(beta), _ptr(c), _i(c.shape[0]))

    def dtrsm(self, side, uplo, ta, diag, m, n, alpha, a, b):
        self._f("dtrsm_")(_c(side), _c(uplo), _c(ta), _c(diag), _i(m), _i(n), _d(alpha),
                          _ptr(a), _i(a.shape[0]), _ptr(b), _i(b.shape[0]))

    def dtrmm(self, side, uplo, ta, diag, m, n, alpha, a, b):
        self._f("dtrmm_")(_c(side), _c(uplo), _c(ta), _c(diag), _i(m), _i(n), _d(alpha),
                          _ptr(a), _i(a.shape[0]), _ptr(b), _i(b.shape[0]))

    def dgemv(self, trans, m, n, alpha, a, x, incx, beta, y, incy):
        self._f("dgemv_")(_c(trans), _i(m), _i(n), _d(alpha), _ptr(a), _i(a.shape[0]),
                          _ptr(x), _i(incx), _d(beta), _ptr(y), _i(incy))

    def daxpy(self, n, alpha, x, incx, y, incy):
        self._f("daxpy_")(_i(n), _d(alpha), _ptr(x), _i(incx), _ptr(y), _i(incy))

    def ddot(self, n, x, incx, y, incy):
        return self._f("ddot_")(_i(n), _ptr(x), _i(incx), _ptr(y), _i(incy))

    def dnrm2(self, n, x, incx):
        return self._f("dnrm2_")(_i(n), _ptr(x), _i(incx))

    def idamax(self, n, x, incx):
        return self._f("idamax_")(_i(n), _ptr(x), _i(incx))

    def idamin(self, n, x, incx):
        return self._f("idamin_")(_i(n), _ptr(x), _i(incx))


_CPU = None


def get() -> CpuBlas:
    global _CPU
    if _CPU is None:
        _CPU = CpuBlas()
    return _CPU
