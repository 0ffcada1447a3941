"""libgpublas_gb300 -- GB300-native BLAS offload library (libgbxblas.so).

The product is the C shared library ``libgbxblas.so`` built from ``csrc/``:
Fortran-ABI and CBLAS drop-in symbols over hand-written sm_103a kernels, plus
the gbx_* device-pointer C ABI declared in ``include/gbxblas.h``.  This
Python package only builds it (``build.build_library``) and binds it with
ctypes (``_lib``) for tests and benchmarks.  ``libgbxdiag.so`` (from
``csrc_diag/``, declared in ``include/gbxdiag.h``) holds the diagnostics the
benchmarks and failure-path tests use; the BLAS library does not need it.
"""
from ._lib import (F77, OP_DOT, OP_GEMM, OP_NRM2, OP_SYRK, OP_TRSM, Device, GbxError, GbxOp,  # noqa: F401
                   DIAG_HEADERS, DIAG_LIB_PATH, LIB_PATH, Server, cholesky_trace, declared_symbols, load,
                   load_diag, ops_trace, stats)
