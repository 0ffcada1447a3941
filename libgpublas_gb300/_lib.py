"""ctypes binding of libgbxblas.so.

Two views of the same library:

* ``F77``    -- the drop-in Fortran-ABI symbols (dgemm_, dtrsm_, ...) called
  exactly as a Fortran program calls them (every argument by reference), on
  host numpy arrays in Fortran order.
* ``Device`` -- the gbx_* C ABI over device pointers (torch CUDA tensors or
  raw integers), asynchronous on a context's stream.

There is no fallback: if the shared library is missing or fails to load, the
import error propagates.
"""
import ctypes as C
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbxblas.so")
DIAG_LIB_PATH = os.path.join(HERE, "libgbxdiag.so")
HEADERS = [os.path.join(os.path.dirname(HERE), "include", h)
           for h in ("gbxblas.h", "gbxblas_f77.h")]
DIAG_HEADERS = [os.path.join(os.path.dirname(HERE), "include", "gbxdiag.h")]

_P = C.c_void_p
_I = C.c_int
_D = C.c_double
_CH = C.c_char

_lib = None
_diag = None


def load(path=None):
    """Load libgbxblas.so (once).  Raises OSError if it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise OSError(f"{path} is missing: build it with __graft_entry__.build() "
                      "(libgpublas_gb300.build.build_library())")
    lib = C.CDLL(path, mode=C.RTLD_GLOBAL)
    _declare(lib)
    _lib = lib
    return lib


def load_diag():
    """Load libgbxdiag.so (benchmark and failure-path diagnostics; it
    resolves its calls into libgbxblas.so, loaded first)."""
    global _diag
    if _diag is not None:
        return _diag
    load()
    if not os.path.exists(DIAG_LIB_PATH):
        raise OSError(f"{DIAG_LIB_PATH} is missing: build it with __graft_entry__.build()")
    d = C.CDLL(DIAG_LIB_PATH)
    d.gbx_diag_fp64_peak.argtypes = [_P, C.POINTER(_D)]
    d.gbx_diag_expire_wait.argtypes = [_P]
    d.gbx_diag_pipe_rates.argtypes = [_P, _P]
    d.gbx_diag_ops_trace.argtypes = [_P, _I, _I, C.POINTER(_P), C.POINTER(_I), C.POINTER(TraceStats)]
    d.gbx_diag_mma_issue.argtypes = [_P, _I, _I, _I, C.POINTER(_D), C.POINTER(_D)]
    d.gbx_diag_cholesky_trace.argtypes = [_P, _I, _I, C.POINTER(_I), C.POINTER(_I), C.POINTER(_P),
                                          C.POINTER(_I), _P, _I, C.POINTER(TraceStats)]
    _diag = d
    return d


def declared_symbols(headers=None):
    """Function names declared in the public headers (default: those of
    libgbxblas.so; DIAG_HEADERS for libgbxdiag.so)."""
    names = []
    for h in headers or HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", text, flags=re.M):
            name = m.group(1)
            if name in ("if", "defined", "sizeof"):
                continue
            names.append(name)
    return sorted(set(names))


def _declare(L):
    pp = C.POINTER(_P)
    L.gbx_ctx_create.argtypes = [pp, _I]
    L.gbx_ctx_create.restype = _I
    L.gbx_ctx_destroy.argtypes = [_P]
    L.gbx_thread_ctx.restype = _P
    L.gbx_ctx_set_stream.argtypes = [_P, _P]
    L.gbx_ctx_get_stream.argtypes = [_P]
    L.gbx_ctx_get_stream.restype = _P
    L.gbx_ctx_sync.argtypes = [_P]
    L.gbx_ctx_reserve.argtypes = [_P, C.c_size_t]
    L.gbx_ctx_launches.argtypes = [_P]
    L.gbx_ctx_launches.restype = C.c_uint64
    L.gbx_ctx_last_error.argtypes = [_P]
    L.gbx_ctx_last_error.restype = C.c_char_p
    L.gbx_status_string.argtypes = [_I]
    L.gbx_status_string.restype = C.c_char_p
    L.gbx_daxpy.argtypes = [_P, _I, _D, _P, _I, _P, _I]
    L.gbx_dscal.argtypes = [_P, _I, _D, _P, _I]
    L.gbx_ddot.argtypes = [_P, _I, _P, _I, _P, _I, _P]
    L.gbx_dnrm2.argtypes = [_P, _I, _P, _I, _P]
    L.gbx_idamax.argtypes = [_P, _I, _P, _I, _P]
    L.gbx_idamin.argtypes = [_P, _I, _P, _I, _P]
    L.gbx_dgemv.argtypes = [_P, _CH, _I, _I, _D, _P, _I, _P, _I, _D, _P, _I]
    L.gbx_dgemm.argtypes = [_P, _CH, _CH, _I, _I, _I, _D, _P, _I, _P, _I, _D, _P, _I]
    L.gbx_zgemm.argtypes = [_P, _CH, _CH, _I, _I, _I, _P, _P, _I, _P, _I, _P, _P, _I]
    L.gbx_dsyrk.argtypes = [_P, _CH, _CH, _I, _I, _D, _P, _I, _D, _P, _I]
    L.gbx_dtrsm.argtypes = [_P, _CH, _CH, _CH, _CH, _I, _I, _D, _P, _I, _P, _I]
    L.gbx_dtrmm.argtypes = [_P, _CH, _CH, _CH, _CH, _I, _I, _D, _P, _I, _P, _I]
    L.gbx_dtrsm_ozaki.argtypes = [_P, _CH, _CH, _CH, _CH, _I, _I, _D, _P, _I, _P, _I, _D, _I, C.POINTER(_I)]
    L.gbx_dger.argtypes = [_P, _I, _I, _D, _P, _I, _P, _I, _P, _I]
    L.gbx_dsymv.argtypes = [_P, _CH, _I, _D, _P, _I, _P, _I, _D, _P, _I]
    L.gbx_dtrsv.argtypes = [_P, _CH, _CH, _CH, _I, _P, _I, _P, _I]
    # the Level-3 set in S/D/C/Z (complex scalars: pointers to host pairs)
    _F = C.c_float
    for p, S in (("s", _F), ("d", _D), ("c", _P), ("z", _P)):
        if p in "sc":
            getattr(L, f"gbx_{p}gemm").argtypes = [_P, _CH, _CH, _I, _I, _I, S, _P, _I, _P, _I, S, _P, _I]
        getattr(L, f"gbx_{p}symm").argtypes = [_P, _CH, _CH, _I, _I, S, _P, _I, _P, _I, S, _P, _I]
        getattr(L, f"gbx_{p}syr2k").argtypes = [_P, _CH, _CH, _I, _I, S, _P, _I, _P, _I, S, _P, _I]
        if p != "d":
            getattr(L, f"gbx_{p}syrk").argtypes = [_P, _CH, _CH, _I, _I, S, _P, _I, S, _P, _I]
            for r in ("trmm", "trsm"):
                getattr(L, f"gbx_{p}{r}").argtypes = [_P, _CH, _CH, _CH, _CH, _I, _I, S, _P, _I, _P, _I]
    for p, R in (("c", _F), ("z", _D)):
        getattr(L, f"gbx_{p}hemm").argtypes = [_P, _CH, _CH, _I, _I, _P, _P, _I, _P, _I, _P, _P, _I]
        getattr(L, f"gbx_{p}herk").argtypes = [_P, _CH, _CH, _I, _I, R, _P, _I, R, _P, _I]
        getattr(L, f"gbx_{p}her2k").argtypes = [_P, _CH, _CH, _I, _I, _P, _P, _I, _P, _I, R, _P, _I]
    L.gbx_dgemm_ozaki.argtypes = [_P, _CH, _CH, _I, _I, _I, _D, _P, _I, _P, _I, _D, _P, _I,
                                  _D, _I, C.POINTER(_I)]
    L.gbx_zgemm_ozaki.argtypes = [_P, _CH, _CH, _I, _I, _I, _P, _P, _I, _P, _I, _P, _P, _I,
                                  _D, _I, C.POINTER(_I)]
    L.gbx_dsyrk_ozaki.argtypes = [_P, _CH, _CH, _I, _I, _D, _P, _I, _D, _P, _I, _D, _I,
                                  C.POINTER(_I)]
    L.ddot_.restype = _D
    L.dnrm2_.restype = _D
    L.idamax_.restype = _I
    L.idamin_.restype = _I
    L.cblas_ddot.restype = _D
    L.cblas_ddot.argtypes = [_I, _P, _I, _P, _I]
    L.cblas_dnrm2.restype = _D
    L.cblas_dnrm2.argtypes = [_I, _P, _I]
    L.cblas_idamax.argtypes = [_I, _P, _I]
    L.cblas_idamin.argtypes = [_I, _P, _I]
    L.cblas_dgemm.argtypes = [_I, _I, _I, _I, _I, _I, _D, _P, _I, _P, _I, _D, _P, _I]
    L.gbx_stats.argtypes = [C.POINTER(C.c_uint64)] * 5
    L.gbx_plan_create.argtypes = [_P, _P, _I, C.POINTER(_P)]
    L.gbx_plan_launch.argtypes = [_P, _P]
    L.gbx_plan_graph_launch.argtypes = [_P, _P]
    L.gbx_plan_destroy.argtypes = [_P]
    L.gbx_plan_info.argtypes = [_P, C.POINTER(_I), C.POINTER(_D)]
    L.gbx_ops_run.argtypes = [_P, _P, _I]
    L.gbx_dpotrf_small.argtypes = [_P, _CH, _I, _P, _I, _P]
    L.gbx_server_create.argtypes = [_I, _I, C.c_size_t, C.POINTER(_P)]
    L.gbx_server_submit.argtypes = [_P, _P, C.POINTER(C.c_uint64)]
    L.gbx_server_wait.argtypes = [_P, C.c_uint64, C.POINTER(_D)]
    L.gbx_server_call.argtypes = [_P, _P, C.POINTER(_D)]
    L.gbx_server_admit.argtypes = [_P, C.c_size_t]
    L.gbx_server_release.argtypes = [_P, C.c_size_t]
    L.gbx_server_stats.argtypes = [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                   C.POINTER(C.c_uint64), C.POINTER(_D), C.POINTER(_D),
                                   C.POINTER(C.c_uint64)]
    L.gbx_server_reset_stats.argtypes = [_P]
    L.gbx_server_loop_stats.argtypes = [_P, C.POINTER(_I), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    L.gbx_server_destroy.argtypes = [_P]
    L.gbx_ctx_enable_timing.argtypes = [_P, _I]
    L.gbx_ctx_kernel_time.argtypes = [_P, _I, C.POINTER(_D), C.POINTER(C.c_uint64)]


class GbxOp(C.Structure):
    """gbx_op of include/gbxblas.h (one operation of a grouped plan)."""
    _fields_ = [("kind", C.c_int), ("transa", C.c_char), ("transb", C.c_char),
                ("side", C.c_char), ("uplo", C.c_char), ("diag", C.c_char),
                ("m", C.c_int), ("n", C.c_int), ("k", C.c_int),
                ("alpha", C.c_double), ("beta", C.c_double),
                ("A", C.c_void_p), ("lda", C.c_int), ("B", C.c_void_p), ("ldb", C.c_int),
                ("C", C.c_void_p), ("ldc", C.c_int)]


OP_GEMM, OP_TRSM, OP_SYRK, OP_DOT, OP_NRM2 = 1, 2, 3, 4, 5

TRACE_MAX_THREADS, TRACE_KINDS = 64, 16


class TraceStats(C.Structure):
    """gbx_trace_stats of include/gbxdiag.h."""
    _fields_ = [("calls", C.c_uint64), ("wall_s", C.c_double), ("p50_us", C.c_double),
                ("p99_us", C.c_double), ("kind_calls", C.c_uint64 * TRACE_KINDS),
                ("kind_sum_us", C.c_double * TRACE_KINDS),
                ("thread_finish_s", C.c_double * TRACE_MAX_THREADS), ("first_error", C.c_int)]


def cholesky_trace(server, device, n, nb, mats, info_ptr, ozaki):
    """Runs the native Cholesky-trace driver (gbx_diag_cholesky_trace):
    len(n) host threads, thread t factorising the device matrix whose address
    is mats[t] (n[t] x n[t], leading dimension n[t], block nb[t]); server is
    a Server or None (plain per-call dispatch).  Returns gbx_trace_stats as a
    dict."""
    L = load_diag()
    k = len(n)
    ni = (_I * k)(*n)
    nbi = (_I * k)(*nb)
    ai = (_P * k)(*mats)
    ld = (_I * k)(*n)
    out = TraceStats()
    st = L.gbx_diag_cholesky_trace(server.h if server else None, device, k, ni, nbi, ai, ld, info_ptr,
                                   1 if ozaki else 0, C.byref(out))
    if st != 0:
        raise GbxError(f"gbx_diag_cholesky_trace failed with status {st}")
    return {"calls": out.calls, "wall_s": out.wall_s, "p50_us": out.p50_us, "p99_us": out.p99_us,
            "kind_calls": list(out.kind_calls), "kind_sum_us": list(out.kind_sum_us),
            "thread_finish_s": list(out.thread_finish_s)[:k], "first_error": out.first_error}


def ops_trace(server, device, per_thread_ops):
    """Runs gbx_diag_ops_trace: thread t issues per_thread_ops[t] (a list of
    GbxOp) one call at a time; returns gbx_trace_stats as a dict."""
    L = load_diag()
    k = len(per_thread_ops)
    arrays = [(GbxOp * len(o))(*o) for o in per_thread_ops]
    ptrs = (_P * k)(*[C.cast(a, _P) for a in arrays])
    cnt = (_I * k)(*[len(o) for o in per_thread_ops])
    out = TraceStats()
    st = L.gbx_diag_ops_trace(server.h if server else None, device, k, ptrs, cnt, C.byref(out))
    if st != 0:
        raise GbxError(f"gbx_diag_ops_trace failed with status {st}")
    return {"calls": out.calls, "wall_s": out.wall_s, "p50_us": out.p50_us, "p99_us": out.p99_us,
            "first_error": out.first_error}


class Server:
    """The serving loop (gbx_server_*): calls from many threads on
    device-resident operands, continuously batched."""

    def __init__(self, device=0, slots=8, mem_budget=0):
        self.L = load()
        h = _P()
        st = self.L.gbx_server_create(device, slots, mem_budget, C.byref(h))
        if st != 0:
            raise GbxError(f"gbx_server_create failed with status {st}")
        self.h = h

    def call(self, op):
        lat = C.c_double(0.0)
        st = self.L.gbx_server_call(self.h, C.byref(op), C.byref(lat))
        return st, lat.value

    def submit(self, op):
        t = C.c_uint64(0)
        st = self.L.gbx_server_submit(self.h, C.byref(op), C.byref(t))
        if st != 0:
            raise GbxError(f"submit failed with status {st}")
        return t.value

    def wait(self, ticket):
        lat = C.c_double(0.0)
        st = self.L.gbx_server_wait(self.h, ticket, C.byref(lat))
        return st, lat.value

    def admit(self, nbytes):
        return self.L.gbx_server_admit(self.h, nbytes)

    def release(self, nbytes):
        return self.L.gbx_server_release(self.h, nbytes)

    def stats(self):
        c, b, g = C.c_uint64(), C.c_uint64(), C.c_uint64()
        p50, p99, w = C.c_double(), C.c_double(), C.c_uint64()
        self.L.gbx_server_stats(self.h, C.byref(c), C.byref(b), C.byref(g), C.byref(p50),
                                C.byref(p99), C.byref(w))
        return dict(completed=c.value, batches=b.value, grouped_calls=g.value, p50_us=p50.value,
                    p99_us=p99.value, admission_waits=w.value)

    def loop_stats(self):
        """(enabled, calls run on the device-side request loop, kernel launches)."""
        e, c, l = C.c_int(), C.c_uint64(), C.c_uint64()
        self.L.gbx_server_loop_stats(self.h, C.byref(e), C.byref(c), C.byref(l))
        return bool(e.value), c.value, l.value

    def reset_stats(self):
        self.L.gbx_server_reset_stats(self.h)

    def close(self):
        if self.h:
            self.L.gbx_server_destroy(self.h)
            self.h = None


def stats():
    L = load()
    v = [C.c_uint64() for _ in range(5)]
    L.gbx_stats(*[C.byref(x) for x in v])
    return dict(zip(("calls", "hits", "misses", "bytes_h2d", "bytes_d2h"), [x.value for x in v]))


class GbxError(RuntimeError):
    pass


def _ch(c):
    return c.encode() if isinstance(c, str) else c


def _byref_i(v):
    return C.byref(C.c_int(int(v)))


def _byref_d(v):
    return C.byref(C.c_double(float(v)))


def _hp(a):
    """Pointer to a host numpy array, or a raw integer address."""
    if a is None:
        return None
    if isinstance(a, int):
        return C.c_void_p(a)
    return a.ctypes.data_as(_P)


class F77:
    """The Fortran-ABI entry points, called by reference as Fortran does."""

    def __init__(self):
        self.L = load()

    def dgemm(self, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
        self.L.dgemm_(C.c_char_p(_ch(ta)), C.c_char_p(_ch(tb)), _byref_i(m), _byref_i(n),
                      _byref_i(k), _byref_d(alpha), _hp(a), _byref_i(lda), _hp(b), _byref_i(ldb),
                      _byref_d(beta), _hp(c), _byref_i(ldc))

    def zgemm(self, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
        al = np.array([complex(alpha)], dtype=np.complex128)
        be = np.array([complex(beta)], dtype=np.complex128)
        self.L.zgemm_(C.c_char_p(_ch(ta)), C.c_char_p(_ch(tb)), _byref_i(m), _byref_i(n),
                      _byref_i(k), _hp(al), _hp(a), _byref_i(lda), _hp(b), _byref_i(ldb), _hp(be),
                      _hp(c), _byref_i(ldc))

    def dsyrk(self, uplo, trans, n, k, alpha, a, lda, beta, c, ldc):
        self.L.dsyrk_(C.c_char_p(_ch(uplo)), C.c_char_p(_ch(trans)), _byref_i(n), _byref_i(k),
                      _byref_d(alpha), _hp(a), _byref_i(lda), _byref_d(beta), _hp(c), _byref_i(ldc))

    def dtrsm(self, side, uplo, ta, diag, m, n, alpha, a, lda, b, ldb):
        self.L.dtrsm_(C.c_char_p(_ch(side)), C.c_char_p(_ch(uplo)), C.c_char_p(_ch(ta)),
                      C.c_char_p(_ch(diag)), _byref_i(m), _byref_i(n), _byref_d(alpha), _hp(a),
                      _byref_i(lda), _hp(b), _byref_i(ldb))

    def dtrmm(self, side, uplo, ta, diag, m, n, alpha, a, lda, b, ldb):
        self.L.dtrmm_(C.c_char_p(_ch(side)), C.c_char_p(_ch(uplo)), C.c_char_p(_ch(ta)),
                      C.c_char_p(_ch(diag)), _byref_i(m), _byref_i(n), _byref_d(alpha), _hp(a),
                      _byref_i(lda), _hp(b), _byref_i(ldb))

    def dgemv(self, trans, m, n, alpha, a, lda, x, incx, beta, y, incy):
        self.L.dgemv_(C.c_char_p(_ch(trans)), _byref_i(m), _byref_i(n), _byref_d(alpha), _hp(a),
                      _byref_i(lda), _hp(x), _byref_i(incx), _byref_d(beta), _hp(y), _byref_i(incy))

    def daxpy(self, n, alpha, x, incx, y, incy):
        self.L.daxpy_(_byref_i(n), _byref_d(alpha), _hp(x), _byref_i(incx), _hp(y), _byref_i(incy))

    def ddot(self, n, x, incx, y, incy):
        return self.L.ddot_(_byref_i(n), _hp(x), _byref_i(incx), _hp(y), _byref_i(incy))

    def dnrm2(self, n, x, incx):
        return self.L.dnrm2_(_byref_i(n), _hp(x), _byref_i(incx))

    def idamax(self, n, x, incx):
        return self.L.idamax_(_byref_i(n), _hp(x), _byref_i(incx))

    def idamin(self, n, x, incx):
        return self.L.idamin_(_byref_i(n), _hp(x), _byref_i(incx))

    def dger(self, m, n, alpha, x, incx, y, incy, a, lda):
        self.L.dger_(_byref_i(m), _byref_i(n), _byref_d(alpha), _hp(x), _byref_i(incx), _hp(y), _byref_i(incy),
                     _hp(a), _byref_i(lda))

    def dsymv(self, uplo, n, alpha, a, lda, x, incx, beta, y, incy):
        self.L.dsymv_(C.c_char_p(_ch(uplo)), _byref_i(n), _byref_d(alpha), _hp(a), _byref_i(lda), _hp(x),
                      _byref_i(incx), _byref_d(beta), _hp(y), _byref_i(incy))

    def dtrsv(self, uplo, trans, diag, n, a, lda, x, incx):
        self.L.dtrsv_(C.c_char_p(_ch(uplo)), C.c_char_p(_ch(trans)), C.c_char_p(_ch(diag)), _byref_i(n), _hp(a),
                      _byref_i(lda), _hp(x), _byref_i(incx))

    # ---- the Level-3 family in every precision: p is 's', 'd', 'c' or 'z';
    # scalars are passed by reference in the routine's type (real for the
    # Hermitian alpha/beta that netlib declares real)
    @staticmethod
    def _s(p, v, real=False):
        if p in "sc":
            dt = np.float32 if (p == "s" or real) else np.complex64
        else:
            dt = np.float64 if (p == "d" or real) else np.complex128
        return np.array([v], dtype=dt)

    def _fn(self, name):
        return getattr(self.L, name + "_")

    def gemm(self, p, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
        al, be = self._s(p, alpha), self._s(p, beta)
        self._fn(p + "gemm")(C.c_char_p(_ch(ta)), C.c_char_p(_ch(tb)), _byref_i(m), _byref_i(n), _byref_i(k),
                             _hp(al), _hp(a), _byref_i(lda), _hp(b), _byref_i(ldb), _hp(be), _hp(c),
                             _byref_i(ldc))

    def symm(self, p, side, uplo, m, n, alpha, a, lda, b, ldb, beta, c, ldc, herm=False):
        al, be = self._s(p, alpha), self._s(p, beta)
        self._fn(p + ("hemm" if herm else "symm"))(
            C.c_char_p(_ch(side)), C.c_char_p(_ch(uplo)), _byref_i(m), _byref_i(n), _hp(al), _hp(a),
            _byref_i(lda), _hp(b), _byref_i(ldb), _hp(be), _hp(c), _byref_i(ldc))

    def syrk(self, p, uplo, trans, n, k, alpha, a, lda, beta, c, ldc, herm=False):
        al, be = self._s(p, alpha, herm), self._s(p, beta, herm)
        self._fn(p + ("herk" if herm else "syrk"))(
            C.c_char_p(_ch(uplo)), C.c_char_p(_ch(trans)), _byref_i(n), _byref_i(k), _hp(al), _hp(a),
            _byref_i(lda), _hp(be), _hp(c), _byref_i(ldc))

    def syr2k(self, p, uplo, trans, n, k, alpha, a, lda, b, ldb, beta, c, ldc, herm=False):
        al, be = self._s(p, alpha), self._s(p, beta, herm)
        self._fn(p + ("her2k" if herm else "syr2k"))(
            C.c_char_p(_ch(uplo)), C.c_char_p(_ch(trans)), _byref_i(n), _byref_i(k), _hp(al), _hp(a),
            _byref_i(lda), _hp(b), _byref_i(ldb), _hp(be), _hp(c), _byref_i(ldc))

    def trxm(self, p, routine, side, uplo, ta, diag, m, n, alpha, a, lda, b, ldb):
        al = self._s(p, alpha)
        self._fn(p + routine)(C.c_char_p(_ch(side)), C.c_char_p(_ch(uplo)), C.c_char_p(_ch(ta)),
                              C.c_char_p(_ch(diag)), _byref_i(m), _byref_i(n), _hp(al), _hp(a), _byref_i(lda),
                              _hp(b), _byref_i(ldb))


def _dp(t):
    """Device pointer of a torch tensor (or an int address)."""
    if t is None:
        return None
    if isinstance(t, int):
        return C.c_void_p(t)
    return C.c_void_p(t.data_ptr())


class Device:
    """A gbx context and the device-pointer C ABI."""

    def __init__(self, device=0, stream=None):
        self.L = load()
        h = _P()
        st = self.L.gbx_ctx_create(C.byref(h), device)
        if st != 0:
            raise GbxError(f"gbx_ctx_create failed with status {st}")
        self.ctx = h
        if stream is not None:
            self.L.gbx_ctx_set_stream(self.ctx, C.c_void_p(stream))

    @classmethod
    def of_thread(cls):
        """The calling thread's own context (the one the Fortran-ABI symbols
        use), wrapped without taking ownership: close() leaves it alive."""
        self = cls.__new__(cls)
        self.L = load()
        self.L.gbx_thread_ctx.restype = _P
        h = self.L.gbx_thread_ctx()
        if not h:
            raise GbxError("gbx_thread_ctx failed")
        self.ctx = _P(h)
        self._borrowed = True
        return self

    def close(self):
        if self.ctx:
            if not getattr(self, "_borrowed", False):
                self.L.gbx_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, st, what):
        if st != 0:
            msg = self.L.gbx_ctx_last_error(self.ctx).decode(errors="replace")
            raise GbxError(f"{what}: {self.L.gbx_status_string(st).decode()} ({msg})")

    def status(self, st):
        return st

    def sync(self):
        self._ok(self.L.gbx_ctx_sync(self.ctx), "sync")

    def launches(self):
        return self.L.gbx_ctx_launches(self.ctx)

    def stream(self):
        return self.L.gbx_ctx_get_stream(self.ctx)

    def set_stream(self, s):
        self.L.gbx_ctx_set_stream(self.ctx, C.c_void_p(s) if s else None)

    def last_error(self):
        return self.L.gbx_ctx_last_error(self.ctx).decode(errors="replace")

    TIMER_GEMM_FP64, TIMER_OZAKI_MMA, TIMER_OZAKI_SPLIT = 1, 2, 3
    TIMER_LEVEL1, TIMER_GEMV, TIMER_BATCH = 4, 5, 6
    TIMER_H2D, TIMER_D2H = 7, 8

    def enable_timing(self, on=True):
        self._ok(self.L.gbx_ctx_enable_timing(self.ctx, 1 if on else 0), "enable_timing")

    def kernel_time(self, tag):
        """(total milliseconds, launches) recorded for one timer tag."""
        ms, n = C.c_double(0.0), C.c_uint64(0)
        self._ok(self.L.gbx_ctx_kernel_time(self.ctx, tag, C.byref(ms), C.byref(n)), "kernel_time")
        return ms.value, n.value

    # grouped plans
    def plan_create(self, ops):
        arr = (GbxOp * len(ops))(*ops)
        h = _P()
        self._ok(self.L.gbx_plan_create(self.ctx, arr, len(ops), C.byref(h)), "plan_create")
        return h

    def plan_launch(self, plan, graph=False):
        f = self.L.gbx_plan_graph_launch if graph else self.L.gbx_plan_launch
        self._ok(f(self.ctx, plan), "plan_launch")

    def ops_run(self, ops_array, count):
        """Issue each operation alone through the regular routines."""
        self._ok(self.L.gbx_ops_run(self.ctx, ops_array, count), "ops_run")

    def dpotrf_small(self, n, a, lda, info):
        self._ok(self.L.gbx_dpotrf_small(self.ctx, b"L", n, _dp(a), lda, _dp(info)), "dpotrf_small")

    def plan_destroy(self, plan):
        self.L.gbx_plan_destroy(plan)

    def plan_info(self, plan):
        n, fl = C.c_int(0), C.c_double(0.0)
        self.L.gbx_plan_info(plan, C.byref(n), C.byref(fl))
        return n.value, fl.value

    def fp64_peak(self):
        t = C.c_double(0.0)
        self._ok(load_diag().gbx_diag_fp64_peak(self.ctx, C.byref(t)), "fp64_peak")
        return t.value

    def pipe_rates(self):
        """gbx_diag_pipe_rates as a dict (TFLOP/s, TOP/s, cycles)."""
        class Rates(C.Structure):
            _fields_ = [("dfma", _D), ("dmma", _D), ("imma", _D), ("hmma_bf16", _D), ("qmma_e4m3", _D),
                        ("mix", _D * 3), ("lat", (_D * 5) * 3)]
        r = Rates()
        self._ok(load_diag().gbx_diag_pipe_rates(self.ctx, C.byref(r)), "pipe_rates")
        names = ("dfma", "ffma", "dmul", "lds_dfma", "shfl_dmul")
        return {"dfma_tflops": r.dfma, "dmma_tflops": r.dmma, "imma_s8_tops": r.imma,
                "hmma_bf16_tflops": r.hmma_bf16, "qmma_e4m3_tflops": r.qmma_e4m3,
                "mix_dfma_only_tflops": r.mix[0], "mix_dmma_only_tflops": r.mix[1],
                "mix_half_half_tflops": r.mix[2],
                "latency_cycles": {str(t): dict(zip(names, list(r.lat[i])))
                                   for i, t in enumerate((1, 32, 256))}}

    def mma_issue(self, n, count, grid):
        """(issue, completion) SM cycles per tcgen05.mma of width n."""
        a, b = C.c_double(), C.c_double()
        self._ok(load_diag().gbx_diag_mma_issue(self.ctx, n, count, grid, C.byref(a), C.byref(b)), "mma_issue")
        return a.value, b.value

    def expire_wait(self):
        """Launch the diagnostic whose bounded device wait runs out (about
        2 s); the next sync reports GBX_ERR_TIMEOUT."""
        self._ok(load_diag().gbx_diag_expire_wait(self.ctx), "expire_wait")

    # Level 1
    def daxpy(self, n, alpha, x, incx, y, incy):
        self._ok(self.L.gbx_daxpy(self.ctx, n, alpha, _dp(x), incx, _dp(y), incy), "daxpy")

    def dscal(self, n, alpha, x, incx):
        self._ok(self.L.gbx_dscal(self.ctx, n, alpha, _dp(x), incx), "dscal")

    def ddot(self, n, x, incx, y, incy, res):
        self._ok(self.L.gbx_ddot(self.ctx, n, _dp(x), incx, _dp(y), incy, _dp(res)), "ddot")

    def dnrm2(self, n, x, incx, res):
        self._ok(self.L.gbx_dnrm2(self.ctx, n, _dp(x), incx, _dp(res)), "dnrm2")

    def idamax(self, n, x, incx, res):
        self._ok(self.L.gbx_idamax(self.ctx, n, _dp(x), incx, _dp(res)), "idamax")

    def idamin(self, n, x, incx, res):
        self._ok(self.L.gbx_idamin(self.ctx, n, _dp(x), incx, _dp(res)), "idamin")

    # Level 2 / 3
    def dgemv(self, trans, m, n, alpha, a, lda, x, incx, beta, y, incy):
        self._ok(self.L.gbx_dgemv(self.ctx, _ch(trans), m, n, alpha, _dp(a), lda, _dp(x), incx,
                                  beta, _dp(y), incy), "dgemv")

    def dgemm(self, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
        return self.L.gbx_dgemm(self.ctx, _ch(ta), _ch(tb), m, n, k, alpha, _dp(a), lda, _dp(b),
                                ldb, beta, _dp(c), ldc)

    def dgemm_checked(self, *args):
        self._ok(self.dgemm(*args), "dgemm")

    def zgemm(self, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
        al = (C.c_double * 2)(complex(alpha).real, complex(alpha).imag)
        be = (C.c_double * 2)(complex(beta).real, complex(beta).imag)
        self._ok(self.L.gbx_zgemm(self.ctx, _ch(ta), _ch(tb), m, n, k, al, _dp(a), lda, _dp(b),
                                  ldb, be, _dp(c), ldc), "zgemm")

    def dsyrk(self, uplo, trans, n, k, alpha, a, lda, beta, c, ldc):
        self._ok(self.L.gbx_dsyrk(self.ctx, _ch(uplo), _ch(trans), n, k, alpha, _dp(a), lda, beta,
                                  _dp(c), ldc), "dsyrk")

    def dtrsm(self, side, uplo, ta, diag, m, n, alpha, a, lda, b, ldb):
        self._ok(self.L.gbx_dtrsm(self.ctx, _ch(side), _ch(uplo), _ch(ta), _ch(diag), m, n, alpha,
                                  _dp(a), lda, _dp(b), ldb), "dtrsm")

    def dtrmm(self, side, uplo, ta, diag, m, n, alpha, a, lda, b, ldb):
        self._ok(self.L.gbx_dtrmm(self.ctx, _ch(side), _ch(uplo), _ch(ta), _ch(diag), m, n, alpha,
                                  _dp(a), lda, _dp(b), ldb), "dtrmm")

    def dgemm_ozaki(self, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, tol=0.0, slices=0,
                    want_slices=True):
        """Returns the slice count used (a stream synchronisation), or None
        with want_slices=False (the call stays asynchronous)."""
        used = C.c_int(0)
        self._ok(self.L.gbx_dgemm_ozaki(self.ctx, _ch(ta), _ch(tb), m, n, k, alpha, _dp(a), lda,
                                        _dp(b), ldb, beta, _dp(c), ldc, tol, slices,
                                        C.byref(used) if want_slices else None), "dgemm_ozaki")
        return used.value if want_slices else None

    def zgemm_ozaki(self, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, tol=0.0, slices=0):
        al = (C.c_double * 2)(complex(alpha).real, complex(alpha).imag)
        be = (C.c_double * 2)(complex(beta).real, complex(beta).imag)
        used = C.c_int(0)
        self._ok(self.L.gbx_zgemm_ozaki(self.ctx, _ch(ta), _ch(tb), m, n, k, al, _dp(a), lda,
                                        _dp(b), ldb, be, _dp(c), ldc, tol, slices,
                                        C.byref(used)), "zgemm_ozaki")
        return used.value

    def dsyrk_ozaki(self, uplo, trans, n, k, alpha, a, lda, beta, c, ldc, tol=0.0, slices=0):
        used = C.c_int(0)
        self._ok(self.L.gbx_dsyrk_ozaki(self.ctx, _ch(uplo), _ch(trans), n, k, alpha, _dp(a), lda,
                                        beta, _dp(c), ldc, tol, slices, C.byref(used)),
                 "dsyrk_ozaki")
        return used.value

    def dtrsm_ozaki(self, side, uplo, ta, diag, m, n, alpha, a, lda, b, ldb, tol=0.0, slices=0):
        used = C.c_int(0)
        self._ok(self.L.gbx_dtrsm_ozaki(self.ctx, _ch(side), _ch(uplo), _ch(ta), _ch(diag), m, n, alpha, _dp(a),
                                        lda, _dp(b), ldb, tol, slices, C.byref(used)), "dtrsm_ozaki")
        return used.value
