"""gbx_ddot_noalloc, the dot product that allocates nothing, against the
regular gbx_ddot (which draws its scratch from the context workspace).

Callers that cannot allocate when they need a reduction (a malloc/free
interposer, code recording a CUDA graph, code under a fixed memory budget)
use this entry point; its scratch is a fixed 32 KiB device array, which
limits n to 2^28.  Tolerance is the one the Level-1 tests use:
|a - b| <= 2 * n * u * sum|x_i y_i|.  Two calls in a row must both agree
(the shared scratch keeps the previous call's contents and must not leak
into the next result).  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
U = 2.0 ** -53
NOALLOC_MAX_N = 4096 * 65536


def _fn(lib):
    f = lib.gbx_ddot_noalloc
    f.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p]
    f.restype = C.c_int
    return f


def test_ddot_noalloc_matches_ddot_twice(lib, orc, dev):
    import torch
    f = _fn(lib)
    stream = torch.cuda.current_stream().cuda_stream
    for n, incx, incy, seed in [(3 * (1 << 20) + 7, 1, 1, 41), (100003, 2, -3, 42)]:
        xh, s = orc.uniform(n * abs(incx), seed)
        yh, _ = orc.uniform(n * abs(incy), s)
        x = torch.from_numpy(xh).cuda()
        y = torch.from_numpy(yh).cuda()
        res_ref = torch.zeros(1, dtype=torch.float64, device="cuda")
        dev.ddot(n, x, incx, y, incy, res_ref)
        dev.sync()
        ref = res_ref.item()
        bound = 2 * n * U * float(np.abs(xh[::abs(incx)][:n]) @ np.abs(yh[::abs(incy)][:n]))
        res = torch.zeros(1, dtype=torch.float64, device="cuda")
        st = f(C.c_void_p(stream), n, C.c_void_p(x.data_ptr()), incx, C.c_void_p(y.data_ptr()),
               incy, C.c_void_p(res.data_ptr()))
        assert st == 0
        torch.cuda.synchronize()
        assert abs(res.item() - ref) <= bound
        assert abs(res.item() - orc.ddot_dd(n, xh, incx, yh, incy)) <= bound


def test_ddot_noalloc_limits(lib):
    import torch
    f = _fn(lib)
    x = torch.ones(16, dtype=torch.float64, device="cuda")
    res = torch.full((1,), 7.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    # beyond the scratch capacity: rejected before any launch, res untouched
    st = f(C.c_void_p(stream), NOALLOC_MAX_N + 1, C.c_void_p(x.data_ptr()), 1,
           C.c_void_p(x.data_ptr()), 1, C.c_void_p(res.data_ptr()))
    assert st == 1
    torch.cuda.synchronize()
    assert res.item() == 7.0
    st = f(C.c_void_p(stream), 0, C.c_void_p(x.data_ptr()), 1, C.c_void_p(x.data_ptr()), 1,
           C.c_void_p(res.data_ptr()))
    assert st == 0
    torch.cuda.synchronize()
    assert res.item() == 0.0
    st = f(C.c_void_p(stream), 16, C.c_void_p(x.data_ptr()), 1, C.c_void_p(x.data_ptr()), 1,
           C.c_void_p(res.data_ptr()))
    torch.cuda.synchronize()
    assert st == 0 and res.item() == 16.0
