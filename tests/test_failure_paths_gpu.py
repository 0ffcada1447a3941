"""Failure paths, made without a GPU fault.

* A bounded device wait that runs out: the diagnostic launch waits, through
  the tensor-core kernels' own bounded mbarrier wait, on a barrier nothing
  arrives on.  The wait gives up after its limit (2 s), the status reaches
  the host through the context's mapped mirror, gbx_ctx_sync returns
  GBX_ERR_TIMEOUT, and the same context then runs Ozaki products (whose
  kernels use the same waits and status word) correctly.
* A device allocation that fails: GBX_FAULT_ALLOC=<n> makes the n-th
  workspace allocation of the process report failure on the host, before
  any device call.  The Fortran-ABI call reports it (errors=return), leaves
  the caller's output untouched, and the next call succeeds.

The reference aborts the process on any runtime failure
(runtime.c:208-213); here the status reaches the caller.
"""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GBX_ERR_TIMEOUT = 4


def to_dev(a):
    # the library's context stream does not order with torch's stream: the
    # copy is complete before the call is issued
    import torch
    t = torch.from_numpy(np.asfortranarray(a).ravel(order="F").copy()).cuda()
    torch.cuda.synchronize()
    return t


def test_expired_wait_reports_timeout_and_context_recovers(orc, lib):
    import time
    import libgpublas_gb300 as g
    d = g.Device(0)
    try:
        t0 = time.perf_counter()
        d.expire_wait()
        st = d.L.gbx_ctx_sync(d.ctx)
        waited = time.perf_counter() - t0
        assert st == GBX_ERR_TIMEOUT, (st, d.last_error())
        assert "bounded device wait" in d.last_error()
        assert 1.5 <= waited <= 30.0, waited
        assert d.L.gbx_ctx_sync(d.ctx) == 0          # the status was cleared
        # the same context runs both Ozaki product kernels (bounded waits,
        # shared status word) and the FP64 path correctly afterwards
        for m, n, k in [(256, 192, 2048), (200, 96, 128)]:
            a, s = orc.matrix(m, k, 11 + k)
            b, s = orc.matrix(k, n, s)
            c, _ = orc.matrix(m, n, s)
            ref = orc.dgemm_dd("N", "N", m, n, k, 1.0, a, b, 0.5, c)
            C = to_dev(c)
            d.dgemm_ozaki("N", "N", m, n, k, 1.0, to_dev(a), m, to_dev(b), k, 0.5, C, m)
            got = C.cpu().numpy().reshape(m, n, order="F")
            assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-14
            C = to_dev(c)
            d.dgemm_checked("N", "N", m, n, k, 1.0, to_dev(a), m, to_dev(b), k, 0.5, C, m)
            d.sync()
            got = C.cpu().numpy().reshape(m, n, order="F")
            assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-13
    finally:
        d.close()


CHILD = textwrap.dedent("""
    import numpy as np, oracle, libgpublas_gb300 as g
    orc = oracle.get(); f = g.F77()
    m = n = k = 300
    a, s = orc.matrix(m, k, 1); b, s = orc.matrix(k, n, s); c, s = orc.matrix(m, n, s)
    ref = orc.dgemm_dd('N', 'N', m, n, k, 1.0, a, b, 0.5, c)
    got = c.copy(order='F')
    f.dgemm('N', 'N', m, n, k, 1.0, a, m, b, k, 0.5, got, m)
    print('UNCHANGED', bool(np.array_equal(got, c)))
    f.dgemm('N', 'N', m, n, k, 1.0, a, m, b, k, 0.5, got, m)
    print('ERR', np.linalg.norm(got - ref) / np.linalg.norm(ref))
""")


@pytest.mark.parametrize("nth", [1, 3])     # staging of A fails; staging of C fails
def test_injected_allocation_failure_reports_and_recovers(lib, nth):
    env = dict(os.environ, PYTHONPATH=ROOT, GBX_FAULT_ALLOC=str(nth), BLAS2CUDA_OPTIONS="errors=return")
    r = subprocess.run([sys.executable, "-c", CHILD], capture_output=True, text=True, env=env, cwd=ROOT,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "DGEMM failed" in r.stderr and "injected allocation failure" in r.stderr, r.stderr[-2000:]
    assert "UNCHANGED True" in r.stdout, r.stdout
    err = float(r.stdout.split("ERR")[1])
    assert err <= 1e-13
