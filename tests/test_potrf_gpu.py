"""gbx_dpotrf_small: the diagonal-block Cholesky of the blocked factorization
(lower, n <= 256), in 64-column steps.  Checked against numpy's Cholesky on
SPD blocks (relative Frobenius error 1e-13), the strict upper triangle left
untouched, and the LAPACK info convention on a block whose 1-based column j
has a non-positive pivot."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def spd(n, seed):
    rng = np.random.default_rng(seed)
    g = rng.uniform(-1, 1, (n, n))
    return g @ g.T + n * np.eye(n)


@pytest.mark.parametrize("n", [1, 2, 63, 64, 65, 130, 200, 256])
def test_dpotrf_small_matches_numpy(dev, n):
    import torch
    a = spd(n, n)
    lda = n + 5
    big = np.zeros((lda, n))
    big[:n] = a
    big[n:] = 7.0
    A = torch.from_numpy(np.ascontiguousarray(big.T)).cuda()
    info = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    st = dev.dpotrf_small(n, A.data_ptr(), lda, info.data_ptr())
    assert st in (0, None)
    dev.sync()
    got = A.cpu().numpy().T
    assert int(info.item()) == 0
    ref = np.linalg.cholesky(a)
    low = np.tril(got[:n])
    assert np.linalg.norm(low - ref) <= 1e-13 * np.linalg.norm(ref)
    assert np.array_equal(np.triu(got[:n], 1), np.triu(a, 1))   # upper untouched
    assert np.all(got[n:] == 7.0)                               # rows below n untouched


@pytest.mark.parametrize("n,bad", [(100, 1), (100, 64), (200, 130), (256, 256)])
def test_dpotrf_small_info(dev, n, bad):
    import torch
    a = spd(n, 3)
    # make the leading (bad x bad) minor indefinite: pivot bad fails first
    a[bad - 1, bad - 1] = -abs(a[bad - 1, bad - 1]) - 1e6
    A = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    dev.dpotrf_small(n, A.data_ptr(), n, info.data_ptr())
    dev.sync()
    assert int(info.item()) == bad
