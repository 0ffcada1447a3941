"""Host-side logic of bench.py without a GPU.

  * the blocked right-looking Cholesky call list of the serving trace (the
    open-loop form issues it from Python threads) is a factorisation: the
    calls, interpreted with numpy on the matrix they address, leave L with
    L L^T = A (relative error <= 1e-13), for ragged and exact block sizes;
  * the serving ratios and the bounds on any scheduler's gain follow their
    definitions.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def run_calls(calls, a, lda):
    """Interprets gbx_op records whose addresses are byte offsets into a."""
    def at(addr):
        off = (addr or 0) // 8
        return off % lda, off // lda

    for op in calls:
        if op.kind == 6:            # DPOTRF of the diagonal block, lower
            i, j = at(op.C)
            n = op.n
            blk = a[i:i + n, j:j + n]
            low = np.linalg.cholesky(np.tril(blk) + np.tril(blk, -1).T)
            blk[np.tril_indices(n)] = low[np.tril_indices(n)]
        elif op.kind == 2:          # DTRSM R, L, T, N: X L^T = B
            ai, aj = at(op.A)
            ci, cj = at(op.C)
            low = np.tril(a[ai:ai + op.n, aj:aj + op.n])
            b = a[ci:ci + op.m, cj:cj + op.n]
            b[:] = op.alpha * np.linalg.solve(low, b.T).T
        elif op.kind == 3:          # DSYRK L, N: lower(C) = alpha A A^T + beta C
            ai, aj = at(op.A)
            ci, cj = at(op.C)
            p = a[ai:ai + op.n, aj:aj + op.k]
            c = a[ci:ci + op.n, cj:cj + op.n]
            upd = op.alpha * (p @ p.T) + op.beta * c
            c[np.tril_indices(op.n)] = upd[np.tril_indices(op.n)]
        elif op.kind == 1:          # DGEMM N, T: C = alpha A B^T + beta C
            ai, aj = at(op.A)
            bi, bj = at(op.B)
            ci, cj = at(op.C)
            c = a[ci:ci + op.m, cj:cj + op.n]
            c[:] = op.alpha * (a[ai:ai + op.m, aj:aj + op.k] @ a[bi:bi + op.n, bj:bj + op.k].T) + op.beta * c
        else:
            raise AssertionError(f"unexpected kind {op.kind}")


@pytest.mark.parametrize("n,nb", [(300, 64), (256, 128), (97, 128), (513, 128)])
def test_cholesky_call_list_factors(lib, n, nb):
    import bench
    rng = np.random.default_rng(n + nb)
    g = rng.uniform(-1.0, 1.0, (n, n))
    spd = g @ g.T + n * np.eye(n)
    a = np.asfortranarray(spd.copy())
    calls = bench.cholesky_calls(n, nb, 0, n, 0)
    run_calls(calls, a, n)
    low = np.tril(a)
    assert np.linalg.norm(low @ low.T - spd) <= 1e-13 * np.linalg.norm(spd)
    nblk = -(-n // nb)
    # one DPOTRF per block column, one DTRSM per block column but the last,
    # one DSYRK per (block column, later block column), a DGEMM below it
    assert sum(op.kind == 6 for op in calls) == nblk
    assert sum(op.kind == 2 for op in calls) == nblk - 1
    assert sum(op.kind == 3 for op in calls) == nblk * (nblk - 1) // 2
    assert sum(op.kind == 1 for op in calls) == (nblk - 1) * (nblk - 2) // 2


def test_serving_ratios_and_bounds():
    import bench
    res = {
        "plain": {"calls_per_s": 100.0, "wall_s": 2.0, "flops": 3.0e12,
                  "chains": {"longest_alone_s": 0.8}},
        "served": {"calls_per_s": 110.0},
        "served_loop": {"calls_per_s": 50.0},
        "ozaki_plain": {"calls_per_s": 400.0, "wall_s": 0.5, "chains": {"longest_alone_s": 0.25}},
        "ozaki": {"calls_per_s": 440.0},
    }
    r = bench.serving_ratios(res, fp64_peak_tflops=2.0)
    assert r["served_vs_plain_fp64"] == pytest.approx(1.1)
    assert r["served_loop_vs_plain_fp64"] == pytest.approx(0.5)
    assert r["served_vs_plain_ozaki"] == pytest.approx(1.1)
    assert r["ozaki_plain_vs_fp64_plain"] == pytest.approx(4.0)
    assert r["ozaki_served_vs_fp64_plain"] == pytest.approx(4.4)
    assert r["plain_wall_over_longest_chain_fp64"] == pytest.approx(2.5)
    assert r["plain_wall_over_longest_chain_ozaki"] == pytest.approx(2.0)
    # the FP64 work at the pipe's rate: 3e12 flop / 2e12 flop/s = 1.5 s;
    # no scheduler beats the larger of that and the longest chain
    assert r["fp64_pipe_bound_s"] == pytest.approx(1.5)
    assert r["max_gain_fp64_any_scheduler"] == pytest.approx(2.0 / 1.5)
