"""Batched AMG-PCG (one persistent launch for many independent systems)
against the CPU oracle.

The systems are the diagonal blocks of one matrix; the oracle sets up the same
block-diagonal matrix and solves each system by its ordinary PCG on a
right-hand side that is zero outside the system (every operation of the
hierarchy is block local, so that is the system's own solve).  FP64 cycle:
residual histories to 1e-10 and equal iteration counts; FP32 cycle: every
system's FP64 true residual below the tolerance."""
import numpy as np
import pytest

from hypre_gb300 import problems as G

pytestmark = pytest.mark.gpu


def _csr(I, J, V):
    import scipy.sparse as sp
    n = len(I) - 1
    return sp.csr_matrix((V, J, I), shape=(n, n))


def _batch(gb, I, J, V, off, prec, shape=None, maxit=100):
    n = len(I) - 1
    A = gb.IJMatrix(I, J, V)
    amg = gb.BoomerAMG(StrongThreshold=0.25, RelaxType=18, Tol=0.0, MaxIter=1)
    bp = gb.BatchedPCG(amg, tol=1e-8, maxit=maxit, prec=prec, shape=shape)
    bp.setup(A, off)
    return A, amg, bp, n


def test_batched_fp64_matches_oracle(gb, oracle_mod):
    O = oracle_mod
    I, J, V, off, ns, eps = G.aniso2d_batch(24, nmin=6, nmax=22, seed=5)
    A, amg, bp, n = _batch(gb, I, J, V, off, prec=0, shape=(2, 128))
    H = O.Hierarchy(I, J, V, O.default_params(strong_threshold=0.25))
    assert amg.num_levels() == H.num_levels
    for l in range(H.num_levels):
        Ig, Jg, Vg, _ = amg.level_csr(l, "A")
        Io, Jo, Vo, _ = H.csr("A", l)
        assert np.array_equal(Jg, Jo) and np.array_equal(Vg, Vo), f"A{l}"
        lo = bp.level_offsets(l)
        assert lo[0] == 0 and lo[-1] == len(Io) - 1
    b = O.rand_uniform(n, 22775)
    bv, xv = gb.IJVector(n, b), gb.IJVector(n, np.zeros(n))
    assert bp.solve(bv, xv) == 0
    its = bp.iterations()
    for s in range(len(ns)):
        be = np.zeros(n)
        be[off[s]:off[s + 1]] = b[off[s]:off[s + 1]]
        _, rel_o, it_o = H.pcg(be, tol=1e-8, maxit=100)
        assert its[s] == it_o, f"system {s}"
        np.testing.assert_allclose(bp.history(s), rel_o, rtol=1e-10, atol=0, err_msg=f"system {s}")


@pytest.mark.parametrize("num", [64, 512])
def test_batched_fp32_cycle_converges(gb, oracle_mod, num):
    """FP32 V-cycle inside FP64 PCG, n in [16, 128], eps log-uniform in [1e-3, 1]:
    every system reaches FP64 true ||r||/||b|| < 1e-8 (autotuned kernel shape)."""
    I, J, V, off, ns, eps = G.aniso2d_batch(num, seed=11)
    A, amg, bp, n = _batch(gb, I, J, V, off, prec=1)
    b = oracle_mod.rand_uniform(n, 22775)
    bv, xv = gb.IJVector(n, b), gb.IJVector(n, np.zeros(n))
    assert bp.solve(bv, xv) == 0
    x = xv.values()
    r = b - _csr(I, J, V) @ x
    for s in range(num):
        sl = slice(off[s], off[s + 1])
        assert np.linalg.norm(r[sl]) < 1e-8 * np.linalg.norm(b[sl]), f"system {s} (n={ns[s]}, eps={eps[s]:.2e})"
    assert np.all(bp.relres() < 1e-8)
    lpr, blk = bp.shape()
    assert lpr in (1, 2, 4, 8) and blk in (128, 256, 512)
    assert np.all(bp.tuning_times() > 0)


def test_batched_rejects_coupled_systems(gb):
    I, J, V, off, ns, eps = G.aniso2d_batch(4, nmin=6, nmax=8, seed=1)
    off = off.copy()
    off[2] += 1          # a split that cuts through a system's couplings
    n = len(I) - 1
    A = gb.IJMatrix(I, J, V)
    amg = gb.BoomerAMG(Tol=0.0, MaxIter=1)
    bp = gb.BatchedPCG(amg)
    rc = gb.lib().HYPRE_GB300_BatchedPCGSetup(bp.h, amg.h, A.par, 4, off.ctypes.data)
    assert rc != 0
    gb.lib().HYPRE_ClearAllErrors()
