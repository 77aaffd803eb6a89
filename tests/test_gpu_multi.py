"""Multiple right-hand sides: PCG on multi-vectors (one PCG per column, SpMM
V-cycle) against the single-vector PCG of each column (FP64 cycle: residual
histories to 1e-10, equal iteration counts) and the FP32-cycle variant to the
FP64 true residual."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _csr(I, J, V):
    import scipy.sparse as sp
    n = len(I) - 1
    return sp.csr_matrix((V, J, I), shape=(n, n))


@pytest.mark.parametrize("nv", [1, 5, 32, 64])
def test_multi_rhs_matches_single(gb, oracle_mod, nv):
    O = oracle_mod
    I, J, V = O.stencil(27, 14, 14, 14)
    n = len(I) - 1
    B = np.stack([O.rand_uniform(n, 22775 + c) for c in range(nv)], 1)
    A = gb.IJMatrix(I, J, V)
    amg = gb.BoomerAMG(MaxRowSum=1.0, StrongThreshold=0.5, Tol=0.0, MaxIter=1)
    k = gb.Krylov("pcg", tol=1e-8, maxit=100, amg=amg)
    b1, x1 = gb.IJVector(n, B[:, 0]), gb.IJVector(n, np.zeros(n))
    k.setup(A, b1, x1)
    Bm, Xm = gb.MultiVector(B), gb.MultiVector(np.zeros((n, nv)))
    assert gb.lib().HYPRE_ParCSRPCGSolve(k.h, A.par, Bm.par, Xm.par) == 0
    its, rel, hist = gb.multi_results(k, nv, 100)
    X = Xm.values()
    for c in sorted({0, nv // 2, nv - 1}):
        b1.set(B[:, c])
        x1.set(np.zeros(n))
        k.solve(A, b1, x1)
        assert its[c] == k.iterations(), c
        np.testing.assert_allclose(hist[c], k.history(), rtol=1e-10, atol=0)
        np.testing.assert_allclose(X[:, c], x1.values(), rtol=0, atol=1e-9 * np.abs(x1.values()).max())
    R = B - _csr(I, J, V) @ X
    assert np.all(np.linalg.norm(R, axis=0) < 1e-8 * np.linalg.norm(B, axis=0))


def test_multi_rhs_fp32_cycle(gb, oracle_mod):
    O = oracle_mod
    I, J, V = O.stencil(27, 18, 18, 18)
    n, nv = len(I) - 1, 64
    B = np.stack([O.rand_uniform(n, 100 + c) for c in range(nv)], 1)
    A = gb.IJMatrix(I, J, V)
    amg = gb.BoomerAMG(MaxRowSum=1.0, StrongThreshold=0.5, AggNumLevels=1, AggInterpType=6, Tol=0.0, MaxIter=1)
    amg.set("CyclePrecision", 1)
    k = gb.Krylov("pcg", tol=1e-8, maxit=100, amg=amg)
    b1, x1 = gb.IJVector(n, B[:, 0]), gb.IJVector(n, np.zeros(n))
    k.setup(A, b1, x1)
    Bm, Xm = gb.MultiVector(B), gb.MultiVector(np.zeros((n, nv)))
    assert gb.lib().HYPRE_ParCSRPCGSolve(k.h, A.par, Bm.par, Xm.par) == 0
    R = B - _csr(I, J, V) @ Xm.values()
    assert np.all(np.linalg.norm(R, axis=0) < 1e-8 * np.linalg.norm(B, axis=0))
