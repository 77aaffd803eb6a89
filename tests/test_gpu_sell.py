"""SELL-32 forms on levels large enough to use them (>= 4096 rows for the
SpMV, >= 65,536 rows for the lower-part form of two-stage Gauss-Seidel), in
both index encodings: 16-bit offsets from the row when every |j - i| < 2^15,
int32 indices otherwise (here forced by one long-range coupling)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _with_far_pair(I, J, V, a, b, w=0.05):
    """A symmetric coupling -w between rows a and b (w added to both
    diagonals, so the matrix stays an M-matrix)."""
    import scipy.sparse as sp
    n = len(I) - 1
    A = sp.csr_matrix((V, J, I), shape=(n, n)).tolil()
    A[a, b] = -w
    A[b, a] = -w
    A[a, a] += w
    A[b, b] += w
    A = A.tocsr()
    A.sort_indices()
    I2, J2, V2 = A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data.astype(np.float64)
    # rows as the stencil generators write them: diagonal first, then ascending
    for r in range(n):
        s, e = I2[r], I2[r + 1]
        p = s + int(np.nonzero(J2[s:e] == r)[0][0])
        if p > s:
            J2[s + 1:p + 1], V2[s + 1:p + 1] = J2[s:p].copy(), V2[s:p].copy()
            J2[s], V2[s] = r, A[r, r]
    return I2, J2, V2


def _csr_matvec(I, J, V, x):
    import scipy.sparse as sp
    n = len(I) - 1
    return sp.csr_matrix((V, J, I), shape=(n, n)) @ x


def _case(O, name):
    if name == "offsets16":
        return O.stencil(27, 20, 20, 20)
    if name == "ragged":
        return O.stencil(7, 17, 19, 23)       # 7429 rows: the last slice is partly padding
    I, J, V = O.stencil(7, 41, 41, 41)
    n = len(I) - 1
    return _with_far_pair(I, J, V, 3, n - 4)  # |j - i| > 2^15: int32 indices


@pytest.mark.parametrize("name", ["offsets16", "ragged", "int32"])
def test_sell_matvec(gb, oracle_mod, name):
    I, J, V = _case(oracle_mod, name)
    n = len(I) - 1
    assert n >= 4096
    rng = np.random.default_rng(11)
    x = rng.standard_normal(n)
    y = rng.standard_normal(n)
    A = gb.IJMatrix(I, J, V)
    xv, yv = gb.IJVector(n, x), gb.IJVector(n, y)
    gb.check(gb.lib().HYPRE_ParCSRMatrixMatvec(2.0, A.par, xv.par, -0.5, yv.par))
    ref = 2.0 * _csr_matvec(I, J, V, x) - 0.5 * y
    np.testing.assert_allclose(yv.values(), ref, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("far", [False, True])
def test_two_stage_gs_on_a_large_level(gb, oracle_mod, far):
    """FlexGMRES with two-stage Gauss-Seidel on a 74,088-row finest level
    (lower-part SELL form): residual history against the oracle."""
    O = oracle_mod
    I, J, V = O.stencil(7, 42, 42, 42)
    n = len(I) - 1
    if far:
        I, J, V = _with_far_pair(I, J, V, 3, n - 4)
    b = O.rhs_normalised(n)
    prm = O.default_params(max_row_sum=1.0, strong_threshold=0.25, relax_down=11, relax_up=11)
    H = O.Hierarchy(I, J, V, prm)
    _, res_o, it_o = H.fgmres(b, tol=1e-8, maxit=100, kdim=30)
    A = gb.IJMatrix(I, J, V)
    bv, xv = gb.IJVector(n, b), gb.IJVector(n, np.zeros(n))
    amg = gb.BoomerAMG(MaxRowSum=1.0, StrongThreshold=0.25, RelaxType=11, Tol=0.0, MaxIter=1)
    k = gb.Krylov("fgmres", tol=1e-8, maxit=100, kdim=30, amg=amg)
    k.setup(A, bv, xv)
    k.solve(A, bv, xv)
    assert k.iterations() == it_o
    m = min(len(res_o), len(k.history()))
    np.testing.assert_allclose(k.history()[:m], res_o[:m] / np.linalg.norm(b), rtol=1e-10, atol=0)
