"""GPU parity of the polynomial smoother (relax type 16, Chebyshev) against the
CPU oracle: the D^{-1/2} scaling bit for bit, the CG-Lanczos eigenvalue
estimates and polynomial coefficients to 1e-12 relative (the GPU inner
products sum in a different order), and the FP64 PCG residual history to
1e-10 relative with the same iteration count."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL_VAL = 1e-12
RTOL_HIST = 1e-10


def _matvec(I, J, V, x):
    import scipy.sparse as sp
    n = len(I) - 1
    return sp.csr_matrix((V, J, I), shape=(n, n)) @ x


@pytest.mark.parametrize("order,scale,variant", [(1, 1, 0), (2, 1, 0), (3, 1, 0), (4, 1, 0), (2, 0, 0),
                                                 (3, 1, 1), (4, 0, 1)])
def test_chebyshev_setup(gb, oracle_mod, order, scale, variant):
    O = oracle_mod
    I, J, V = O.stencil(7, 14, 14, 14)
    prm = O.default_params(max_row_sum=1.0, relax_down=16, relax_up=16, cheby_order=order, cheby_scale=scale,
                           cheby_variant=variant)
    H = O.Hierarchy(I, J, V, prm)
    A = gb.IJMatrix(I, J, V)
    n = len(I) - 1
    bv, xv = gb.IJVector(n, np.zeros(n)), gb.IJVector(n, np.zeros(n))
    amg = gb.BoomerAMG(MaxRowSum=1.0, RelaxType=16, ChebyOrder=order, ChebyScale=scale, ChebyVariant=variant,
                       Tol=0.0, MaxIter=1)
    gb.check(gb.lib().HYPRE_BoomerAMGSetup(amg.h, A.par, bv.par, xv.par), "setup")
    assert amg.num_levels() == H.num_levels
    for l in range(H.num_levels):
        nl = len(H.csr("A", l)[0]) - 1
        co, eo, dso = H.cheby(l, order)
        cg, eg, dsg = amg.level_cheby(l, nl, order)
        assert np.array_equal(dsg, dso), f"D^-1/2 level {l}"
        np.testing.assert_allclose(eg, eo, rtol=RTOL_VAL, atol=0, err_msg=f"eigenvalue estimates level {l}")
        np.testing.assert_allclose(cg, co, rtol=1e-11, atol=0, err_msg=f"coefficients level {l}")


@pytest.mark.parametrize("kind,nx,th,order", [(7, 20, 0.25, 2), (27, 14, 0.5, 3)])
def test_chebyshev_pcg_history(gb, oracle_mod, kind, nx, th, order):
    O = oracle_mod
    I, J, V = O.stencil(kind, nx, nx, nx)
    n = len(I) - 1
    b = O.rhs_normalised(n)
    H = O.Hierarchy(I, J, V, O.default_params(max_row_sum=1.0, strong_threshold=th, relax_down=16, relax_up=16,
                                              cheby_order=order))
    _, rel_o, it_o = H.pcg(b, tol=1e-8, maxit=100)
    A = gb.IJMatrix(I, J, V)
    bv, xv = gb.IJVector(n, b), gb.IJVector(n, np.zeros(n))
    amg = gb.BoomerAMG(MaxRowSum=1.0, StrongThreshold=th, RelaxType=16, ChebyOrder=order, Tol=0.0, MaxIter=1)
    k = gb.Krylov("pcg", tol=1e-8, maxit=100, amg=amg)
    k.setup(A, bv, xv)
    k.solve(A, bv, xv)
    assert k.iterations() == it_o
    np.testing.assert_allclose(k.history(), rel_o, rtol=RTOL_HIST, atol=0)
    r = b - _matvec(I, J, V, xv.values())
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1e-8


@pytest.mark.parametrize("prec", [1, 2])
def test_chebyshev_mixed_precision(gb, oracle_mod, prec):
    """FP32 (FP16-finest) Chebyshev V-cycle inside FP64 PCG reaches the FP64
    true residual 1e-8 within a few iterations of the FP64 cycle."""
    O = oracle_mod
    I, J, V = O.stencil(27, 16, 16, 16)
    n = len(I) - 1
    b = O.rhs_normalised(n)
    H = O.Hierarchy(I, J, V, O.default_params(max_row_sum=1.0, strong_threshold=0.5, relax_down=16, relax_up=16))
    _, _, it_o = H.pcg(b, tol=1e-8, maxit=100)
    A = gb.IJMatrix(I, J, V)
    bv, xv = gb.IJVector(n, b), gb.IJVector(n, np.zeros(n))
    amg = gb.BoomerAMG(MaxRowSum=1.0, StrongThreshold=0.5, RelaxType=16, Tol=0.0, MaxIter=1)
    amg.set("CyclePrecision", prec)
    k = gb.Krylov("pcg", tol=1e-8, maxit=100, amg=amg)
    k.setup(A, bv, xv)
    k.solve(A, bv, xv)
    r = b - _matvec(I, J, V, xv.values())
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1.2e-8
    assert k.iterations() <= it_o + 3
