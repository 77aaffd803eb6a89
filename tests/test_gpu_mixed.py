"""Mixed-precision V-cycles on a problem with coefficients far outside FP16's
range: finite-volume diffusion with log-normal coefficients and 8^3 blocks
scaled by 10^+-4.  The FP32 cycle and the FP16-finest cycle (row-scaled FP16
values, FP32 row scales) inside FP64 FlexGMRES(30) reach the FP64 true
relative residual 1e-8."""
import numpy as np
import pytest

from hypre_gb300 import problems as G

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_fv_diffusion_mixed_precision(gb, prec):
    import scipy.sparse as sp
    I, J, V = G.fv_diffusion(32, seed=3)
    n = len(I) - 1
    b = G.rhs(n)
    A = gb.IJMatrix(I, J, V)
    amg = gb.BoomerAMG(StrongThreshold=0.25, RelaxType=18, Tol=0.0, MaxIter=1)
    amg.set("CyclePrecision", prec)
    k = gb.Krylov("fgmres", tol=1e-8, maxit=200, kdim=30, amg=amg)
    bv, xv = gb.IJVector(n, b), gb.IJVector(n, np.zeros(n))
    k.setup(A, bv, xv)
    k.solve(A, bv, xv)
    r = b - sp.csr_matrix((V, J, I), shape=(n, n)) @ xv.values()
    rel = np.linalg.norm(r) / np.linalg.norm(b)
    assert np.isfinite(rel) and rel < 1.2e-8, rel
    assert k.iterations() < 120
