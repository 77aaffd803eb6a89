"""The CUDA path against the reference library's own output: each golden
fixture (the reference's serial BoomerAMG compiled from its sources, dumped by
tests/golden/make_golden.py) is set up and solved through the C ABI on the GPU.
Hierarchy integers and FP64 values must be identical; Chebyshev eigenvalue
estimates and coefficients agree to 1e-12 relative (GPU inner products sum
in another order); PCG and FlexGMRES residual histories to 1e-10 with the
same iteration count (values at the rounding level, below 1e-14, to 1e-14);
BoomerAMG as the solver: the same number of cycles and the final relative
residual to 1e-14."""
import ctypes as C

import numpy as np
import pytest

import golden_cases as G

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", G.case_names())
def test_gpu_matches_reference(gb, oracle_mod, name):
    g = G.load(name)
    c = g["case"]
    I, J, V = G.matrix(c, oracle_mod, g)
    n = len(I) - 1
    b = oracle_mod.rhs_normalised(n)
    G.check_array(g, "b", b)
    A = gb.IJMatrix(I, J, V)
    bv, xv = gb.IJVector(n, b), gb.IJVector(n, np.zeros(n))
    kind = {1: "pcg", 0: "amg"}.get(c["solver"], "fgmres")
    if kind == "amg":
        # BoomerAMG as the solver: V-cycles in place on (b, x) to rel-res 1e-8
        amg = gb.BoomerAMG(Tol=1e-8, MaxIter=100, **G.amg_params(c))
        gb.check(gb.lib().HYPRE_BoomerAMGSetup(amg.h, A.par, bv.par, xv.par), "setup")
    else:
        amg = gb.BoomerAMG(Tol=0.0, MaxIter=1, **G.amg_params(c))
        k = gb.Krylov(kind, tol=1e-8, maxit=100, kdim=c.get("k", 30), amg=amg, rel_change=c.get("rel_change", 0))
        k.setup(A, bv, xv)
    nl = amg.num_levels()

    def rows(l):
        return int(g["lev_rows"][l])

    G.check_hierarchy(g, nl, lambda w, l: amg.level_csr(l, w)[:3], lambda l: amg.level_cf(l, rows(l)),
                      lambda l: amg.level_l1(l, rows(l)),
                      cheby=lambda l, o: amg.level_cheby(l, rows(l), o), value_rtol=0.0, cheby_rtol=1e-12)
    it_ref = int(g["iters"][0])
    if kind == "amg":
        gb.check(gb.lib().HYPRE_BoomerAMGSolve(amg.h, A.par, bv.par, xv.par), "solve")
        it = C.c_int(); rel = C.c_double()
        gb.lib().HYPRE_BoomerAMGGetNumIterations(amg.h, C.byref(it))
        gb.lib().HYPRE_BoomerAMGGetFinalRelativeResidualNorm(amg.h, C.byref(rel))
        assert it.value == it_ref
        # the residual after many in-place cycles carries the rounding of x
        # (the GPU's sums differ from the reference's in the last bits):
        # equal to 1e-14 of ||b||
        np.testing.assert_allclose(rel.value, float(g["final_relres"][0]), rtol=0, atol=1e-14)
    else:
        k.solve(A, bv, xv)
    if kind == "amg":
        pass
    elif kind == "pcg":
        assert k.iterations() == it_ref
        # residuals at the rounding level (a solve that ends exactly) only to 1e-14
        np.testing.assert_allclose(k.history()[1:], g["relres"][1:], rtol=1e-10, atol=1e-14)
    else:
        assert k.iterations() == it_ref
        ref = g["resnorms"] / g["resnorms"][0]    # absolute norms in the reference; x0 = 0, so r0 = b
        np.testing.assert_allclose(k.history(), ref, rtol=1e-10, atol=1e-14)
    x = xv.values()
    if "x" in g:
        assert np.linalg.norm(x - g["x"]) <= 1e-7 * np.linalg.norm(g["x"])
    else:
        idx = g["sample_idx:x"]
        np.testing.assert_allclose(x[idx], g["sample:x"], rtol=1e-6, atol=1e-9 * np.abs(g["sample:x"]).max())
