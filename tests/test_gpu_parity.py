"""GPU parity tests: the CUDA path (through the C ABI) against the CPU oracle.

Integer results (strength pattern, C/F splitting, interpolation and coarse
operator sparsity and column order) and the FP64 hierarchy values are
compared bit for bit; residual histories of the FP64 Krylov solves to 1e-10
relative with the iteration count equal."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL_HIST = 1e-10


def _setup_both(gb, O, I, J, V, **prm):
    oprm = dict(max_row_sum=prm.get("MaxRowSum", 0.9), max_coarse_size=prm.get("MaxCoarseSize", 9),
                strong_threshold=prm.get("StrongThreshold", 0.25), p_max_elmts=prm.get("PMaxElmts", 4),
                trunc_factor=prm.get("TruncFactor", 0.0), agg_num_levels=prm.get("AggNumLevels", 0),
                agg_interp_type=prm.get("AggInterpType", 4))
    if "RelaxType" in prm:
        oprm.update(relax_down=prm["RelaxType"], relax_up=prm["RelaxType"])
    H = O.Hierarchy(I, J, V, O.default_params(**oprm))
    A = gb.IJMatrix(I, J, V)
    n = len(I) - 1
    bv = gb.IJVector(n, np.zeros(n))
    xv = gb.IJVector(n, np.zeros(n))
    amg = gb.BoomerAMG(Tol=0.0, MaxIter=1, **prm)
    gb.check(gb.lib().HYPRE_BoomerAMGSetup(amg.h, A.par, bv.par, xv.par), "setup")
    return H, A, amg, bv, xv


def _compare_hierarchy(H, amg):
    assert amg.num_levels() == H.num_levels
    for l in range(H.num_levels):
        Ig, Jg, Vg, _ = amg.level_csr(l, "A")
        Io, Jo, Vo, _ = H.csr("A", l)
        assert np.array_equal(Ig, Io), f"A{l} row pointers"
        assert np.array_equal(Jg, Jo), f"A{l} columns (pattern and order)"
        assert np.array_equal(Vg, Vo), f"A{l} values"
        n = len(Io) - 1
        assert np.array_equal(amg.level_l1(l, n), H.l1(l)), f"l1 norms level {l}"
        if l < H.num_levels - 1:
            Sg = amg.level_csr(l, "S")
            So = H.csr("S", l)
            assert np.array_equal(Sg[0], So[0]) and np.array_equal(Sg[1], So[1]), f"S{l}"
            assert np.array_equal(amg.level_cf(l, n), H.cf(l)), f"CF{l}"
            Pg = amg.level_csr(l, "P")
            Po = H.csr("P", l)
            assert np.array_equal(Pg[0], Po[0]) and np.array_equal(Pg[1], Po[1]), f"P{l} pattern"
            assert np.array_equal(Pg[2], Po[2]), f"P{l} values"


@pytest.mark.parametrize("kind,nx,th,mcs", [(7, 12, 0.25, 9), (7, 30, 0.25, 100), (27, 10, 0.25, 9),
                                            (27, 16, 0.5, 20), (7, 5, 0.25, 9)])
def test_hierarchy_bitexact(gb, oracle_mod, kind, nx, th, mcs):
    O = oracle_mod
    I, J, V = O.stencil(kind, nx, nx, nx)
    H, A, amg, bv, xv = _setup_both(gb, O, I, J, V, MaxRowSum=1.0, StrongThreshold=th, MaxCoarseSize=mcs)
    _compare_hierarchy(H, amg)


@pytest.mark.parametrize("kind,nx,th,agg", [(27, 20, 0.5, 1), (7, 24, 0.25, 1), (7, 30, 0.25, 2), (27, 12, 0.5, 1)])
def test_hierarchy_aggressive_bitexact(gb, oracle_mod, kind, nx, th, agg):
    """Aggressive coarsening (second-order strength, PMIS on it, modified and
    partial extended+i, P1 P2) on the first levels."""
    O = oracle_mod
    I, J, V = O.stencil(kind, nx, nx, nx)
    H, A, amg, bv, xv = _setup_both(gb, O, I, J, V, MaxRowSum=1.0, StrongThreshold=th, AggNumLevels=agg,
                                    AggInterpType=6)
    _compare_hierarchy(H, amg)


@pytest.mark.parametrize("kind,nx,th,agg", [(27, 20, 0.5, 1), (7, 24, 0.25, 1), (7, 12, 0.25, 0)])
def test_hierarchy_global_tables_bitexact(gb, oracle_mod, kind, nx, th, agg):
    """Every row of the ordered setup kernels (sparse products, second-order
    strength, extended+i) in global-memory tables -- the tier that rows too
    long for shared memory take -- gives the same hierarchy."""
    O = oracle_mod
    I, J, V = O.stencil(kind, nx, nx, nx)
    H, A, amg, bv, xv = _setup_both(gb, O, I, J, V, MaxRowSum=1.0, StrongThreshold=th, AggNumLevels=agg,
                                    AggInterpType=6, SetupTables=1)
    _compare_hierarchy(H, amg)


def test_aggressive_fgmres_two_stage_gs(gb, oracle_mod):
    """Miniature of the 160^3 configuration: aggressive first level, PMIS 0.5,
    two-stage Gauss-Seidel, FlexGMRES(30)."""
    O = oracle_mod
    I, J, V = O.stencil(27, 24, 24, 24)
    n = len(I) - 1
    b = O.rhs_normalised(n)
    prm = O.default_params(max_row_sum=1.0, strong_threshold=0.5, agg_num_levels=1, agg_interp_type=6,
                           relax_down=11, relax_up=11)
    H = O.Hierarchy(I, J, V, prm)
    _, res_o, it_o = H.fgmres(b, tol=1e-8, maxit=100, kdim=30)
    A = gb.IJMatrix(I, J, V)
    bv, xv = gb.IJVector(n, b), gb.IJVector(n, np.zeros(n))
    amg = gb.BoomerAMG(MaxRowSum=1.0, StrongThreshold=0.5, AggNumLevels=1, AggInterpType=6, RelaxType=11,
                       Tol=0.0, MaxIter=1)
    k = gb.Krylov("fgmres", tol=1e-8, maxit=100, kdim=30, amg=amg)
    k.setup(A, bv, xv)
    k.solve(A, bv, xv)
    assert k.iterations() == it_o
    m = min(len(res_o), len(k.history()))
    np.testing.assert_allclose(k.history()[:m], res_o[:m] / np.linalg.norm(b), rtol=1e-10, atol=0)


def test_hierarchy_fv_diffusion(gb, oracle_mod):
    """Jumping coefficients: non-uniform values exercise ties and truncation."""
    O = oracle_mod
    from hypre_gb300 import problems as G
    I, J, V = G.fv_diffusion(14, seed=3, sigma=2.0, block=4)
    H, A, amg, bv, xv = _setup_both(gb, O, I, J, V, MaxRowSum=0.9, StrongThreshold=0.25)
    _compare_hierarchy(H, amg)


def test_hierarchy_aniso2d(gb, oracle_mod):
    O = oracle_mod
    from hypre_gb300 import problems as G
    I, J, V = G.aniso2d(40, 1e-2)
    H, A, amg, bv, xv = _setup_both(gb, O, I, J, V, MaxRowSum=1.0, StrongThreshold=0.25, TruncFactor=0.1)
    _compare_hierarchy(H, amg)


@pytest.mark.parametrize("kind,nx,th", [(7, 20, 0.25), (27, 14, 0.5)])
def test_pcg_history(gb, oracle_mod, kind, nx, th):
    O = oracle_mod
    I, J, V = O.stencil(kind, nx, nx, nx)
    n = len(I) - 1
    b = O.rhs_normalised(n)
    H = O.Hierarchy(I, J, V, O.default_params(max_row_sum=1.0, strong_threshold=th, max_coarse_size=50))
    _, rel_o, it_o = H.pcg(b, tol=1e-8, maxit=100)
    A = gb.IJMatrix(I, J, V)
    bv, xv = gb.IJVector(n, b), gb.IJVector(n, np.zeros(n))
    amg = gb.BoomerAMG(MaxRowSum=1.0, StrongThreshold=th, MaxCoarseSize=50, Tol=0.0, MaxIter=1)
    k = gb.Krylov("pcg", tol=1e-8, maxit=100, amg=amg)
    k.setup(A, bv, xv)
    k.solve(A, bv, xv)
    assert k.iterations() == it_o
    np.testing.assert_allclose(k.history(), rel_o, rtol=RTOL_HIST, atol=0)
    # true residual of the returned solution
    x = xv.values()
    r = b - O_matvec(I, J, V, x)
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1e-8


def O_matvec(I, J, V, x):
    import scipy.sparse as sp
    n = len(I) - 1
    return sp.csr_matrix((V, J, I), shape=(n, n)) @ x


def test_fgmres_history(gb, oracle_mod):
    O = oracle_mod
    I, J, V = O.stencil(7, 18, 18, 18)
    n = len(I) - 1
    b = O.rhs_normalised(n)
    H = O.Hierarchy(I, J, V, O.default_params(max_row_sum=1.0, max_coarse_size=40))
    _, res_o, it_o = H.fgmres(b, tol=1e-8, maxit=100, kdim=30)
    A = gb.IJMatrix(I, J, V)
    bv, xv = gb.IJVector(n, b), gb.IJVector(n, np.zeros(n))
    amg = gb.BoomerAMG(MaxRowSum=1.0, MaxCoarseSize=40, Tol=0.0, MaxIter=1)
    k = gb.Krylov("fgmres", tol=1e-8, maxit=100, kdim=30, amg=amg)
    k.setup(A, bv, xv)
    k.solve(A, bv, xv)
    assert k.iterations() == it_o
    m = min(len(res_o), len(k.history()))
    np.testing.assert_allclose(k.history()[:m], res_o[:m] / np.linalg.norm(b), rtol=RTOL_HIST, atol=0)


@pytest.mark.parametrize("prec", [1, 2])
def test_mixed_precision_cycle_converges(gb, oracle_mod, prec):
    """FP32 (or FP16-finest) V-cycle inside FP64 PCG: the FP64 true residual
    reaches 1e-8 within a few more iterations than the FP64 cycle."""
    O = oracle_mod
    I, J, V = O.stencil(27, 16, 16, 16)
    n = len(I) - 1
    b = O.rhs_normalised(n)
    A = gb.IJMatrix(I, J, V)
    bv, xv = gb.IJVector(n, b), gb.IJVector(n, np.zeros(n))
    amg = gb.BoomerAMG(MaxRowSum=1.0, StrongThreshold=0.5, Tol=0.0, MaxIter=1)
    amg.set("CyclePrecision", prec)
    k = gb.Krylov("pcg", tol=1e-8, maxit=100, amg=amg)
    k.setup(A, bv, xv)
    k.solve(A, bv, xv)
    x = xv.values()
    r = b - O_matvec(I, J, V, x)
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1.2e-8
    assert k.iterations() < 40


def test_two_stage_gs_fgmres(gb, oracle_mod):
    O = oracle_mod
    I, J, V = O.stencil(27, 12, 12, 12)
    n = len(I) - 1
    b = O.rhs_normalised(n)
    prm = O.default_params(max_row_sum=1.0, strong_threshold=0.5, relax_down=11, relax_up=11)
    H = O.Hierarchy(I, J, V, prm)
    _, res_o, it_o = H.fgmres(b, tol=1e-8, maxit=100, kdim=30)
    A = gb.IJMatrix(I, J, V)
    bv, xv = gb.IJVector(n, b), gb.IJVector(n, np.zeros(n))
    amg = gb.BoomerAMG(MaxRowSum=1.0, StrongThreshold=0.5, RelaxType=11, Tol=0.0, MaxIter=1)
    k = gb.Krylov("fgmres", tol=1e-8, maxit=100, kdim=30, amg=amg)
    k.setup(A, bv, xv)
    k.solve(A, bv, xv)
    assert k.iterations() == it_o
    m = min(len(res_o), len(k.history()))
    np.testing.assert_allclose(k.history()[:m], res_o[:m] / np.linalg.norm(b), rtol=1e-10, atol=0)


def test_matvec_and_vector_ops(gb, oracle_mod):
    O = oracle_mod
    import ctypes as C
    I, J, V = O.stencil(27, 9, 10, 11)
    n = len(I) - 1
    rng = np.random.default_rng(5)
    x = rng.standard_normal(n)
    y = rng.standard_normal(n)
    A = gb.IJMatrix(I, J, V)
    xv, yv = gb.IJVector(n, x), gb.IJVector(n, y)
    L = gb.lib()
    gb.check(L.HYPRE_ParCSRMatrixMatvec(2.0, A.par, xv.par, -0.5, yv.par))
    ref = 2.0 * O_matvec(I, J, V, x) - 0.5 * y
    np.testing.assert_allclose(yv.values(), ref, rtol=1e-13, atol=1e-13)
    d = C.c_double()
    L.HYPRE_ParVectorInnerProd(xv.par, xv.par, C.byref(d))
    assert abs(d.value - x @ x) < 1e-10 * (x @ x)
    gb.check(L.HYPRE_ParCSRMatrixMatvecT(1.0, A.par, xv.par, 0.0, yv.par))
    np.testing.assert_allclose(yv.values(), O_matvec(I, J, V, x), rtol=1e-13, atol=1e-13)


def test_error_flags(gb):
    import ctypes as C
    L = gb.lib()
    L.HYPRE_ClearAllErrors()
    h = C.c_void_p()
    # bad range -> argument error, nothing created
    err = L.HYPRE_IJMatrixCreate(0, 5, 2, 0, 3, C.byref(h))
    assert err & gb.HYPRE_ERROR_ARG
    L.HYPRE_ClearAllErrors()
    assert L.HYPRE_BoomerAMGSetup(None, None, None, None) & gb.HYPRE_ERROR_ARG
    L.HYPRE_ClearAllErrors()



def test_unsupported_options_are_refused(gb, oracle_mod):
    """Option values without a bit-exact implementation return
    HYPRE_ERROR_GENERIC instead of silently running something else; the
    supported ones (including BAMG-direct 15, which the reference's host path
    builds as the direct interpolation) are accepted."""
    import ctypes as C
    L = gb.lib()
    amg = gb.BoomerAMG()
    for v in (0, 1, 2, 4, 5, 8):
        L.HYPRE_ClearAllErrors()
        assert amg.set("InterpType", v) & gb.HYPRE_ERROR_GENERIC, v
    for v in (3, 6, 14, 15, 16, 17, 18):
        L.HYPRE_ClearAllErrors()
        assert amg.set("InterpType", v) == 0, v
    for name, bad, good in (("NumPaths", 2, 1), ("CycleType", 3, 2), ("RelaxOrder", 2, 1), ("RAP2", 1, 0),
                            ("ModuleRAP2", 1, 0)):
        L.HYPRE_ClearAllErrors()
        assert amg.set(name, bad) & gb.HYPRE_ERROR_GENERIC, name
        L.HYPRE_ClearAllErrors()
        assert amg.set(name, good) == 0, name
    L.HYPRE_ClearAllErrors()
    amg.destroy()
    # aggressive interpolation types are checked at setup: the two-stage
    # standard one (2) is refused
    I, J, V = oracle_mod.stencil(7, 8, 8, 8)
    n = len(I) - 1
    A = gb.IJMatrix(I, J, V)
    b, x = gb.IJVector(n, np.ones(n)), gb.IJVector(n, np.zeros(n))
    for at, ok in ((2, False), (3, True), (8, True)):
        amg = gb.BoomerAMG(MaxRowSum=1.0, StrongThreshold=0.25, AggNumLevels=1, AggInterpType=at, Tol=0.0,
                           MaxIter=1)
        L.HYPRE_ClearAllErrors()
        err = L.HYPRE_BoomerAMGSetup(amg.h, A.par, b.par, x.par)
        assert bool(err & gb.HYPRE_ERROR_GENERIC) != ok, at
        L.HYPRE_ClearAllErrors()
        amg.destroy()
    A.destroy(); b.destroy(); x.destroy()


def test_getters_and_min_iter(gb, oracle_mod):
    """The BoomerAMG getters return what the setters stored, single-value
    settings refuse other values, and MinIter makes the stand-alone solve run
    at least that many cycles (par_amg_solve.c: cycle while the residual is
    above tol or fewer than min_iter cycles ran)."""
    import ctypes as C
    L = gb.lib()
    L.HYPRE_ClearAllErrors()
    amg = gb.BoomerAMG(StrongThreshold=0.3, MaxIter=20, Tol=0.5, PMaxElmts=3, MaxLevels=7)
    i, d = C.c_int(), C.c_double()
    for name, want in (("MaxIter", 20), ("PMaxElmts", 3), ("MaxLevels", 7), ("CycleType", 1)):
        gb.check(getattr(L, "HYPRE_BoomerAMGGet" + name)(amg.h, C.byref(i)))
        assert i.value == want, name
    for name, want in (("Tol", 0.5), ("StrongThreshold", 0.3)):
        gb.check(getattr(L, "HYPRE_BoomerAMGGet" + name)(amg.h, C.byref(d)))
        assert d.value == want, name
    gb.check(L.HYPRE_BoomerAMGGetCycleRelaxType(amg.h, C.byref(i), 1))
    assert i.value == 18
    for name, bad, good in (("NumFunctions", 2, 1), ("Nodal", 1, 0), ("MeasureType", 1, 0)):
        L.HYPRE_ClearAllErrors()
        assert getattr(L, "HYPRE_BoomerAMGSet" + name)(amg.h, bad) & gb.HYPRE_ERROR_GENERIC, name
        L.HYPRE_ClearAllErrors()
        assert getattr(L, "HYPRE_BoomerAMGSet" + name)(amg.h, good) == 0, name
    I, J, V = oracle_mod.stencil(7, 8, 8, 8)
    n = len(I) - 1
    A = gb.IJMatrix(I, J, V)
    b, x = gb.IJVector(n, np.ones(n)), gb.IJVector(n, np.zeros(n))
    gb.check(L.HYPRE_BoomerAMGSetMinIter(amg.h, 5))
    gb.check(L.HYPRE_BoomerAMGSetup(amg.h, A.par, b.par, x.par))
    gb.check(L.HYPRE_BoomerAMGSolve(amg.h, A.par, b.par, x.par))
    gb.check(L.HYPRE_BoomerAMGGetNumIterations(amg.h, C.byref(i)))
    assert i.value == 5
    amg.destroy(); A.destroy(); b.destroy(); x.destroy()
