"""Pins the CPU oracle to the reference library: every golden fixture (written
from the reference's own serial BoomerAMG compiled from its sources) is
reproduced bit for bit by the oracle run single-threaded -- hierarchy
integers and values, residual histories, iteration counts, solutions -- and
the oracle reproduces the complexities the reference's own regression suite
saves (src/test/TEST_ij/default.saved).  CPU only."""
import numpy as np
import pytest

import golden_cases as G


@pytest.fixture(scope="module")
def O(oracle_mod):
    oracle_mod.set_threads(1)
    return oracle_mod


@pytest.mark.parametrize("name", G.case_names())
def test_oracle_matches_reference(O, name):
    g = G.load(name)
    c = g["case"]
    I, J, V = G.matrix(c, O, g)
    H = O.Hierarchy(I, J, V, O.default_params(**G.oracle_params(c)))
    G.check_hierarchy(g, H.num_levels, lambda w, l: H.csr(w, l)[:3], H.cf, H.l1,
                      cheby=lambda l, o: H.cheby(l, o), value_rtol=0.0, cheby_rtol=0.0)
    n = len(I) - 1
    b = O.rhs_normalised(n)
    G.check_array(g, "b", b)
    if c["solver"] == 1:
        x, rel, it = H.pcg(b, tol=1e-8, maxit=100)
        assert it == int(g["iters"][0])
        np.testing.assert_array_equal(rel[1:], g["relres"][1:])
    elif c["solver"] == 0:
        x, rel, it = H.amg_solve(b, tol=1e-8, maxit=100)
        assert it == int(g["iters"][0])
        assert rel[-1] == float(g["final_relres"][0])
    else:
        x, res, it = H.fgmres(b, tol=1e-8, maxit=100, kdim=c.get("k", 30))
        assert it == int(g["iters"][0])
        ref = g["resnorms"] / g["resnorms"][0]   # the reference keeps absolute norms (x0 = 0: r0 = b)
        np.testing.assert_allclose(res, ref, rtol=1e-14, atol=0)
    G.check_array(g, "x", x)


@pytest.mark.parametrize("name", G.matmat_names())
def test_oracle_matmat_matches_reference(O, name):
    """C = A*A of the reference's HYPRE_ParCSRMatrixMatmat (column order, sums,
    diagonal-first rule with and without empty rows) reproduced bit for bit."""
    g = G.load(name)
    A = (g["A0_i"], g["A0_j"], g["A0_v"])
    n = len(g["A0_i"]) - 1
    Ci, Cj, Cv = O.matmat(A, A, n, n)
    assert np.array_equal(Ci, g["C0_i"]) and np.array_equal(Cj, g["C0_j"])
    assert np.array_equal(Cv, g["C0_v"])


def test_golden_fixtures_present():
    names = G.case_names()
    assert len(names) >= 8
    for n in names:
        g = G.load(n)
        # every case but the one without strong couplings has a coarse level
        assert int(g["iters"][0]) > 0 and (int(g["nlev"][0]) >= 2 or g["case"].get("gen") == "diag")


def test_reference_suite_complexities(O):
    """src/test/TEST_ij/default.jobs:11 (ij -pmis1 -Pmx 0, one process: the 10^3
    7-point Laplacian, PMIS, theta 0.25, extended+i without truncation) saves
    grid complexity 1.407000 and operator complexity 3.252344
    (src/test/TEST_ij/default.saved:4-5).  With one process PMIS with the
    sequential random numbers (-pmis1) draws the same measures as -pmis."""
    I, J, V = O.stencil(7, 10, 10, 10)
    H = O.Hierarchy(I, J, V, O.default_params(max_row_sum=1.0, strong_threshold=0.25, p_max_elmts=0))
    rows = [len(H.csr("A", l)[0]) - 1 for l in range(H.num_levels)]
    nnz = [len(H.csr("A", l)[1]) for l in range(H.num_levels)]
    assert "%.6f" % (sum(rows) / rows[0]) == "1.407000"
    assert "%.6f" % (sum(nnz) / nnz[0]) == "3.252344"


def test_tridiagonal_eigenvalues(O):
    """The QL eigenvalue routine the Chebyshev setup uses, against numpy."""
    rng = np.random.default_rng(3)
    for n in (1, 2, 5, 10):
        d = rng.uniform(1, 3, n)
        e = np.concatenate([[0.0], rng.uniform(-1, 1, n - 1)])
        T = np.diag(d) + np.diag(e[1:], 1) + np.diag(e[1:], -1)
        np.testing.assert_allclose(O.eig_tridiag(d, e), np.linalg.eigvalsh(T), rtol=1e-13, atol=1e-14)


def test_mlp_reference_gradient_finite_differences():
    """The CPU reference of the learned-parameter MLP (exact FP64 mode) against
    central finite differences of its own loss."""
    import mlp_ref
    rng = np.random.default_rng(0)
    X = rng.uniform(-1, 1, (40, 16))
    T = rng.uniform(0, 1, (40, 2))
    p = mlp_ref.init_params(1)
    p[-2:] = [0.3, 0.8]
    _, g = mlp_ref.gradient(X, T, p, rounding=False)
    idx = rng.choice(len(p), 60, replace=False)
    for k in idx:
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (mlp_ref.gradient(X, T, pp, rounding=False)[0] - mlp_ref.gradient(X, T, pm, rounding=False)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(g[k]), (k, fd, g[k])
