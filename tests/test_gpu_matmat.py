"""HYPRE_ParCSRMatrixMatmat (C = A*B) on the GPU through the C ABI.

* Against the reference library itself: every mm_* fixture (C = A*A written
  by the reference's HYPRE_ParCSRMatrixMatmat on its IJ-assembled A, including
  a matrix with empty rows, where the reference reserves no diagonal, and a
  random unsymmetric one) is reproduced bit for bit -- the IJ-assembled A
  from the same puts, then C's row pointers, column order and FP64 values.
* The reference's own SpGEMM benchmark (src/test/TEST_bench/benchmark_spgemm.jobs:13-16,
  saved output benchmark_spgemm.saved.tioga): the A^2 nonzero counts of the
  7-point and 27-point Laplacians on 128^3 and of the 5-point and 9-point
  Laplacians on 1024^2 grids, with a seeded sample of rows checked bit for
  bit against the sequential product.
"""
import numpy as np
import pytest

import golden_cases as G

pytestmark = pytest.mark.gpu

# A^2 nonzeros saved by the reference's benchmark (benchmark_spgemm.saved.tioga)
SPGEMM_NNZ = {"lap7_128": 51742208, "lap27_128": 254840104, "lap5_1024": 13611012, "lap9_1024": 26152996}


def _host_matrix(gb, I, J, V):
    import ctypes as C
    A = C.c_void_p()
    I, J, V = (np.ascontiguousarray(I, np.int32), np.ascontiguousarray(J, np.int32),
               np.ascontiguousarray(V, np.float64))
    gb.check(gb.lib().HYPRE_GB300_ParCSRMatrixCreateFromHostCSR(len(I) - 1, I.ctypes.data, J.ctypes.data,
                                                                V.ctypes.data, C.byref(A)), "matrix")
    return A


def _put_rows(g):
    """The rows as the reference driver put them (SetRowSizes, then the rows)."""
    if "in_i" in g:
        return g["in_i"], g["in_j"], g["in_v"]
    from hypre_gb300 import problems as P
    return P.laplace(g["case"]["kind"], *g["case"]["n"])


@pytest.mark.parametrize("name", G.matmat_names())
def test_matmat_matches_reference(gb, name):
    g = G.load(name)
    ij = gb.IJMatrix(*_put_rows(g))
    A = ij.par
    # IJ assembly gives the reference's assembled rows (order included)
    Ia, Ja, Va = gb.parcsr_to_host(A)
    assert np.array_equal(Ia, g["A0_i"]) and np.array_equal(Ja, g["A0_j"]) and np.array_equal(Va, g["A0_v"])
    for rep in range(2):
        Cm = gb.matmat(A, A)
        Ci, Cj, Cv = gb.parcsr_to_host(Cm)
        assert np.array_equal(Ci, g["C0_i"]), f"{name} row pointers (call {rep})"
        assert np.array_equal(Cj, g["C0_j"]), f"{name} column order (call {rep})"
        assert np.array_equal(Cv, g["C0_v"]), f"{name} values (call {rep})"
        gb.check(gb.lib().HYPRE_ParCSRMatrixDestroy(Cm))
    ij.destroy()


def test_matmat_rejects_incompatible(gb):
    from hypre_gb300 import problems as P
    import ctypes as C
    L = gb.lib()
    L.HYPRE_ClearAllErrors()
    A = _host_matrix(gb, *P.laplace(7, 4, 4, 4))
    B = _host_matrix(gb, *P.laplace(7, 4, 4, 3))
    Cp = C.c_void_p()
    err = L.HYPRE_ParCSRMatrixMatmat(A, B, C.byref(Cp))
    assert err & gb.HYPRE_ERROR_ARG and not Cp.value
    L.HYPRE_ClearAllErrors()
    for M in (A, B):
        L.HYPRE_GB300_ParCSRMatrixDestroy(M)


def _stencil(name):
    from hypre_gb300 import problems as P
    if name == "lap7_128":
        return P.laplace(7, 128, 128, 128)
    if name == "lap27_128":
        return P.laplace(27, 128, 128, 128)
    I, J, V = P.laplace(7 if name == "lap5_1024" else 27, 1024, 1024, 1)
    diag = J == np.repeat(np.arange(len(I) - 1), np.diff(I))
    return I, J, np.where(diag, 4.0 if name == "lap5_1024" else 8.0, V)


def _row_product(I, J, V, i):
    """Row i of A*A as the reference's sequential product forms it: diagonal
    first, then columns in discovery order, terms added in product order."""
    cols = {i: 0}
    order, vals = [i], [0.0]
    for ka in range(I[i], I[i + 1]):
        r, a = J[ka], V[ka]
        for kb in range(I[r], I[r + 1]):
            c = J[kb]
            if c not in cols:
                cols[c] = len(order)
                order.append(c)
                vals.append(a * V[kb])
            else:
                vals[cols[c]] += a * V[kb]
    return np.array(order, np.int32), np.array(vals)


@pytest.mark.parametrize("name", list(SPGEMM_NNZ))
def test_spgemm_benchmark_nnz(gb, name):
    I, J, V = _stencil(name)
    n = len(I) - 1
    A = _host_matrix(gb, I, J, V)
    Cm = gb.matmat(A, A)
    Ci, Cj, Cv = gb.parcsr_to_host(Cm)
    assert int(Ci[-1]) == SPGEMM_NNZ[name], (name, int(Ci[-1]))
    rng = np.random.default_rng(17)
    rows = np.concatenate([[0, 1, n // 2, n - 1], rng.choice(n, 60, replace=False)])
    for i in rows:
        cols, vals = _row_product(I, J, V, int(i))
        assert np.array_equal(Cj[Ci[i]:Ci[i + 1]], cols), (name, int(i))
        assert np.array_equal(Cv[Ci[i]:Ci[i + 1]], vals), (name, int(i))
    gb.check(gb.lib().HYPRE_ParCSRMatrixDestroy(Cm))
    gb.lib().HYPRE_GB300_ParCSRMatrixDestroy(A)
