"""The reference's own IJ test fixtures read and solved through the C ABI.

tests/golden/ij_poisson_10x10x10_np1/ holds the reference's binary IJ files
(src/test/TEST_ij/data/poisson_10x10x10_np1/IJ.{A,b,x0}.{i4f8,i8f8,i4f4,i8f4}.00000.bin:
a 10^3 Poisson matrix, right-hand side and initial guess with 32/64-bit
indices and 32/64-bit values).  The reference's io tests
(src/test/TEST_ij/io.jobs:11-29) read each set with `ij -solver 2 -tol 1e-2`
(diagonally scaled PCG) and save 11 iterations and final relative residual
6.733697e-03 (src/test/TEST_ij/io.saved:1-14).  Here each set is read with
HYPRE_IJMatrixReadBinary / HYPRE_IJVectorReadBinary and solved the same way,
and the same matrix is solved by BoomerAMG-PCG against the oracle (hierarchy
bit for bit, residual history to 1e-10)."""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ij_poisson_10x10x10_np1")
HYPRE_PARCSR = 5555


def _read(gb, kind, prefix):
    L = gb.lib()
    h = C.c_void_p()
    fn = L.HYPRE_IJMatrixReadBinary if kind == "A" else L.HYPRE_IJVectorReadBinary
    assert fn(os.path.join(DATA, prefix).encode(), 0, HYPRE_PARCSR, C.byref(h)) == 0, prefix
    par = C.c_void_p()
    (L.HYPRE_IJMatrixGetObject if kind == "A" else L.HYPRE_IJVectorGetObject)(h, C.byref(par))
    return h, par


@pytest.mark.parametrize("fmt", ["i4f8", "i8f8", "i4f4", "i8f4"])
def test_reference_io_job(gb, fmt):
    """io.jobs:11-29: DS-PCG, tol 1e-2, from the files' x0."""
    L = gb.lib()
    L.HYPRE_ClearAllErrors()
    hA, A = _read(gb, "A", "IJ.A." + fmt)
    hb, b = _read(gb, "b", "IJ.b." + fmt)
    hx, x = _read(gb, "x", "IJ.x0." + fmt)
    pcg = C.c_void_p()
    gb.check(L.HYPRE_ParCSRPCGCreate(0, C.byref(pcg)))
    L.HYPRE_PCGSetMaxIter(pcg, 1000)
    L.HYPRE_PCGSetTol(pcg, 1e-2)
    L.HYPRE_PCGSetTwoNorm(pcg, 1)
    L.HYPRE_PCGSetRelChange(pcg, 0)
    L.HYPRE_PCGSetPrecond(pcg, gb.fn_ptr("HYPRE_ParCSRDiagScale"), gb.fn_ptr("HYPRE_ParCSRDiagScaleSetup"), None)
    gb.check(L.HYPRE_ParCSRPCGSetup(pcg, A, b, x))
    gb.check(L.HYPRE_ParCSRPCGSolve(pcg, A, b, x))
    it, rel = C.c_int(), C.c_double()
    L.HYPRE_PCGGetNumIterations(pcg, C.byref(it))
    L.HYPRE_PCGGetFinalRelativeResidualNorm(pcg, C.byref(rel))
    assert it.value == 11
    assert "%e" % rel.value == "6.733697e-03", rel.value
    L.HYPRE_ParCSRPCGDestroy(pcg)
    for h, f in ((hx, L.HYPRE_IJVectorDestroy), (hb, L.HYPRE_IJVectorDestroy), (hA, L.HYPRE_IJMatrixDestroy)):
        f(h)


def test_fixture_amg_pcg_matches_oracle(gb, oracle_mod):
    """The file's matrix and right-hand side through BoomerAMG-PCG (x0 = 0)
    against the oracle: every level bit for bit, history to 1e-10."""
    O = oracle_mod
    L = gb.lib()
    hA, A = _read(gb, "A", "IJ.A.i4f8")
    hb, b = _read(gb, "b", "IJ.b.i4f8")
    I, J, V = gb.parcsr_to_host(A)
    n = len(I) - 1
    bh = np.empty(n)
    L.HYPRE_IJVectorGetValues(hb, n, None, bh.ctypes.data)
    H = O.Hierarchy(I, J, V, O.default_params(max_row_sum=1.0))
    _, rel_o, it_o = H.pcg(bh, tol=1e-8, maxit=100)

    class _M:
        par = A

    bv, xv = gb.IJVector(n, bh), gb.IJVector(n, np.zeros(n))
    amg = gb.BoomerAMG(MaxRowSum=1.0, Tol=0.0, MaxIter=1)
    k = gb.Krylov("pcg", tol=1e-8, maxit=100, amg=amg)
    k.setup(_M, bv, xv)
    k.solve(_M, bv, xv)
    assert amg.num_levels() == H.num_levels
    for l in range(H.num_levels):
        for w in ("A", "P") if l < H.num_levels - 1 else ("A",):
            g, o = amg.level_csr(l, w)[:3], H.csr(w, l)[:3]
            assert all(np.array_equal(a, c) for a, c in zip(g, o)), (w, l)
    assert k.iterations() == it_o
    np.testing.assert_allclose(k.history(), rel_o, rtol=1e-10, atol=0)
    for o in (k, amg, xv, bv):
        o.destroy()
    L.HYPRE_IJVectorDestroy(hb)
    L.HYPRE_IJMatrixDestroy(hA)
