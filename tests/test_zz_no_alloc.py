"""GPU test of the transpose mat-vec that allocates nothing
(HYPRE_GB300_ParCSRMatrixMatvecTNoAlloc), called through the C ABI.

Callers that cannot allocate device memory -- code running while a stream is
captured into a CUDA graph, or a host framework that owns all device memory --
use this entry point; its transpose lives in a fixed 32 MiB device array.
Its result must match the allocating HYPRE_ParCSRMatrixMatvecT on two calls
in a row (the array keeps the previous call's contents, which must not leak
into the next result), and a matrix too large for the array must be rejected
with an argument error.  This file is collected last so a failure here comes
after every other test has run."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-13


def _vec(gb, v):
    return gb.IJVector(len(v), v)


def test_no_alloc_matvecT_matches_allocating_form(gb):
    from hypre_gb300 import problems as G
    L = gb.lib()
    L.HYPRE_GB300_ParCSRMatrixMatvecTNoAlloc.argtypes = [C.c_double, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]
    L.HYPRE_GB300_ParCSRMatrixMatvecTNoAlloc.restype = C.c_int
    L.HYPRE_ClearAllErrors()
    # a non-symmetric matrix so A^T x differs from A x
    I, J, V = G.laplace(27, 14, 15, 16)
    rng = np.random.default_rng(11)
    V = V * (1.0 + 0.5 * rng.random(len(V)))
    A = gb.IJMatrix(I, J, V)
    n = len(I) - 1
    for call, (alpha, beta, seed) in enumerate(((1.0, 0.0, 1), (-0.7, 1.3, 2))):
        r = np.random.default_rng(seed)
        x = r.standard_normal(n)
        y0 = r.standard_normal(n)
        xv, y_ref, y_na = _vec(gb, x), _vec(gb, y0), _vec(gb, y0)
        assert L.HYPRE_ParCSRMatrixMatvecT(alpha, A.par, xv.par, beta, y_ref.par) == 0
        assert L.HYPRE_GB300_ParCSRMatrixMatvecTNoAlloc(alpha, A.par, xv.par, beta, y_na.par) == 0, f"call {call}"
        ref, got = y_ref.values(), y_na.values()
        np.testing.assert_allclose(got, ref, rtol=RTOL, atol=RTOL * np.abs(ref).max())
        for v in (xv, y_ref, y_na):
            v.destroy()
    A.destroy()


def test_no_alloc_matvecT_rejects_too_large(gb):
    from hypre_gb300 import problems as G
    L = gb.lib()
    L.HYPRE_ClearAllErrors()
    I, J, V = G.laplace(27, 48, 48, 48)     # 2.9M nonzeros: transpose needs > 32 MiB
    A = gb.IJMatrix(I, J, V)
    n = len(I) - 1
    xv, yv = _vec(gb, np.ones(n)), _vec(gb, np.zeros(n))
    err = L.HYPRE_GB300_ParCSRMatrixMatvecTNoAlloc(1.0, A.par, xv.par, 0.0, yv.par)
    assert err & gb.HYPRE_ERROR_ARG
    assert np.all(yv.values() == 0.0)
    L.HYPRE_ClearAllErrors()
    for o in (xv, yv, A):
        o.destroy()
