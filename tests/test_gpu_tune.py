"""The SpMV launch-shape autotuner (gb_tune.c) through the C ABI.

* Every SELL-32 shape (prefetch depth 1/2/4/8 x block 128/256/512) sums each
  row in element order: its result equals the default shape's bit for bit.
* CSR lane counts (2..32 lanes per row) split a row's sum: their results agree
  with the default's to rounding (1e-14 relative).
* Tuning a new matrix shape writes the choice to the JSON cache named by
  HYPRE_GB300_TUNE_CACHE, and a solve with tuning on reproduces the solve with
  tuning off (residual history to 1e-12, same iterations)."""
import ctypes as C
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _matrix(gb, I, J, V):
    A = C.c_void_p()
    I, J, V = (np.ascontiguousarray(I, np.int32), np.ascontiguousarray(J, np.int32),
               np.ascontiguousarray(V, np.float64))
    gb.check(gb.lib().HYPRE_GB300_ParCSRMatrixCreateFromHostCSR(len(I) - 1, I.ctypes.data, J.ctypes.data,
                                                                V.ctypes.data, C.byref(A)), "matrix")
    return A


def _matvec(gb, A, x):
    n = len(x)
    xv, yv = gb.IJVector(n, x), gb.IJVector(n, np.zeros(n))
    gb.check(gb.lib().HYPRE_ParCSRMatrixMatvec(1.0, A, xv.par, 0.0, yv.par))
    y = yv.values()
    xv.destroy(); yv.destroy()
    return y


def _shape(gb, A, prec=0):
    f, b, d = C.c_int(), C.c_int(), C.c_int()
    gb.check(gb.lib().HYPRE_GB300_ParCSRMatrixGetSpMVShape(A, prec, C.byref(f), C.byref(b), C.byref(d)))
    return f.value, b.value, d.value


def test_sell_shapes_identical(gb):
    from hypre_gb300 import problems as P
    L = gb.lib()
    I, J, V = P.laplace(27, 40, 41, 42)
    V = V * (1.0 + 0.25 * np.random.default_rng(3).random(len(V)))
    A = _matrix(gb, I, J, V)
    x = np.random.default_rng(4).standard_normal(len(I) - 1)
    gb.check(L.HYPRE_GB300_ParCSRMatrixSetSpMVShape(A, 0, 0, 0))
    assert _shape(gb, A)[0] == 1                     # SELL-32
    ref = _matvec(gb, A, x)
    for D in (1, 2, 4, 8):
        for T in (128, 256, 512):
            gb.check(L.HYPRE_GB300_ParCSRMatrixSetSpMVShape(A, 0, T, D))
            assert _shape(gb, A) == (1, T, D)
            assert np.array_equal(_matvec(gb, A, x), ref), (D, T)
    L.HYPRE_GB300_ParCSRMatrixDestroy(A)


def test_csr_lanes_agree(gb):
    L = gb.lib()
    rng = np.random.default_rng(8)
    n = 30000
    lens = rng.integers(1, 120, n)                   # uneven rows: the CSR form
    I = np.zeros(n + 1, np.int64)
    np.cumsum(lens, out=I[1:])
    J = np.concatenate([np.sort(rng.choice(n, l, replace=False)) for l in lens]).astype(np.int32)
    V = rng.standard_normal(len(J))
    A = _matrix(gb, I.astype(np.int32), J, V)
    assert _shape(gb, A)[0] == 0
    x = rng.standard_normal(n)
    ref = _matvec(gb, A, x)
    for K in (2, 4, 8, 16, 32):
        for T in (128, 256, 512):
            gb.check(L.HYPRE_GB300_ParCSRMatrixSetSpMVShape(A, 0, T, K))
            assert _shape(gb, A) == (0, T, K)
            np.testing.assert_allclose(_matvec(gb, A, x), ref, rtol=1e-14, atol=1e-14 * np.abs(ref).max())
    L.HYPRE_GB300_ParCSRMatrixDestroy(A)


def test_tuned_solve_matches_default_and_cache_written(gb, tmp_path, monkeypatch):
    from hypre_gb300 import problems as P
    L = gb.lib()
    cache = tmp_path / "tune.json"
    monkeypatch.setenv("HYPRE_GB300_TUNE_CACHE", str(cache))
    I, J, V = P.laplace(27, 37, 38, 39)              # a shape no other test tunes
    n = len(I) - 1
    b = P.rhs(n)
    runs = []
    for on in (0, 1):
        L.HYPRE_GB300_SetAutotune(on)
        A = gb.IJMatrix(I, J, V)
        bv, xv = gb.IJVector(n, b), gb.IJVector(n, np.zeros(n))
        amg = gb.BoomerAMG(MaxRowSum=1.0, StrongThreshold=0.5, Tol=0.0, MaxIter=1)
        k = gb.Krylov("pcg", tol=1e-8, maxit=100, amg=amg)
        k.setup(A, bv, xv)
        k.solve(A, bv, xv)
        runs.append((k.iterations(), k.history(), _shape(gb, A.par, 0)))
        for o in (k, amg, xv, bv, A):
            o.destroy()
    L.HYPRE_GB300_SetAutotune(1)
    (it0, h0, s0), (it1, h1, s1) = runs
    assert it0 == it1
    np.testing.assert_allclose(h1, h0, rtol=1e-12, atol=0)
    assert s0 == (1, 256, 4)                          # untuned: the default SELL shape
    entries = json.load(open(cache))
    key = "sell:f64v32:i16:%d:%d" % (n, len(J))
    assert key in entries and entries[key][:2] == [s1[1], s1[2]], (entries, s1)


def _multi_solve(gb, O, I, J, V, B, prec):
    n, nv = B.shape
    A = gb.IJMatrix(I, J, V)
    amg = gb.BoomerAMG(MaxRowSum=1.0, StrongThreshold=0.5, Tol=0.0, MaxIter=1)
    amg.set("CyclePrecision", prec)
    k = gb.Krylov("pcg", tol=1e-8, maxit=100, amg=amg)
    b1, x1 = gb.IJVector(n, B[:, 0]), gb.IJVector(n, np.zeros(n))
    k.setup(A, b1, x1)
    Bm, Xm = gb.MultiVector(B), gb.MultiVector(np.zeros((n, nv)))
    assert gb.lib().HYPRE_ParCSRPCGSolve(k.h, A.par, Bm.par, Xm.par) == 0
    its, rel, hist = gb.multi_results(k, nv, 100)
    X = Xm.values()
    for o in (k, amg, x1, b1, A):
        o.destroy()
    return its, hist, X


def test_spmm_shapes_identical(gb, oracle_mod, monkeypatch):
    """Every SpMM launch shape (block 128/256/512 x 1/2/4/8 rows of x in
    flight) gives the multi-vector PCG the same iterations, histories and
    solution, bit for bit, in the FP64 and the FP32 cycle."""
    O = oracle_mod
    I, J, V = O.stencil(27, 30, 30, 30)              # 27,000 rows: tuned operands
    n, nv = len(I) - 1, 6
    B = np.stack([O.rand_uniform(n, 500 + c) for c in range(nv)], 1)
    for prec in (0, 1):
        monkeypatch.setenv("HYPRE_GB300_SPMM_SHAPE", "256,2")
        ref = _multi_solve(gb, O, I, J, V, B, prec)
        for T in (128, 256, 512):
            for U in (1, 2, 4, 8):
                monkeypatch.setenv("HYPRE_GB300_SPMM_SHAPE", f"{T},{U}")
                its, hist, X = _multi_solve(gb, O, I, J, V, B, prec)
                assert np.array_equal(its, ref[0]), (prec, T, U)
                assert len(hist) == len(ref[1])
                assert all(np.array_equal(a, b) for a, b in zip(hist, ref[1])), (prec, T, U)
                assert np.array_equal(X, ref[2]), (prec, T, U)


def test_spmm_tuned_cache_written(gb, oracle_mod, tmp_path, monkeypatch):
    O = oracle_mod
    cache = tmp_path / "tune.json"
    monkeypatch.setenv("HYPRE_GB300_TUNE_CACHE", str(cache))
    monkeypatch.delenv("HYPRE_GB300_SPMM_SHAPE", raising=False)
    gb.lib().HYPRE_GB300_SetAutotune(1)
    I, J, V = O.stencil(27, 29, 30, 31)              # shapes no other test tunes
    n, nv = len(I) - 1, 7
    B = np.stack([O.rand_uniform(n, 900 + c) for c in range(nv)], 1)
    its, hist, X = _multi_solve(gb, O, I, J, V, B, 0)
    entries = json.load(open(cache))
    key = "spmm:f64:nv%d:%d:%d:%d" % (nv, n, n, len(J))
    assert key in entries, sorted(entries)
    T, U = entries[key][:2]
    assert T in (128, 256, 512) and U in (1, 2, 4, 8)
