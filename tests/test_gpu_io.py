"""IJ matrix and vector files: the reference's text IJ format, Matrix Market
coordinate files and the binary IJ format (src/IJ_mv/IJMatrix.c:110-520,
src/parcsr_mv/par_csr_matrix.c:940-1330, src/IJ_mv/HYPRE_IJVector.c:785-925,
src/IJ_mv/IJVector.c:110-240, src/parcsr_mv/par_vector.c:1360-1440).  Files are
written here with numpy in the formats those functions read and write; the
matrices read back are checked against the IJ interface's assembly rules
(first appearance sets a row's column order, a repeated entry replaces the
earlier value, the diagonal moves to the front of its row)."""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HYPRE_PARCSR = 5555
ERR_GENERIC, ERR_ARG = 1, 4


def _entries(n, seed):
    """A 7-point-like pattern on a 1-D index set with random values, the
    entries shuffled, plus one repeated entry whose second value wins."""
    rng = np.random.default_rng(seed)
    rows, cols = [], []
    for i in range(n):
        for j in (i - 7, i - 1, i, i + 1, i + 7):
            if 0 <= j < n:
                rows.append(i)
                cols.append(j)
    rows, cols = np.array(rows), np.array(cols)
    vals = rng.standard_normal(len(rows))
    vals[rows == cols] += 10.0
    p = rng.permutation(len(rows))
    rows, cols, vals = rows[p], cols[p], vals[p]
    k = len(rows) // 3
    rows = np.append(rows, rows[k])
    cols = np.append(cols, cols[k])
    vals = np.append(vals, 123.25)
    return rows, cols, vals


def _assembled(n, rows, cols, vals):
    """CSR by the IJ rules: column order of first appearance, last value,
    diagonal shifted to the front."""
    order = [dict() for _ in range(n)]
    for r, c, v in zip(rows, cols, vals):
        order[r][int(c)] = float(v)   # dicts keep first-insertion order; later values replace
    I, J, V = [0], [], []
    for i in range(n):
        items = list(order[i].items())
        d = [t for t in items if t[0] == i]
        rest = [t for t in items if t[0] != i]
        for c, v in d + rest:
            J.append(c)
            V.append(v)
        I.append(len(J))
    return np.array(I, np.int32), np.array(J, np.int32), np.array(V)


def _read_matrix(gb, fn, path):
    L = gb.lib()
    h = C.c_void_p()
    err = getattr(L, fn)(path.encode(), 0, HYPRE_PARCSR, C.byref(h))
    assert err == 0, f"{fn} error {err}"
    par = C.c_void_p()
    L.HYPRE_IJMatrixGetObject(h, C.byref(par))
    csr = gb.parcsr_to_host(par)
    return h, csr


def _check_csr(got, want):
    assert np.array_equal(got[0], want[0]), "row pointers"
    assert np.array_equal(got[1], want[1]), "columns (pattern and order)"
    assert np.array_equal(got[2], want[2]), "values"


def _write_ij(path, n, rows, cols, vals):
    with open(path + ".00000", "w") as f:
        f.write(f"0 {n - 1} 0 {n - 1}\n")
        for r, c, v in zip(rows, cols, vals):
            f.write(f"{r} {c} {float(v)!r}\n")


def test_ij_text_read(gb, tmp_path):
    n = 300
    rows, cols, vals = _entries(n, 1)
    path = str(tmp_path / "A")
    _write_ij(path, n, rows, cols, vals)
    h, got = _read_matrix(gb, "HYPRE_IJMatrixRead", path)
    _check_csr(got, _assembled(n, rows, cols, vals))
    gb.lib().HYPRE_IJMatrixDestroy(h)


def test_ij_text_print_format_and_round_trip(gb, tmp_path):
    n = 200
    rows, cols, vals = _entries(n, 2)
    I, J, V = _assembled(n, rows, cols, vals)
    A = gb.IJMatrix(I, J, V)
    path = str(tmp_path / "P")
    assert gb.lib().HYPRE_IJMatrixPrint(A.h, path.encode()) == 0
    want = [f"0 {n - 1} 0 {n - 1}\n"]
    for i in range(n):
        for k in range(I[i], I[i + 1]):
            want.append("%d %d %.14e\n" % (i, J[k], V[k]))
    assert open(path + ".00000").read() == "".join(want)
    h, got = _read_matrix(gb, "HYPRE_IJMatrixRead", path)
    # %.14e keeps 15 significant digits: the values read back are those printed
    _check_csr(got, (I, J, np.array([float("%.14e" % v) for v in V])))
    gb.lib().HYPRE_IJMatrixDestroy(h)


@pytest.mark.parametrize("sym", [False, True])
def test_matrix_market_read(gb, tmp_path, sym):
    n = 150
    rows, cols, vals = _entries(n, 3)
    if sym:
        # one triangle in the file; the reader mirrors (j, i) after each (i, j)
        keep = rows >= cols
        rows, cols, vals = rows[keep], cols[keep], vals[keep]
        er, ec, ev = [], [], []
        for r, c, v in zip(rows, cols, vals):
            er.append(r); ec.append(c); ev.append(v)
            if r != c:
                er.append(c); ec.append(r); ev.append(v)
        want = _assembled(n, np.array(er), np.array(ec), np.array(ev))
    else:
        want = _assembled(n, rows, cols, vals)
    path = str(tmp_path / "A.mtx")
    with open(path, "w") as f:
        f.write("%%%%MatrixMarket matrix coordinate real %s\n" % ("symmetric" if sym else "general"))
        f.write("% a comment line\n")
        f.write(f"{n} {n} {len(rows)}\n")
        for r, c, v in zip(rows, cols, vals):
            f.write(f"{r + 1} {c + 1} {float(v)!r}\n")
    h, got = _read_matrix(gb, "HYPRE_IJMatrixReadMM", path)
    _check_csr(got, want)
    gb.lib().HYPRE_IJMatrixDestroy(h)


def test_binary_round_trip_and_foreign_widths(gb, tmp_path):
    n = 250
    rows, cols, vals = _entries(n, 4)
    I, J, V = _assembled(n, rows, cols, vals)
    A = gb.IJMatrix(I, J, V)
    path = str(tmp_path / "B")
    assert gb.lib().HYPRE_IJMatrixPrintBinary(A.h, path.encode()) == 0
    raw = open(path + ".00000.bin", "rb").read()
    hdr = np.frombuffer(raw[:88], np.uint64)
    nnz = int(I[-1])
    assert list(hdr) == [1, 4, 8, n, n, nnz, nnz, 0, n - 1, 0, n - 1]
    h, got = _read_matrix(gb, "HYPRE_IJMatrixReadBinary", path)
    _check_csr(got, (I, J, V))
    gb.lib().HYPRE_IJMatrixDestroy(h)
    # 64-bit indices and FP32 values, entries in shuffled order
    path2 = str(tmp_path / "C")
    v32 = vals.astype(np.float32)
    with open(path2 + ".00000.bin", "wb") as f:
        f.write(np.array([1, 8, 4, n, n, len(rows), len(rows), 0, n - 1, 0, n - 1], np.uint64).tobytes())
        f.write(rows.astype(np.uint64).tobytes())
        f.write(cols.astype(np.uint64).tobytes())
        f.write(v32.tobytes())
    h, got = _read_matrix(gb, "HYPRE_IJMatrixReadBinary", path2)
    _check_csr(got, _assembled(n, rows, cols, v32.astype(np.float64)))
    gb.lib().HYPRE_IJMatrixDestroy(h)


def test_read_then_solve(gb, oracle_mod, tmp_path):
    """A Laplacian read from a file solves like the same matrix put directly."""
    O = oracle_mod
    I, J, V = O.stencil(7, 10, 10, 10)
    n = len(I) - 1
    path = str(tmp_path / "L")
    rows = np.repeat(np.arange(n), np.diff(I))
    _write_ij(path, n, rows, J, V)
    h, got = _read_matrix(gb, "HYPRE_IJMatrixRead", path)
    _check_csr(got, (I, J, V))
    L = gb.lib()

    class _Read:
        par = C.c_void_p()

    A = _Read()
    L.HYPRE_IJMatrixGetObject(h, C.byref(A.par))
    b = O.rhs_normalised(n)
    bv, xv = gb.IJVector(n, b), gb.IJVector(n, np.zeros(n))
    amg = gb.BoomerAMG(MaxRowSum=1.0, Tol=0.0, MaxIter=1)
    k = gb.Krylov("pcg", tol=1e-8, maxit=100, amg=amg)
    k.setup(A, bv, xv)
    k.solve(A, bv, xv)
    x = xv.values()
    import scipy.sparse as sp
    r = b - sp.csr_matrix((V, J, I), shape=(n, n)) @ x
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1e-8
    L.HYPRE_IJMatrixDestroy(h)


def test_vector_text_and_binary(gb, tmp_path):
    L = gb.lib()
    n = 97
    rng = np.random.default_rng(5)
    x = rng.standard_normal(n)
    # text, entries shuffled, one written twice (the second value wins)
    path = str(tmp_path / "b")
    p = rng.permutation(n)
    with open(path + ".00000", "w") as f:
        f.write(f"0 {n - 1}\n")
        for j in p:
            f.write(f"{j} {float(x[j])!r}\n")
        f.write(f"{p[0]} 7.5\n")
    want = x.copy()
    want[p[0]] = 7.5
    h = C.c_void_p()
    assert L.HYPRE_IJVectorRead(path.encode(), 0, HYPRE_PARCSR, C.byref(h)) == 0
    got = np.empty(n)
    L.HYPRE_IJVectorGetValues(h, n, None, got.ctypes.data)
    assert np.array_equal(got, want)
    jl, ju = C.c_int(), C.c_int()
    L.HYPRE_IJVectorGetLocalRange(h, C.byref(jl), C.byref(ju))
    assert (jl.value, ju.value) == (0, n - 1)
    # print: header, then "j %.14e"
    out = str(tmp_path / "bp")
    assert L.HYPRE_IJVectorPrint(h, out.encode()) == 0
    text = open(out + ".00000").read()
    assert text == f"0 {n - 1}\n" + "".join("%d %.14e\n" % (j, want[j]) for j in range(n))
    # binary round trip, then an FP32 file
    outb = str(tmp_path / "bb")
    assert L.HYPRE_IJVectorPrintBinary(h, outb.encode()) == 0
    raw = open(outb + ".00000.bin", "rb").read()
    assert list(np.frombuffer(raw[:64], np.uint64)) == [1, 8, 0, n, n, n, 1, 0]
    h2 = C.c_void_p()
    assert L.HYPRE_IJVectorReadBinary(outb.encode(), 0, HYPRE_PARCSR, C.byref(h2)) == 0
    L.HYPRE_IJVectorGetValues(h2, n, None, got.ctypes.data)
    assert np.array_equal(got, want)
    f32 = str(tmp_path / "b32")
    with open(f32 + ".00000.bin", "wb") as f:
        f.write(np.array([1, 4, 0, n, n, n, 1, 0], np.uint64).tobytes())
        f.write(x.astype(np.float32).tobytes())
    h3 = C.c_void_p()
    assert L.HYPRE_IJVectorReadBinary(f32.encode(), 0, HYPRE_PARCSR, C.byref(h3)) == 0
    L.HYPRE_IJVectorGetValues(h3, n, None, got.ctypes.data)
    assert np.array_equal(got, x.astype(np.float32).astype(np.float64))
    for v in (h, h2, h3):
        L.HYPRE_IJVectorDestroy(v)


def test_read_errors(gb, tmp_path):
    L = gb.lib()
    h = C.c_void_p()
    L.HYPRE_ClearAllErrors()
    missing = str(tmp_path / "nothing")
    err = L.HYPRE_IJMatrixRead(missing.encode(), 0, HYPRE_PARCSR, C.byref(h))
    assert err & ERR_ARG
    L.HYPRE_ClearAllErrors()
    bad = str(tmp_path / "bad")
    with open(bad + ".00000", "w") as f:
        f.write("0 3 0 3\n0 0 1.0\n1 1.5\n")
    err = L.HYPRE_IJMatrixRead(bad.encode(), 0, HYPRE_PARCSR, C.byref(h))
    assert err & ERR_GENERIC
    L.HYPRE_ClearAllErrors()
    mm = str(tmp_path / "c.mtx")
    with open(mm, "w") as f:
        f.write("%%MatrixMarket matrix coordinate complex general\n2 2 1\n1 1 1.0 0.0\n")
    err = L.HYPRE_IJMatrixReadMM(mm.encode(), 0, HYPRE_PARCSR, C.byref(h))
    assert err & ERR_GENERIC
    L.HYPRE_ClearAllErrors()
    assert not os.path.exists(missing + ".00000")


def test_par_vector_print_read_and_get_values(gb, tmp_path):
    """HYPRE_ParVectorPrint writes the reference's one-process files
    (<name>.0: the size, then %.14e per line; <name>.INFO.0: global size and
    row range), HYPRE_ParVectorRead reads them back, and
    HYPRE_ParVectorGetValues returns values by index."""
    import ctypes as C
    L = gb.lib()
    L.HYPRE_ParVectorPrint.argtypes = [C.c_void_p, C.c_char_p]
    L.HYPRE_ParVectorRead.argtypes = [C.c_int, C.c_char_p, C.POINTER(C.c_void_p)]
    L.HYPRE_ParVectorGetValues.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    L.HYPRE_ClearAllErrors()
    n = 37
    x = np.random.default_rng(5).standard_normal(n)
    v = gb.IJVector(n, x)
    name = str(tmp_path / "vec")
    gb.check(L.HYPRE_ParVectorPrint(v.par, name.encode()))
    lines = open(name + ".0").read().split()
    assert int(lines[0]) == n and lines[1] == "%.14e" % x[0]
    assert open(name + ".INFO.0").read().split() == [str(n), "0", str(n)]
    w = C.c_void_p()
    gb.check(L.HYPRE_ParVectorRead(0, name.encode(), C.byref(w)))
    back = np.zeros(n)
    gb.check(L.HYPRE_ParVectorGetValues(w, n, None, back.ctypes.data))
    np.testing.assert_array_equal(back, np.array([float("%.14e" % t) for t in x]))
    idx = np.array([3, 0, 36], np.int32)
    got = np.zeros(3)
    gb.check(L.HYPRE_ParVectorGetValues(v.par, 3, idx.ctypes.data, got.ctypes.data))
    np.testing.assert_array_equal(got, x[idx])
    L.HYPRE_ParVectorDestroy(w)
    v.destroy()


def test_parcsr_print_and_read(gb, oracle_mod, tmp_path):
    """HYPRE_ParCSRMatrixPrint writes the reference's one-process files
    (<name>.D.0: row count, 1-based row pointers and columns, %.14e values;
    <name>.INFO.0: sizes and ranges) and HYPRE_ParCSRMatrixRead reads them
    back to the same matrix."""
    import ctypes as C
    L = gb.lib()
    L.HYPRE_ParCSRMatrixPrint.argtypes = [C.c_void_p, C.c_char_p]
    L.HYPRE_ParCSRMatrixRead.argtypes = [C.c_int, C.c_char_p, C.POINTER(C.c_void_p)]
    L.HYPRE_ClearAllErrors()
    I, J, V = oracle_mod.stencil(27, 5, 4, 3)
    V = V * (1.0 + 0.001 * np.arange(len(V)))
    n = len(I) - 1
    A = gb.IJMatrix(I, J, V)
    name = str(tmp_path / "mat")
    gb.check(L.HYPRE_ParCSRMatrixPrint(A.par, name.encode()))
    d = open(name + ".D.0").read().split()
    I2, J2, V2 = A.csr()
    assert int(d[0]) == n and [int(t) for t in d[1:n + 2]] == list(I2 + 1)
    assert open(name + ".INFO.0").read().split() == [str(n), str(n), "0", "0", str(n), "0", str(n)]
    B = C.c_void_p()
    gb.check(L.HYPRE_ParCSRMatrixRead(0, name.encode(), C.byref(B)))
    I3, J3, V3 = gb.parcsr_to_host(B)
    np.testing.assert_array_equal(I3, I2)
    np.testing.assert_array_equal(J3, J2)
    np.testing.assert_array_equal(V3, np.array([float("%.14e" % t) for t in V2]))
    L.HYPRE_ParCSRMatrixDestroy(B)
    A.destroy()
