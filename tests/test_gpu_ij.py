"""IJ matrix assembly: the device path (one large SetValues call, copied to
the device and gathered there) and the host path (many small calls) give the
same CSR as the reference's rules (IJMatrix_parcsr.c): repeated columns of a
fresh row merged at their first position with the last value, AddToValues
adding to existing entries and appending new ones, and the diagonal moved to
the front of each row by shifting the entries before it, or by swapping it
with the first entry after SetDiagOffdSizes."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def random_rows(n, seed, maxlen=80, dup_rows=()):
    rng = np.random.default_rng(seed)
    rows = []
    for r in range(n):
        l = int(rng.integers(0, maxlen + 1))
        cols = rng.choice(n, size=min(l, n), replace=False)
        if l > 0 and rng.random() < 0.8 and r not in cols:
            cols[rng.integers(0, len(cols))] = r
        cols = list(int(c) for c in cols)
        if r in dup_rows and len(cols) > 2:
            cols.append(cols[1])
        vals = list(rng.standard_normal(len(cols)))
        rows.append((cols, vals))
    return rows


def expected_csr(rows, swap=False, adds=(), sizes=None):
    """The reference's assembly of the puts.  With SetRowSizes (not swap) the
    entry moved to the front of row r is the one whose column is r's ordinal
    among the rows that have space (a size above zero or entries): r itself
    unless some earlier row was given size 0 and no entries
    (IJMatrix_parcsr.c:2830-2906, aux_parcsr_matrix.c:164-215)."""
    out = []
    for r, (cols, vals) in enumerate(rows):
        ec, ev = [], []
        for c, v in zip(cols, vals):
            if c in ec:
                ev[ec.index(c)] = v
            else:
                ec.append(c)
                ev.append(v)
        out.append([ec, ev])
    for r, cols, vals in adds:
        ec, ev = out[r]
        for c, v in zip(cols, vals):
            if c in ec:
                ev[ec.index(c)] += v
            else:
                ec.append(c)
                ev.append(v)
    I, J, V = [0], [], []
    ordinal = 0
    for r, (ec, ev) in enumerate(out):
        ec, ev = list(ec), list(ev)
        front = r if (swap or sizes is None) else ordinal
        if sizes is not None and (sizes[r] > 0 or len(ec) > 0):
            ordinal += 1
        if front in ec:
            d = ec.index(front)
            if d > 0:
                if swap:
                    ec[0], ec[d] = ec[d], ec[0]
                    ev[0], ev[d] = ev[d], ev[0]
                else:
                    ec.insert(0, ec.pop(d))
                    ev.insert(0, ev.pop(d))
        J += ec
        V += ev
        I.append(len(J))
    return np.array(I, np.int32), np.array(J, np.int32), np.array(V, np.float64)


def assemble(gb, rows, bulk, swap=False, adds=(), extra=None, strict=True, sizes=None):
    L = gb.lib()
    n = len(rows)
    h = C.c_void_p()
    gb.check(L.HYPRE_IJMatrixCreate(0, 0, n - 1, 0, n - 1, C.byref(h)), "create")
    L.HYPRE_IJMatrixSetObjectType(h, gb.HYPRE_PARCSR)
    if sizes is None:
        sizes = np.array([max(len(c), 1) for c, _ in rows], np.int32)
    if swap:
        L.HYPRE_IJMatrixSetDiagOffdSizes(h, sizes.ctypes.data, None)
    else:
        L.HYPRE_IJMatrixSetRowSizes(h, sizes.ctypes.data)
    L.HYPRE_IJMatrixInitialize(h)
    if bulk:
        nc = np.array([len(c) for c, _ in rows], np.int32)
        ri = np.arange(n, dtype=np.int32)
        J = np.array([c for cs, _ in rows for c in cs], np.int32)
        V = np.array([v for _, vs in rows for v in vs], np.float64)
        L.HYPRE_IJMatrixSetValues(h, n, nc.ctypes.data, ri.ctypes.data, J.ctypes.data, V.ctypes.data)
    else:
        for r, (cs, vs) in enumerate(rows):
            nc = np.array([len(cs)], np.int32)
            ri = np.array([r], np.int32)
            J = np.array(cs, np.int32)
            V = np.array(vs, np.float64)
            L.HYPRE_IJMatrixSetValues(h, 1, nc.ctypes.data, ri.ctypes.data, J.ctypes.data, V.ctypes.data)
    for r, cs, vs in adds:
        nc = np.array([len(cs)], np.int32)
        ri = np.array([r], np.int32)
        J = np.array(cs, np.int32)
        V = np.array(vs, np.float64)
        L.HYPRE_IJMatrixAddToValues(h, 1, nc.ctypes.data, ri.ctypes.data, J.ctypes.data, V.ctypes.data)
    if extra is not None:
        extra(L, h)
    code = L.HYPRE_IJMatrixAssemble(h)
    if strict:
        gb.check(code, "assemble")
    par = C.c_void_p()
    L.HYPRE_IJMatrixGetObject(h, C.byref(par))
    if not strict:
        L.HYPRE_IJMatrixDestroy(h)
        return None
    out = gb.parcsr_to_host(par)
    L.HYPRE_IJMatrixDestroy(h)
    return out


def same(a, b):
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("swap", [False, True])
def test_bulk_and_per_row_puts_match_reference_rules(gb, swap):
    rows = random_rows(6000, seed=5)
    exp = expected_csr(rows, swap=swap)
    assert len(exp[1]) >= 65536          # large enough for the device path
    same(assemble(gb, rows, bulk=True, swap=swap), exp)
    same(assemble(gb, rows, bulk=False, swap=swap), exp)
    assert gb.lib().HYPRE_GetError() == 0


def test_rows_without_space_shift_the_front_entry(gb):
    """SetRowSizes with zeros for the empty rows (as the reference's drivers
    pass the row lengths): the reference moves to the front the entry whose
    column is the row's ordinal among the rows with space, not the diagonal.
    Device path (one large put) and host path (a put per row) alike."""
    rows = random_rows(6000, seed=9)
    for r in range(0, 6000, 7):
        rows[r] = ([], [])
    sizes = np.array([len(c) for c, _ in rows], np.int32)
    exp = expected_csr(rows, sizes=sizes)
    assert len(exp[1]) >= 65536
    assert not np.array_equal(exp[1], expected_csr(rows)[1])     # the rule changes the result here
    same(assemble(gb, rows, bulk=True, sizes=sizes), exp)
    same(assemble(gb, rows, bulk=False, sizes=sizes), exp)
    assert gb.lib().HYPRE_GetError() == 0


def test_repeated_columns_in_a_large_put_are_merged(gb):
    rows = random_rows(5000, seed=6, dup_rows=(7, 1234, 4999))
    exp = expected_csr(rows)
    same(assemble(gb, rows, bulk=True), exp)
    assert gb.lib().HYPRE_GetError() == 0


def test_add_to_values_after_a_large_put(gb):
    rows = random_rows(5000, seed=7)
    rng = np.random.default_rng(8)
    adds = []
    for r in (3, 77, 2500, 4998):
        cs = list(rows[r][0][:2]) + [int(c) for c in rng.choice(5000, 2, replace=False) if c not in rows[r][0]]
        adds.append((r, cs, list(rng.standard_normal(len(cs)))))
    exp = expected_csr(rows, adds=adds)
    same(assemble(gb, rows, bulk=True, adds=adds), exp)
    same(assemble(gb, rows, bulk=False, adds=adds), exp)


def test_get_values_after_a_large_put(gb):
    rows = random_rows(4000, seed=9)
    got = {}

    def read(L, h):
        for r in (0, 11, 1999, 3999):
            cs = rows[r][0]
            if not cs:
                continue
            nc = np.array([len(cs)], np.int32)
            ri = np.array([r], np.int32)
            J = np.array(cs, np.int32)
            V = np.zeros(len(cs))
            L.HYPRE_IJMatrixGetValues(h, 1, nc.ctypes.data, ri.ctypes.data, J.ctypes.data, V.ctypes.data)
            got[r] = V

    assemble(gb, rows, bulk=True, extra=read)
    for r, V in got.items():
        np.testing.assert_array_equal(V, np.array(rows[r][1]))
    assert gb.lib().HYPRE_GetError() == 0


def test_out_of_range_column_in_a_large_put_is_an_argument_error(gb):
    rows = random_rows(3000, seed=10)
    rows[100][0].append(3000)            # one past the last column
    rows[100][1].append(1.0)
    assemble(gb, rows, bulk=True, strict=False)
    assert gb.lib().HYPRE_GetError() & 4        # HYPRE_ERROR_ARG
    gb.lib().HYPRE_ClearAllErrors()


def test_get_row(gb):
    rows = random_rows(3000, seed=11)
    I, J, V = expected_csr(rows)
    A = gb.IJMatrix(I, J, V)
    L = gb.lib()
    for r in (0, 5, 2999):
        size = C.c_int()
        pc = C.POINTER(C.c_int)()
        pv = C.POINTER(C.c_double)()
        gb.check(L.HYPRE_ParCSRMatrixGetRow(A.par, r, C.byref(size), C.byref(pc), C.byref(pv)), "GetRow")
        got_c = np.ctypeslib.as_array(pc, (size.value,)).copy() if size.value else np.zeros(0, np.int32)
        got_v = np.ctypeslib.as_array(pv, (size.value,)).copy() if size.value else np.zeros(0)
        L.HYPRE_ParCSRMatrixRestoreRow(A.par, r, C.byref(size), C.byref(pc), C.byref(pv))
        np.testing.assert_array_equal(got_c, J[I[r]:I[r + 1]])
        np.testing.assert_array_equal(got_v, V[I[r]:I[r + 1]])
    A.destroy()


def test_ij_vector_puts_and_gets(gb):
    L = gb.lib()
    n = 10000
    rng = np.random.default_rng(12)
    a = rng.standard_normal(n)
    v = C.c_void_p()
    L.HYPRE_IJVectorCreate(0, 0, n - 1, C.byref(v))
    L.HYPRE_IJVectorSetObjectType(v, gb.HYPRE_PARCSR)
    L.HYPRE_IJVectorInitialize(v)
    L.HYPRE_IJVectorSetValues(v, n, None, a.ctypes.data)          # all values, in order
    L.HYPRE_IJVectorAssemble(v)
    out = np.zeros(n)
    L.HYPRE_IJVectorGetValues(v, n, None, out.ctypes.data)
    np.testing.assert_array_equal(out, a)
    # indexed puts and adds act on the current values
    idx = np.array([5, 17, 9999, 17], np.int32)
    add = np.array([1.0, 2.0, 3.0, 4.0])
    L.HYPRE_IJVectorAddToValues(v, 4, idx.ctypes.data, add.ctypes.data)
    exp = a.copy()
    for i, x in zip(idx, add):
        exp[i] += x
    got = np.zeros(3)
    gi = np.array([17, 5, 9999], np.int32)
    L.HYPRE_IJVectorGetValues(v, 3, gi.ctypes.data, got.ctypes.data)    # pending puts are visible
    np.testing.assert_array_equal(got, exp[gi])
    L.HYPRE_IJVectorAssemble(v)
    L.HYPRE_IJVectorGetValues(v, n, None, out.ctypes.data)
    np.testing.assert_array_equal(out, exp)
    # the device vector changed by the library (scaled through the ParVector)
    par = C.c_void_p()
    L.HYPRE_IJVectorGetObject(v, C.byref(par))
    L.HYPRE_ParVectorScale(2.0, par)
    one = np.array([3.0])
    L.HYPRE_IJVectorSetValues(v, 1, np.array([0], np.int32).ctypes.data, one.ctypes.data)
    L.HYPRE_IJVectorAssemble(v)
    L.HYPRE_IJVectorGetValues(v, n, None, out.ctypes.data)
    exp = 2.0 * exp
    exp[0] = 3.0
    np.testing.assert_array_equal(out, exp)
    assert L.HYPRE_GetError() == 0
    L.HYPRE_IJVectorDestroy(v)


def test_two_large_puts_in_permuted_row_order(gb):
    # rows staged on the device by two puts, not in row order: the general
    # assembly (per-row offsets) instead of the single in-order put's
    rows = random_rows(8000, seed=13)
    exp = expected_csr(rows)
    L = gb.lib()
    n = len(rows)
    h = C.c_void_p()
    L.HYPRE_IJMatrixCreate(0, 0, n - 1, 0, n - 1, C.byref(h))
    L.HYPRE_IJMatrixSetObjectType(h, gb.HYPRE_PARCSR)
    L.HYPRE_IJMatrixInitialize(h)
    perm = np.random.default_rng(14).permutation(n).astype(np.int32)
    for part in (perm[: n // 2], perm[n // 2:]):
        nc = np.array([len(rows[r][0]) for r in part], np.int32)
        J = np.array([c for r in part for c in rows[r][0]], np.int32)
        V = np.array([v for r in part for v in rows[r][1]], np.float64)
        assert len(J) >= 65536
        L.HYPRE_IJMatrixSetValues(h, len(part), nc.ctypes.data, part.ctypes.data, J.ctypes.data, V.ctypes.data)
    gb.check(L.HYPRE_IJMatrixAssemble(h), "assemble")
    par = C.c_void_p()
    L.HYPRE_IJMatrixGetObject(h, C.byref(par))
    same(gb.parcsr_to_host(par), exp)
    L.HYPRE_IJMatrixDestroy(h)
    assert L.HYPRE_GetError() == 0


def test_matrix_from_device_csr_matches_host_csr(gb):
    torch = pytest.importorskip("torch")
    rows = random_rows(3000, seed=15)
    I = np.zeros(len(rows) + 1, np.int32)
    I[1:] = np.cumsum([len(c) for c, _ in rows])
    J = np.array([c for cs, _ in rows for c in cs], np.int32)
    V = np.array([v for _, vs in rows for v in vs], np.float64)
    L = gb.lib()
    n = len(rows)
    Ah = C.c_void_p()
    gb.check(L.HYPRE_GB300_ParCSRMatrixCreateFromHostCSR(n, I.ctypes.data, J.ctypes.data, V.ctypes.data,
                                                         C.byref(Ah)), "host csr")
    dI = torch.from_numpy(I).cuda()
    dJ = torch.from_numpy(J).cuda()
    dV = torch.from_numpy(V).cuda()
    torch.cuda.synchronize()
    Ad = C.c_void_p()
    gb.check(L.HYPRE_GB300_ParCSRMatrixCreateFromDeviceCSR(n, dI.data_ptr(), dJ.data_ptr(), dV.data_ptr(),
                                                           C.byref(Ad)), "device csr")
    same(gb.parcsr_to_host(Ad), gb.parcsr_to_host(Ah))
    # the diagonal moved first with the entries before it shifted
    same(gb.parcsr_to_host(Ad), expected_csr(rows))
    L.HYPRE_GB300_ParCSRMatrixDestroy(Ad)
    L.HYPRE_GB300_ParCSRMatrixDestroy(Ah)


def test_row_counts_constant_values_and_vector_calls(gb, oracle_mod):
    """GetObjectType, GetRowCounts (rows outside the range count 0),
    SetConstantValues on the assembled matrix (the product then uses the
    constant; GetValues reads it back), and the IJ vector's constant values and
    inner product."""
    L = gb.lib()
    L.HYPRE_IJMatrixGetRowCounts.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    L.HYPRE_IJMatrixSetConstantValues.argtypes = [C.c_void_p, C.c_double]
    L.HYPRE_IJVectorSetConstantValues.argtypes = [C.c_void_p, C.c_double]
    L.HYPRE_IJVectorInnerProd.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
    L.HYPRE_ClearAllErrors()
    I, J, V = oracle_mod.stencil(7, 6, 5, 4)
    n = len(I) - 1
    A = gb.IJMatrix(I, J, V)
    t = C.c_int()
    gb.check(L.HYPRE_IJMatrixGetObjectType(A.h, C.byref(t)))
    assert t.value == gb.HYPRE_PARCSR
    rows = np.array([0, 7, n - 1, n, -1], np.int32)
    cnt = np.zeros(len(rows), np.int32)
    gb.check(L.HYPRE_IJMatrixGetRowCounts(A.h, len(rows), rows.ctypes.data, cnt.ctypes.data))
    lens = np.diff(I)
    assert list(cnt) == [lens[0], lens[7], lens[n - 1], 0, 0]
    gb.check(L.HYPRE_IJMatrixSetConstantValues(A.h, 0.5))
    x = np.random.default_rng(3).standard_normal(n)
    xv, yv = gb.IJVector(n, x), gb.IJVector(n, np.zeros(n))
    gb.check(L.HYPRE_ParCSRMatrixMatvec(1.0, A.par, xv.par, 0.0, yv.par))
    ref = np.array([0.5 * x[J[I[r]:I[r + 1]]].sum() for r in range(n)])
    np.testing.assert_allclose(yv.values(), ref, rtol=1e-14, atol=1e-14)
    ncols = np.array([2], np.int32)
    r = np.array([3], np.int32)
    cols = np.array(J[I[3]:I[3] + 2], np.int32)
    vals = np.zeros(2)
    gb.check(L.HYPRE_IJMatrixGetValues(A.h, 1, ncols.ctypes.data, r.ctypes.data, cols.ctypes.data,
                                       vals.ctypes.data))
    assert list(vals) == [0.5, 0.5]
    gb.check(L.HYPRE_IJVectorGetObjectType(xv.h, C.byref(t)))
    assert t.value == gb.HYPRE_PARCSR
    gb.check(L.HYPRE_IJVectorSetConstantValues(yv.h, 2.0))
    d = C.c_double()
    gb.check(L.HYPRE_IJVectorInnerProd(xv.h, yv.h, C.byref(d)))
    assert abs(d.value - 2.0 * x.sum()) <= 1e-12 * np.abs(x).sum() * 2
    for f in (L.HYPRE_IJMatrixSetMaxOffProcElmts, L.HYPRE_IJMatrixSetPrintLevel, L.HYPRE_IJMatrixSetOMPFlag):
        assert f(A.h, 1) == 0
    for f in (L.HYPRE_IJVectorSetMaxOffProcElmts, L.HYPRE_IJVectorSetPrintLevel):
        assert f(xv.h, 1) == 0
    A.destroy(); xv.destroy(); yv.destroy()
