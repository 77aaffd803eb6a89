"""ctypes wrapper around the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the parity checker / timed CPU baseline.  The
product library (hypre_gb300) never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


class Params(C.Structure):
    """Mirror of or_amg_params in oracle/amg_oracle.h."""
    _fields_ = [
        ("strong_threshold", C.c_double), ("max_row_sum", C.c_double), ("trunc_factor", C.c_double),
        ("p_max_elmts", C.c_int), ("interp_type", C.c_int), ("coarsen_type", C.c_int),
        ("agg_num_levels", C.c_int), ("agg_interp_type", C.c_int), ("agg_p_max_elmts", C.c_int),
        ("agg_p12_max_elmts", C.c_int), ("agg_trunc_factor", C.c_double), ("agg_p12_trunc_factor", C.c_double),
        ("num_paths", C.c_int), ("max_levels", C.c_int), ("max_coarse_size", C.c_int), ("min_coarse_size", C.c_int),
        ("relax_down", C.c_int), ("relax_up", C.c_int), ("relax_coarse", C.c_int), ("num_sweeps", C.c_int),
        ("relax_weight", C.c_double), ("cheby_order", C.c_int), ("cheby_fraction", C.c_double),
        ("cheby_scale", C.c_int), ("cheby_variant", C.c_int), ("cheby_eig_est", C.c_int),
        ("relax_order", C.c_int), ("cycle_type", C.c_int), ("fcycle", C.c_int), ("pcg_rel_change", C.c_int),
        ("outer_weight", C.c_double),
    ]


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        L.or_h_new.restype = C.c_void_p
        L.or_h_delete.argtypes = [C.c_void_p]
        L.or_h_num_levels.argtypes = [C.c_void_p]
        L.or_h_csr.argtypes = [C.c_void_p, C.c_int, C.c_int, P(C.c_int), P(C.c_int),
                               P(P(C.c_int)), P(P(C.c_int)), P(P(C.c_double))]
        L.or_h_cf.argtypes = [C.c_void_p, C.c_int]
        L.or_h_cf.restype = P(C.c_int)
        L.or_h_l1.argtypes = [C.c_void_p, C.c_int]
        L.or_h_l1.restype = P(C.c_double)
        for nm in ("or_h_cheby_coefs", "or_h_cheby_ds"):
            getattr(L, nm).argtypes = [C.c_void_p, C.c_int]
            getattr(L, nm).restype = P(C.c_double)
        L.or_h_cheby_eig.argtypes = [C.c_void_p]
        L.or_h_cheby_eig.restype = P(C.c_double)
        L.or_eig_tridiag.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
        L.or_max_eig_cg.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                    P(C.c_double), P(C.c_double)]
        L.or_setup_flat.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, P(Params), C.c_void_p]
        L.or_pcg_flat.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_double, C.c_int, C.c_void_p, P(C.c_int)]
        L.or_fgmres_flat.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_double, C.c_int, C.c_int, C.c_void_p, P(C.c_int)]
        L.or_vcycle_flat.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.or_amg_solve_flat.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_double, C.c_int, C.c_void_p, C.c_void_p]
        L.or_default_params.argtypes = [P(Params)]
        L.or_set_threads.argtypes = [C.c_int]
        L.or_rand_uniform.argtypes = [C.c_int, C.c_int, C.c_void_p]
        L.or_gen_stencil_flat.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int,
                                          P(P(C.c_int)), P(P(C.c_int)), P(P(C.c_double))]
        L.or_free_ptr.argtypes = [C.c_void_p]
        L.or_matmat_flat.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 6 + \
            [P(P(C.c_int)), P(P(C.c_int)), P(P(C.c_double))]
        _lib = L
    return _lib


def default_params(**kw):
    p = Params()
    lib().or_default_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def set_threads(n):
    lib().or_set_threads(int(n))


def rand_uniform(n, seed):
    out = np.empty(n, dtype=np.float64)
    lib().or_rand_uniform(int(n), int(seed), out.ctypes.data)
    return out


def rhs_normalised(n, seed=22775):
    """b = 2*PM-1 (seeded), scaled to unit 2-norm with a sequential dot product."""
    b = rand_uniform(n, seed)
    s = 0.0
    for v in b.tolist():
        s += v * v
    return b * (1.0 / np.sqrt(s))


def stencil(kind, nx, ny, nz):
    L = lib()
    pi, pj, pv = C.POINTER(C.c_int)(), C.POINTER(C.c_int)(), C.POINTER(C.c_double)()
    nnz = L.or_gen_stencil_flat(kind, nx, ny, nz, C.byref(pi), C.byref(pj), C.byref(pv))
    n = nx * ny * nz
    I = np.ctypeslib.as_array(pi, (n + 1,)).copy()
    J = np.ctypeslib.as_array(pj, (nnz,)).copy()
    V = np.ctypeslib.as_array(pv, (nnz,)).copy()
    for p in (pi, pj, pv):
        L.or_free_ptr(C.cast(p, C.c_void_p))
    return I, J, V


def matmat(A, B, nca, ncb):
    """C = A*B as the reference's HYPRE_ParCSRMatrixMatmat computes it on one
    process (column order, summation order, diagonal rule); A and B are
    (I, J, V) CSR triples with nca and ncb columns."""
    L = lib()
    (Ai, Aj, Av), (Bi, Bj, Bv) = [(np.ascontiguousarray(I, np.int32), np.ascontiguousarray(J, np.int32),
                                   np.ascontiguousarray(V, np.float64)) for I, J, V in (A, B)]
    nra = len(Ai) - 1
    pi, pj, pv = C.POINTER(C.c_int)(), C.POINTER(C.c_int)(), C.POINTER(C.c_double)()
    nnz = L.or_matmat_flat(nra, nca, ncb, Ai.ctypes.data, Aj.ctypes.data, Av.ctypes.data, Bi.ctypes.data,
                           Bj.ctypes.data, Bv.ctypes.data, C.byref(pi), C.byref(pj), C.byref(pv))
    I = np.ctypeslib.as_array(pi, (nra + 1,)).copy()
    J = np.ctypeslib.as_array(pj, (max(nnz, 1),))[:nnz].copy()
    V = np.ctypeslib.as_array(pv, (max(nnz, 1),))[:nnz].copy()
    for p in (pi, pj, pv):
        L.or_free_ptr(C.cast(p, C.c_void_p))
    return I, J, V


class Hierarchy:
    """Oracle AMG hierarchy for a CSR matrix (I, J, V: int32/int32/float64)."""

    def __init__(self, I, J, V, params):
        L = lib()
        self.I = np.ascontiguousarray(I, dtype=np.int32)
        self.J = np.ascontiguousarray(J, dtype=np.int32)
        self.V = np.ascontiguousarray(V, dtype=np.float64)
        self.n = len(self.I) - 1
        self.h = L.or_h_new()
        L.or_setup_flat(self.n, self.I.ctypes.data, self.J.ctypes.data, self.V.ctypes.data,
                        C.byref(params), self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_h_delete(self.h)
            self.h = None

    @property
    def num_levels(self):
        return lib().or_h_num_levels(self.h)

    def csr(self, which, level):
        L = lib()
        nr, nc = C.c_int(), C.c_int()
        pi, pj, pv = C.POINTER(C.c_int)(), C.POINTER(C.c_int)(), C.POINTER(C.c_double)()
        code = {"A": 0, "P": 1, "S": 2}[which]
        nnz = L.or_h_csr(self.h, code, level, C.byref(nr), C.byref(nc), C.byref(pi), C.byref(pj), C.byref(pv))
        I = np.ctypeslib.as_array(pi, (nr.value + 1,)).copy()
        J = np.ctypeslib.as_array(pj, (nnz,)).copy() if nnz else np.zeros(0, np.int32)
        V = np.ctypeslib.as_array(pv, (nnz,)).copy() if (nnz and bool(pv)) else None
        return I, J, V, nc.value

    def cf(self, level):
        n = self.csr("A", level)[0].shape[0] - 1
        return np.ctypeslib.as_array(lib().or_h_cf(self.h, level), (n,)).copy()

    def l1(self, level):
        n = self.csr("A", level)[0].shape[0] - 1
        return np.ctypeslib.as_array(lib().or_h_l1(self.h, level), (n,)).copy()

    def cheby(self, level, order):
        """(coefficients, (max_eig, min_eig), D^{-1/2} scaling) of a level, or None."""
        L = lib()
        pc = L.or_h_cheby_coefs(self.h, level)
        if not pc:
            return None
        n = self.csr("A", level)[0].shape[0] - 1
        order = min(max(order, 1), 4)
        coefs = np.ctypeslib.as_array(pc, (order,)).copy()
        ds = np.ctypeslib.as_array(L.or_h_cheby_ds(self.h, level), (n,)).copy()
        eig = np.ctypeslib.as_array(L.or_h_cheby_eig(self.h), (2 * self.num_levels,))
        return coefs, (float(eig[2 * level]), float(eig[2 * level + 1])), ds

    def pcg(self, b, tol=1e-8, maxit=100):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.n)
        rel = np.zeros(maxit + 1)
        it = C.c_int()
        lib().or_pcg_flat(self.n, self.I.ctypes.data, self.J.ctypes.data, self.V.ctypes.data, self.h,
                          b.ctypes.data, x.ctypes.data, tol, maxit, rel.ctypes.data, C.byref(it))
        return x, rel[: it.value + 1], it.value

    def fgmres(self, b, tol=1e-8, maxit=100, kdim=30):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.n)
        res = np.zeros(maxit + 1)
        it = C.c_int()
        lib().or_fgmres_flat(self.n, self.I.ctypes.data, self.J.ctypes.data, self.V.ctypes.data, self.h,
                             b.ctypes.data, x.ctypes.data, tol, maxit, kdim, res.ctypes.data, C.byref(it))
        return x, res[: it.value + 1], it.value

    def amg_solve(self, b, tol=1e-8, maxit=100):
        """BoomerAMG as the solver from x = 0: (x, relative residuals, cycles)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.n)
        rel = np.zeros(maxit + 1)
        it = C.c_int()
        lib().or_amg_solve_flat(self.n, self.I.ctypes.data, self.J.ctypes.data, self.V.ctypes.data, self.h,
                                b.ctypes.data, x.ctypes.data, tol, maxit, rel.ctypes.data, C.byref(it))
        return x, rel[: it.value + 1], it.value

    def vcycle(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64)
        u = np.zeros(self.n)
        lib().or_vcycle_flat(self.h, f.ctypes.data, u.ctypes.data)
        return u


def eig_tridiag(d, e):
    """Eigenvalues (ascending) of the symmetric tridiagonal (d, e[1:]) by TQL1."""
    d = np.ascontiguousarray(d, dtype=np.float64).copy()
    e = np.ascontiguousarray(e, dtype=np.float64).copy()
    err = lib().or_eig_tridiag(len(d), d.ctypes.data, e.ctypes.data)
    if err:
        raise RuntimeError("tridiagonal QL did not converge")
    return d


def read_records(path):
    """Reads a record file written by oracle/ref/amg_ref_dump.c."""
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    off = 0
    while off < len(data):
        name = data[off:off + 32].split(b"\0", 1)[0].decode()
        dt = np.frombuffer(data, np.int32, 1, off + 32)[0]
        cnt = int(np.frombuffer(data, np.int64, 1, off + 36)[0])
        off += 44
        if dt == 0:
            out[name] = np.frombuffer(data, np.int32, cnt, off).copy()
            off += 4 * cnt
        else:
            out[name] = np.frombuffer(data, np.float64, cnt, off).copy()
            off += 8 * cnt
    return out
