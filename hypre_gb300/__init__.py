"""Python access to libHYPRE_gb300.so, the single-GPU (GB300) drop-in for the
reference library's IJ / ParCSR / BoomerAMG / PCG / FlexGMRES C API.

The product is the C ABI declared in include/HYPRE_gb300.h.  This module only
loads the shared library with ctypes and offers thin wrappers with the same
names and argument meaning (used by the tests and the benchmark).  There is
no CPU fallback: loading fails loudly if the library has not been built.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libHYPRE_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "HYPRE_gb300.h")

HYPRE_PARCSR = 5555
HYPRE_ERROR_GENERIC = 1
HYPRE_ERROR_MEMORY = 2
HYPRE_ERROR_ARG = 4
HYPRE_ERROR_CONV = 256

PREC_F64, PREC_F32, PREC_F16 = 0, 1, 2

_lib = None


def lib():
    """The loaded libHYPRE_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                "libHYPRE_gb300.so is not built: run `python -c \"import __graft_entry__ as g; g.build()\"`")
        L = C.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def _declare(L):
    vp, i32, f64 = C.c_void_p, C.c_int, C.c_double
    P = C.POINTER
    sig = {
        "HYPRE_Initialize": [], "HYPRE_Finalize": [], "HYPRE_GetError": [], "HYPRE_ClearAllErrors": [],
        "HYPRE_IJMatrixCreate": [i32, i32, i32, i32, i32, P(vp)],
        "HYPRE_IJMatrixSetObjectType": [vp, i32], "HYPRE_IJMatrixInitialize": [vp],
        "HYPRE_IJMatrixSetRowSizes": [vp, vp], "HYPRE_IJMatrixSetDiagOffdSizes": [vp, vp, vp],
        "HYPRE_IJMatrixSetValues": [vp, i32, vp, vp, vp, vp], "HYPRE_IJMatrixAddToValues": [vp, i32, vp, vp, vp, vp],
        "HYPRE_IJMatrixAssemble": [vp], "HYPRE_IJMatrixGetObject": [vp, P(vp)], "HYPRE_IJMatrixDestroy": [vp],
        "HYPRE_IJMatrixGetValues": [vp, i32, vp, vp, vp, vp],
        "HYPRE_IJVectorCreate": [i32, i32, i32, P(vp)], "HYPRE_IJVectorSetObjectType": [vp, i32],
        "HYPRE_IJVectorInitialize": [vp], "HYPRE_IJVectorSetValues": [vp, i32, vp, vp],
        "HYPRE_IJVectorAddToValues": [vp, i32, vp, vp], "HYPRE_IJVectorAssemble": [vp],
        "HYPRE_IJVectorGetObject": [vp, P(vp)], "HYPRE_IJVectorGetValues": [vp, i32, vp, vp],
        "HYPRE_IJVectorDestroy": [vp], "HYPRE_IJVectorGetLocalRange": [vp, P(i32), P(i32)],
        "HYPRE_IJMatrixRead": [C.c_char_p, i32, i32, P(vp)], "HYPRE_IJMatrixReadMM": [C.c_char_p, i32, i32, P(vp)],
        "HYPRE_IJMatrixReadBinary": [C.c_char_p, i32, i32, P(vp)],
        "HYPRE_IJMatrixPrint": [vp, C.c_char_p], "HYPRE_IJMatrixPrintBinary": [vp, C.c_char_p],
        "HYPRE_IJVectorRead": [C.c_char_p, i32, i32, P(vp)], "HYPRE_IJVectorReadBinary": [C.c_char_p, i32, i32, P(vp)],
        "HYPRE_IJVectorPrint": [vp, C.c_char_p], "HYPRE_IJVectorPrintBinary": [vp, C.c_char_p],
        "HYPRE_ParVectorCreate": [i32, i32, vp, P(vp)], "HYPRE_ParVectorInitialize": [vp],
        "HYPRE_ParVectorDestroy": [vp],
        "HYPRE_ParVectorInnerProd": [vp, vp, P(f64)], "HYPRE_ParVectorSetConstantValues": [vp, f64],
        "HYPRE_ParVectorCopy": [vp, vp], "HYPRE_ParVectorScale": [f64, vp], "HYPRE_ParVectorAxpy": [f64, vp, vp],
        "HYPRE_ParVectorSetRandomValues": [vp, i32],
        "HYPRE_ParCSRMatrixMatvec": [f64, vp, vp, f64, vp], "HYPRE_ParCSRMatrixMatvecT": [f64, vp, vp, f64, vp],
        "HYPRE_ParCSRMatrixMatmat": [vp, vp, P(vp)], "HYPRE_ParCSRMatrixDestroy": [vp],
        "HYPRE_BoomerAMGCreate": [P(vp)], "HYPRE_BoomerAMGDestroy": [vp],
        "HYPRE_BoomerAMGSetup": [vp, vp, vp, vp], "HYPRE_BoomerAMGSolve": [vp, vp, vp, vp],
        "HYPRE_BoomerAMGGetNumIterations": [vp, P(i32)], "HYPRE_BoomerAMGGetFinalRelativeResidualNorm": [vp, P(f64)],
        "HYPRE_BoomerAMGGetNumLevels": [vp, P(i32)],
        "HYPRE_ParCSRPCGCreate": [i32, P(vp)], "HYPRE_ParCSRPCGDestroy": [vp],
        "HYPRE_ParCSRPCGSetup": [vp, vp, vp, vp], "HYPRE_ParCSRPCGSolve": [vp, vp, vp, vp],
        "HYPRE_PCGSetPrecond": [vp, vp, vp, vp], "HYPRE_ParCSRPCGSetPrecond": [vp, vp, vp, vp],
        "HYPRE_PCGGetNumIterations": [vp, P(i32)], "HYPRE_PCGGetFinalRelativeResidualNorm": [vp, P(f64)],
        "HYPRE_ParCSRFlexGMRESCreate": [i32, P(vp)], "HYPRE_ParCSRFlexGMRESDestroy": [vp],
        "HYPRE_ParCSRFlexGMRESSetup": [vp, vp, vp, vp], "HYPRE_ParCSRFlexGMRESSolve": [vp, vp, vp, vp],
        "HYPRE_FlexGMRESSetPrecond": [vp, vp, vp, vp], "HYPRE_FlexGMRESGetNumIterations": [vp, P(i32)],
        "HYPRE_FlexGMRESGetFinalRelativeResidualNorm": [vp, P(f64)],
        "HYPRE_GB300_BoomerAMGGetLevelCSR": [vp, i32, i32, P(i32), P(i32), P(i32), vp, vp, vp],
        "HYPRE_GB300_ParCSRMatrixCopyToHostCSR": [vp, P(i32), P(i32), vp, vp, vp],
        "HYPRE_GB300_ParCSRMatrixCreateFromDeviceCSR": [i32, vp, vp, vp, P(vp)],
        "HYPRE_ParCSRMatrixGetRow": [vp, i32, P(i32), P(P(i32)), P(P(f64))],
        "HYPRE_ParCSRMatrixRestoreRow": [vp, i32, P(i32), P(P(i32)), P(P(f64))],
        "HYPRE_GB300_BoomerAMGGetLevelCF": [vp, i32, vp], "HYPRE_GB300_BoomerAMGGetLevelL1": [vp, i32, vp],
        "HYPRE_GB300_BoomerAMGGetLevelCheby": [vp, i32, vp, vp, vp],
        "HYPRE_GB300_KrylovGetResidualHistory": [vp, i32, vp, P(i32)],
        "HYPRE_GB300_ParVectorGetDevicePointer": [vp, P(vp), P(i32)],
        "HYPRE_GB300_ParVectorCopyFromHost": [vp, vp, i32], "HYPRE_GB300_ParVectorCopyToHost": [vp, vp, i32],
        "HYPRE_GB300_ParCSRMatrixCreateFromHostCSR": [i32, vp, vp, vp, P(vp)],
        "HYPRE_GB300_ParCSRMatrixDestroy": [vp],
        "HYPRE_GB300_SetStream": [vp], "HYPRE_GB300_GetStream": [P(vp)],
        "HYPRE_GB300_GetKernelLaunchCount": [P(C.c_longlong)], "HYPRE_GB300_ResetKernelLaunchCount": [],
        "HYPRE_GB300_BoomerAMGGetSetupTimes": [vp, vp, i32],
        "HYPRE_GB300_BoomerAMGSetCyclePrecision": [vp, i32], "HYPRE_GB300_BoomerAMGSetUseGraph": [vp, i32],
        "HYPRE_GB300_BoomerAMGSetSetupTables": [vp, i32],
        "HYPRE_GB300_BatchedPCGCreate": [P(vp)], "HYPRE_GB300_BatchedPCGDestroy": [vp],
        "HYPRE_GB300_BatchedPCGSetTol": [vp, f64], "HYPRE_GB300_BatchedPCGSetMaxIter": [vp, i32],
        "HYPRE_GB300_BatchedPCGSetCyclePrecision": [vp, i32],
        "HYPRE_GB300_BatchedPCGSetKernelShape": [vp, i32, i32], "HYPRE_GB300_BatchedPCGSetAutotune": [vp, i32],
        "HYPRE_GB300_BatchedPCGGetKernelShape": [vp, P(i32), P(i32)],
        "HYPRE_GB300_BatchedPCGGetTuningTimes": [vp, vp],
        "HYPRE_GB300_BatchedPCGSetup": [vp, vp, vp, i32, vp], "HYPRE_GB300_BatchedPCGSolve": [vp, vp, vp],
        "HYPRE_GB300_BatchedPCGGetNumIterations": [vp, vp],
        "HYPRE_GB300_BatchedPCGGetFinalRelativeResidualNorms": [vp, vp],
        "HYPRE_GB300_BatchedPCGGetResidualHistory": [vp, i32, i32, vp, P(i32)],
        "HYPRE_GB300_BatchedPCGGetLevelOffsets": [vp, i32, vp],
        "HYPRE_GB300_BatchedPCGGetOperatorComplexities": [vp, vp],
        "HYPRE_GB300_ParVectorCreateMulti": [i32, i32, P(vp)],
        "HYPRE_GB300_BoomerAMGGetSpGEMMStats": [vp, P(f64), P(f64), P(i32)],
        "HYPRE_GB300_BoomerAMGLevelSpMVTime": [vp, i32, i32, i32, P(f64), P(f64)],
        "HYPRE_GB300_SetAutotune": [i32],
        "HYPRE_GB300_ParCSRMatrixGetSpMVShape": [vp, i32, P(i32), P(i32), P(i32)],
        "HYPRE_GB300_ParCSRMatrixSetSpMVShape": [vp, i32, i32, i32],
        "HYPRE_GB300_KrylovGetMultiNumIterations": [vp, vp],
        "HYPRE_GB300_KrylovGetMultiFinalRelativeResidualNorms": [vp, vp],
        "HYPRE_GB300_KrylovGetMultiResidualHistory": [vp, i32, i32, vp, P(i32)],
        "HYPRE_GB300_MLPNumParams": [P(i32)], "HYPRE_GB300_BoomerAMGSetLearnedModel": [vp, vp],
        "HYPRE_GB300_BoomerAMGGetLearnedParams": [vp, P(f64), vp, i32],
        "HYPRE_GB300_MLPRowFeatures": [vp, vp], "HYPRE_GB300_MLPForward": [i32, vp, vp, vp],
        "HYPRE_GB300_MLPGradient": [i32, vp, vp, vp, vp, vp],
        "HYPRE_GB300_MLPAdamStep": [vp, vp, vp, vp, f64, i32],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = i32
    int_setters = ["MaxIter", "MaxCoarseSize", "MinCoarseSize", "MaxLevels", "CoarsenType", "AggNumLevels",
                   "NumPaths", "InterpType", "PMaxElmts", "AggInterpType", "AggPMaxElmts", "AggP12MaxElmts",
                   "CycleType", "FCycle", "NumSweeps", "RelaxType", "RelaxOrder", "ChebyOrder", "ChebyScale",
                   "ChebyVariant", "ChebyEigEst", "PrintLevel", "Logging", "RAP2", "ModuleRAP2", "KeepTranspose"]
    real_setters = ["Tol", "StrongThreshold", "MaxRowSum", "TruncFactor", "AggTruncFactor", "AggP12TruncFactor",
                    "RelaxWt", "OuterWt", "ChebyFraction"]
    for s in int_setters:
        fn = getattr(L, "HYPRE_BoomerAMGSet" + s)
        fn.argtypes = [vp, i32]
        fn.restype = i32
    for s in real_setters:
        fn = getattr(L, "HYPRE_BoomerAMGSet" + s)
        fn.argtypes = [vp, f64]
        fn.restype = i32
    for s, t in [("CycleRelaxType", i32), ("CycleNumSweeps", i32)]:
        fn = getattr(L, "HYPRE_BoomerAMGSet" + s)
        fn.argtypes = [vp, t, i32]
        fn.restype = i32
    L.HYPRE_BoomerAMGSetLevelRelaxWt.argtypes = [vp, f64, i32]
    for pre in ("HYPRE_PCG", "HYPRE_FlexGMRES"):
        for s, t in [("Tol", f64), ("AbsoluteTol", f64), ("MaxIter", i32), ("PrintLevel", i32), ("Logging", i32)]:
            fn = getattr(L, pre + "Set" + s)
            fn.argtypes = [vp, t]
            fn.restype = i32
    for s in ("TwoNorm", "RelChange", "RecomputeResidual"):
        fn = getattr(L, "HYPRE_PCGSet" + s)
        fn.argtypes = [vp, i32]
    L.HYPRE_FlexGMRESSetKDim.argtypes = [vp, i32]


def header_symbols():
    """Every function name declared in include/HYPRE_gb300.h."""
    import re
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:HYPRE_Int|void)\s+(HYPRE_\w+)\s*\(", txt, re.M)))


def fn_ptr(name):
    return C.cast(getattr(lib(), name), C.c_void_p)


def check(code, what=""):
    if code & ~HYPRE_ERROR_CONV:
        raise RuntimeError(f"{what}: hypre error flag {code}")
    return code


# ---------------------------------------------------------------------------
# Thin object wrappers (same calls a C user makes)
# ---------------------------------------------------------------------------
def parcsr_to_host(par):
    """A ParCSR matrix's local CSR arrays copied to host memory."""
    L = lib()
    nr, nnz = C.c_int(), C.c_int()
    check(L.HYPRE_GB300_ParCSRMatrixCopyToHostCSR(par, C.byref(nr), C.byref(nnz), None, None, None), "CopyToHostCSR")
    I = np.empty(nr.value + 1, np.int32)
    J = np.empty(max(nnz.value, 1), np.int32)
    V = np.empty(max(nnz.value, 1), np.float64)
    check(L.HYPRE_GB300_ParCSRMatrixCopyToHostCSR(par, None, None, I.ctypes.data, J.ctypes.data, V.ctypes.data),
          "CopyToHostCSR")
    return I, J[:nnz.value], V[:nnz.value]


def matmat(A, B):
    """C = A*B (HYPRE_ParCSRMatrixMatmat) of two ParCSR handles; returns C's
    handle, which the caller destroys (HYPRE_ParCSRMatrixDestroy)."""
    Cp = C.c_void_p()
    check(lib().HYPRE_ParCSRMatrixMatmat(A, B, C.byref(Cp)), "Matmat")
    return Cp


class IJMatrix:
    """HYPRE_IJMatrix assembled from host CSR arrays, one SetValues call per
    row (the diagonal is moved to the front of each row at assembly)."""

    def __init__(self, I, J, V, set_row_sizes=True):
        L = lib()
        L.HYPRE_Initialize()
        I = np.ascontiguousarray(I, np.int32)
        J = np.ascontiguousarray(J, np.int32)
        V = np.ascontiguousarray(V, np.float64)
        n = len(I) - 1
        self.n = n
        self.h = C.c_void_p()
        check(L.HYPRE_IJMatrixCreate(0, 0, n - 1, 0, n - 1, C.byref(self.h)), "IJMatrixCreate")
        L.HYPRE_IJMatrixSetObjectType(self.h, HYPRE_PARCSR)
        ncols = np.diff(I).astype(np.int32)
        if set_row_sizes:
            L.HYPRE_IJMatrixSetRowSizes(self.h, ncols.ctypes.data)
        L.HYPRE_IJMatrixInitialize(self.h)
        rows = np.arange(n, dtype=np.int32)
        # all rows in one call: ncols per row, rows, concatenated cols/values
        check(L.HYPRE_IJMatrixSetValues(self.h, n, ncols.ctypes.data, rows.ctypes.data, J.ctypes.data,
                                        V.ctypes.data), "IJMatrixSetValues")
        check(L.HYPRE_IJMatrixAssemble(self.h), "IJMatrixAssemble")
        self.par = C.c_void_p()
        L.HYPRE_IJMatrixGetObject(self.h, C.byref(self.par))

    def csr(self):
        """The assembled matrix as host CSR arrays (I, J, V)."""
        return parcsr_to_host(self.par)

    def destroy(self):
        if self.h:
            lib().HYPRE_IJMatrixDestroy(self.h)
            self.h = None


class DeviceMatrix:
    """ParCSR matrix built by the library from CSR arrays in device memory
    (objects with ``data_ptr()``, e.g. CUDA tensors; int32 row pointers and
    columns, float64 values).  The arrays are copied; the diagonal is moved to
    the front of each row."""

    def __init__(self, dI, dJ, dV):
        L = lib()
        self.n = int(dI.numel()) - 1
        self.par = C.c_void_p()
        check(L.HYPRE_GB300_ParCSRMatrixCreateFromDeviceCSR(self.n, dI.data_ptr(), dJ.data_ptr(), dV.data_ptr(),
                                                            C.byref(self.par)), "CreateFromDeviceCSR")

    def csr(self):
        return parcsr_to_host(self.par)

    def destroy(self):
        if self.par:
            lib().HYPRE_GB300_ParCSRMatrixDestroy(self.par)
            self.par = None


class IJVector:
    def __init__(self, n, values=None):
        L = lib()
        self.n = n
        self.h = C.c_void_p()
        L.HYPRE_IJVectorCreate(0, 0, n - 1, C.byref(self.h))
        L.HYPRE_IJVectorSetObjectType(self.h, HYPRE_PARCSR)
        L.HYPRE_IJVectorInitialize(self.h)
        if values is not None:
            v = np.ascontiguousarray(values, np.float64)
            L.HYPRE_IJVectorSetValues(self.h, n, None, v.ctypes.data)
        L.HYPRE_IJVectorAssemble(self.h)
        self.par = C.c_void_p()
        L.HYPRE_IJVectorGetObject(self.h, C.byref(self.par))

    def values(self):
        out = np.empty(self.n)
        lib().HYPRE_IJVectorGetValues(self.h, self.n, None, out.ctypes.data)
        return out

    def set(self, values):
        v = np.ascontiguousarray(values, np.float64)
        lib().HYPRE_GB300_ParVectorCopyFromHost(self.par, v.ctypes.data, self.n)

    def destroy(self):
        if self.h:
            lib().HYPRE_IJVectorDestroy(self.h)
            self.h = None


class BoomerAMG:
    def __init__(self, **params):
        L = lib()
        self.h = C.c_void_p()
        check(L.HYPRE_BoomerAMGCreate(C.byref(self.h)), "BoomerAMGCreate")
        for k, v in params.items():
            self.set(k, v)

    def set(self, name, value):
        L = lib()
        if name == "CycleRelaxType":
            # (type, part), or a list of them
            for t, k in (value if isinstance(value, list) else [value]):
                r = L.HYPRE_BoomerAMGSetCycleRelaxType(self.h, t, k)
            return r
        if name == "CycleNumSweeps":
            return L.HYPRE_BoomerAMGSetCycleNumSweeps(self.h, value[0], value[1])
        if name == "CyclePrecision":
            return L.HYPRE_GB300_BoomerAMGSetCyclePrecision(self.h, value)
        if name == "UseGraph":
            return L.HYPRE_GB300_BoomerAMGSetUseGraph(self.h, value)
        if name == "SetupTables":
            return L.HYPRE_GB300_BoomerAMGSetSetupTables(self.h, value)
        return getattr(L, "HYPRE_BoomerAMGSet" + name)(self.h, value)

    def num_levels(self):
        n = C.c_int()
        lib().HYPRE_BoomerAMGGetNumLevels(self.h, C.byref(n))
        return n.value

    def level_csr(self, level, which):
        L = lib()
        code = {"A": 0, "P": 1, "S": 2}[which]
        nr, nc, nnz = C.c_int(), C.c_int(), C.c_int()
        L.HYPRE_GB300_BoomerAMGGetLevelCSR(self.h, level, code, C.byref(nr), C.byref(nc), C.byref(nnz),
                                           None, None, None)
        I = np.empty(nr.value + 1, np.int32)
        J = np.empty(max(nnz.value, 1), np.int32)
        V = np.empty(max(nnz.value, 1), np.float64)
        L.HYPRE_GB300_BoomerAMGGetLevelCSR(self.h, level, code, C.byref(nr), C.byref(nc), C.byref(nnz),
                                           I.ctypes.data, J.ctypes.data, V.ctypes.data if which != "S" else None)
        return I, J[: nnz.value], (V[: nnz.value] if which != "S" else None), nc.value

    def level_cf(self, level, n):
        out = np.empty(n, np.int32)
        lib().HYPRE_GB300_BoomerAMGGetLevelCF(self.h, level, out.ctypes.data)
        return out

    def level_l1(self, level, n):
        out = np.empty(n, np.float64)
        lib().HYPRE_GB300_BoomerAMGGetLevelL1(self.h, level, out.ctypes.data)
        return out

    def level_cheby(self, level, n, order):
        """(coefficients, (max_eig, min_eig), D^{-1/2}) of a level's Chebyshev smoother."""
        order = min(max(order, 1), 4)
        c = np.zeros(order)
        e = np.zeros(2)
        ds = np.empty(n, np.float64)
        check(lib().HYPRE_GB300_BoomerAMGGetLevelCheby(self.h, level, c.ctypes.data, e.ctypes.data, ds.ctypes.data))
        return c, (float(e[0]), float(e[1])), ds

    def setup_times(self):
        t = np.zeros(6)
        lib().HYPRE_GB300_BoomerAMGGetSetupTimes(self.h, t.ctypes.data, 6)
        return t

    def destroy(self):
        if self.h:
            lib().HYPRE_BoomerAMGDestroy(self.h)
            self.h = None


class Krylov:
    """HYPRE_ParCSRPCG or HYPRE_ParCSRFlexGMRES preconditioned by BoomerAMG
    (HYPRE_BoomerAMGSolve / HYPRE_BoomerAMGSetup passed as function pointers,
    as in the reference's drivers)."""

    def __init__(self, kind="pcg", tol=1e-8, maxit=100, kdim=30, amg=None, two_norm=1, rel_change=0):
        L = lib()
        self.kind = kind
        self.h = C.c_void_p()
        if kind == "pcg":
            check(L.HYPRE_ParCSRPCGCreate(0, C.byref(self.h)), "PCGCreate")
            L.HYPRE_PCGSetTol(self.h, tol)
            L.HYPRE_PCGSetMaxIter(self.h, maxit)
            L.HYPRE_PCGSetTwoNorm(self.h, two_norm)
            L.HYPRE_PCGSetRelChange(self.h, rel_change)
            L.HYPRE_PCGSetLogging(self.h, 1)
            if amg is not None:
                L.HYPRE_PCGSetPrecond(self.h, fn_ptr("HYPRE_BoomerAMGSolve"), fn_ptr("HYPRE_BoomerAMGSetup"), amg.h)
        else:
            check(L.HYPRE_ParCSRFlexGMRESCreate(0, C.byref(self.h)), "FlexGMRESCreate")
            L.HYPRE_FlexGMRESSetKDim(self.h, kdim)
            L.HYPRE_FlexGMRESSetTol(self.h, tol)
            L.HYPRE_FlexGMRESSetMaxIter(self.h, maxit)
            L.HYPRE_FlexGMRESSetLogging(self.h, 1)
            if amg is not None:
                L.HYPRE_FlexGMRESSetPrecond(self.h, fn_ptr("HYPRE_BoomerAMGSolve"),
                                            fn_ptr("HYPRE_BoomerAMGSetup"), amg.h)

    def setup(self, A, b, x):
        L = lib()
        f = L.HYPRE_ParCSRPCGSetup if self.kind == "pcg" else L.HYPRE_ParCSRFlexGMRESSetup
        return check(f(self.h, A.par, b.par, x.par), "KrylovSetup")

    def solve(self, A, b, x):
        L = lib()
        f = L.HYPRE_ParCSRPCGSolve if self.kind == "pcg" else L.HYPRE_ParCSRFlexGMRESSolve
        return check(f(self.h, A.par, b.par, x.par), "KrylovSolve")

    def iterations(self):
        n = C.c_int()
        L = lib()
        (L.HYPRE_PCGGetNumIterations if self.kind == "pcg" else L.HYPRE_FlexGMRESGetNumIterations)(
            self.h, C.byref(n))
        return n.value

    def final_relres(self):
        r = C.c_double()
        L = lib()
        (L.HYPRE_PCGGetFinalRelativeResidualNorm if self.kind == "pcg"
         else L.HYPRE_FlexGMRESGetFinalRelativeResidualNorm)(self.h, C.byref(r))
        return r.value

    def history(self):
        n = C.c_int()
        L = lib()
        L.HYPRE_GB300_KrylovGetResidualHistory(self.h, 0, None, C.byref(n))
        out = np.empty(max(n.value, 1))
        L.HYPRE_GB300_KrylovGetResidualHistory(self.h, n.value, out.ctypes.data, C.byref(n))
        return out[: n.value]

    def destroy(self):
        if self.h:
            L = lib()
            (L.HYPRE_ParCSRPCGDestroy if self.kind == "pcg" else L.HYPRE_ParCSRFlexGMRESDestroy)(self.h)
            self.h = None


def kernel_launches():
    c = C.c_longlong()
    lib().HYPRE_GB300_GetKernelLaunchCount(C.byref(c))
    return c.value


class BatchedPCG:
    """HYPRE_GB300_BatchedPCG*: independent systems (diagonal blocks of one
    matrix) solved by FP64 PCG with a BoomerAMG V-cycle, one persistent launch."""

    def __init__(self, amg, tol=1e-8, maxit=100, prec=1, shape=None):
        L = lib()
        self.amg = amg
        self.h = C.c_void_p()
        check(L.HYPRE_GB300_BatchedPCGCreate(C.byref(self.h)), "BatchedPCGCreate")
        L.HYPRE_GB300_BatchedPCGSetTol(self.h, tol)
        L.HYPRE_GB300_BatchedPCGSetMaxIter(self.h, maxit)
        L.HYPRE_GB300_BatchedPCGSetCyclePrecision(self.h, prec)
        self.maxit = maxit
        if shape is not None:
            check(L.HYPRE_GB300_BatchedPCGSetKernelShape(self.h, shape[0], shape[1]), "shape")

    def setup(self, A, offsets):
        self.off = np.ascontiguousarray(offsets, np.int32)
        self.nsys = len(self.off) - 1
        check(lib().HYPRE_GB300_BatchedPCGSetup(self.h, self.amg.h, A.par, self.nsys, self.off.ctypes.data),
              "BatchedPCGSetup")

    def solve(self, b, x):
        return lib().HYPRE_GB300_BatchedPCGSolve(self.h, b.par, x.par)

    def iterations(self):
        out = np.zeros(self.nsys, np.int32)
        lib().HYPRE_GB300_BatchedPCGGetNumIterations(self.h, out.ctypes.data)
        return out

    def relres(self):
        out = np.zeros(self.nsys)
        lib().HYPRE_GB300_BatchedPCGGetFinalRelativeResidualNorms(self.h, out.ctypes.data)
        return out

    def history(self, s):
        out = np.zeros(self.maxit + 1)
        n = C.c_int()
        lib().HYPRE_GB300_BatchedPCGGetResidualHistory(self.h, s, self.maxit + 1, out.ctypes.data, C.byref(n))
        return out[: n.value]

    def level_offsets(self, level):
        out = np.zeros(self.nsys + 1, np.int32)
        check(lib().HYPRE_GB300_BatchedPCGGetLevelOffsets(self.h, level, out.ctypes.data), "offsets")
        return out

    def complexities(self):
        out = np.zeros(self.nsys)
        check(lib().HYPRE_GB300_BatchedPCGGetOperatorComplexities(self.h, out.ctypes.data), "complexities")
        return out

    def shape(self):
        a, b = C.c_int(), C.c_int()
        lib().HYPRE_GB300_BatchedPCGGetKernelShape(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def tuning_times(self):
        out = np.zeros(12)
        lib().HYPRE_GB300_BatchedPCGGetTuningTimes(self.h, out.ctypes.data)
        return out.reshape(4, 3)

    def __del__(self):
        if getattr(self, "h", None):
            lib().HYPRE_GB300_BatchedPCGDestroy(self.h)
            self.h = None


class MultiVector:
    """HYPRE_GB300_ParVectorCreateMulti: n x nv values, interleaved by row."""

    def __init__(self, values):
        values = np.ascontiguousarray(values, np.float64)
        self.n, self.nv = values.shape
        self.par = C.c_void_p()
        check(lib().HYPRE_GB300_ParVectorCreateMulti(self.n, self.nv, C.byref(self.par)), "CreateMulti")
        self.set(values)

    def set(self, values):
        v = np.ascontiguousarray(values, np.float64)
        check(lib().HYPRE_GB300_ParVectorCopyFromHost(self.par, v.ctypes.data, self.n * self.nv), "copy")

    def values(self):
        out = np.empty((self.n, self.nv))
        check(lib().HYPRE_GB300_ParVectorCopyToHost(self.par, out.ctypes.data, self.n * self.nv), "copy")
        return out

    def __del__(self):
        if getattr(self, "par", None):
            lib().HYPRE_ParVectorDestroy(self.par)
            self.par = None


def multi_results(krylov, nv, maxit):
    """Per-column iterations, final relative residuals and histories of a
    multi-vector PCG solve."""
    L = lib()
    its = np.zeros(nv, np.int32)
    rel = np.zeros(nv)
    L.HYPRE_GB300_KrylovGetMultiNumIterations(krylov.h, its.ctypes.data)
    L.HYPRE_GB300_KrylovGetMultiFinalRelativeResidualNorms(krylov.h, rel.ctypes.data)
    hist = []
    for c in range(nv):
        h = np.zeros(maxit + 1)
        m = C.c_int()
        L.HYPRE_GB300_KrylovGetMultiResidualHistory(krylov.h, c, maxit + 1, h.ctypes.data, C.byref(m))
        hist.append(h[: m.value])
    return its, rel, hist
