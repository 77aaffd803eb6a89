"""GPU test of the transpose mat-vec that allocates nothing
(HYPRE_GB300_ParCSRMatrixMatvecTNoAlloc), called through the C ABI.

Callers that cannot let the library allocate device memory -- code enqueuing
work while a stream is captured into a CUDA graph, or a host framework that
owns all device memory -- use this entry point; its transpose lives in a fixed
32 MiB device array.  Its result must match the allocating
HYPRE_ParCSRMatrixMatvecT on two calls in a row (the array keeps the previous
call's contents, which must not leak into the next result), the two calls must
neither draw on the stream-ordered pool nor change the device's free memory,
and a matrix too large for the array, or a vector of the wrong length, must be
rejected with an argument error.  This file is collected last so a failure
here comes after every other test has run."""
import ctypes as C
import ctypes.util
import glob
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-13
USED_MEM_CURRENT, USED_MEM_HIGH, RESERVED_MEM_CURRENT = 7, 8, 5   # cudaMemPoolAttr values (driver_types.h)


def _vec(gb, v):
    return gb.IJVector(len(v), v)


def _cudart():
    """The CUDA runtime as a shared library, to read the device's default
    memory pool (the pool the library's stream-ordered allocations draw on)."""
    cands = [ctypes.util.find_library("cudart")]
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cands += sorted(glob.glob(os.path.join(home, "lib64", "libcudart.so*")))
    for c in cands:
        if c:
            try:
                return C.CDLL(c)
            except OSError:
                continue
    pytest.skip("no shared CUDA runtime to read the memory pool")


class _Pool:
    def __init__(self):
        self.rt = _cudart()
        dev = C.c_int()
        assert self.rt.cudaGetDevice(C.byref(dev)) == 0
        self.pool = C.c_void_p()
        assert self.rt.cudaDeviceGetDefaultMemPool(C.byref(self.pool), dev) == 0

    def attr(self, a):
        v = C.c_uint64()
        assert self.rt.cudaMemPoolGetAttribute(self.pool, a, C.byref(v)) == 0
        return v.value

    def reset_high(self):
        z = C.c_uint64(0)
        assert self.rt.cudaMemPoolSetAttribute(self.pool, USED_MEM_HIGH, C.byref(z)) == 0

    def free_bytes(self):
        f, t = C.c_size_t(), C.c_size_t()
        assert self.rt.cudaMemGetInfo(C.byref(f), C.byref(t)) == 0
        return f.value

    def sync(self):
        assert self.rt.cudaDeviceSynchronize() == 0


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
    cases = []
    for alpha, beta, seed in ((1.0, 0.0, 1), (-0.7, 1.3, 2)):
        r = np.random.default_rng(seed)
        x, y0 = r.standard_normal(n), r.standard_normal(n)
        xv, y_ref, y_na = _vec(gb, x), _vec(gb, y0), _vec(gb, y0)
        assert L.HYPRE_ParCSRMatrixMatvecT(alpha, A.par, xv.par, beta, y_ref.par) == 0
        cases.append((alpha, beta, xv, y_ref, y_na))
    # the first call on this device looks up the array; a warm-up pass with
    # the same arguments also loads every kernel the calls use, so the two
    # calls checked below run back to back on loaded code
    warm = [_vec(gb, np.zeros(n)) for _ in cases]
    for (alpha, beta, xv, _, _), w in zip(cases, warm):
        assert L.HYPRE_GB300_ParCSRMatrixMatvecTNoAlloc(alpha, A.par, xv.par, beta, w.par) == 0
    pool = _Pool()
    pool.sync()
    used0, reserved0, free0 = pool.attr(USED_MEM_CURRENT), pool.attr(RESERVED_MEM_CURRENT), pool.free_bytes()
    pool.reset_high()
    for call, (alpha, beta, xv, _, y_na) in enumerate(cases):
        assert L.HYPRE_GB300_ParCSRMatrixMatvecTNoAlloc(alpha, A.par, xv.par, beta, y_na.par) == 0, f"call {call}"
    pool.sync()
    assert pool.attr(USED_MEM_HIGH) == used0, "the no-alloc calls drew on the stream-ordered pool"
    assert pool.attr(RESERVED_MEM_CURRENT) == reserved0
    assert pool.free_bytes() == free0, "device memory changed during the no-alloc calls"
    for call, (alpha, beta, xv, y_ref, y_na) in enumerate(cases):
        ref, got = y_ref.values(), y_na.values()
        np.testing.assert_allclose(got, ref, rtol=RTOL, atol=RTOL * np.abs(ref).max(), err_msg=f"call {call}")
    for _, _, xv, y_ref, y_na in cases:
        for v in (xv, y_ref, y_na):
            v.destroy()
    for w in warm:
        w.destroy()
    A.destroy()


def test_no_alloc_matvecT_rejects_bad_arguments(gb):
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
    short = _vec(gb, np.zeros(n - 1))
    err = L.HYPRE_GB300_ParCSRMatrixMatvecTNoAlloc(1.0, A.par, xv.par, 0.0, short.par)
    assert err & gb.HYPRE_ERROR_ARG and (err >> 3) & 0xff == 5, err   # y is argument 5
    L.HYPRE_ClearAllErrors()
    for o in (xv, yv, short, A):
        o.destroy()
