"""Learned AMG parameters: per-row MLP over local stencil features that
predicts the strength threshold and the smoother weight.

Pipeline (all GPU work through libHYPRE_gb300's C ABI; torch only holds device
buffers):

1. `make_problems`: seeded 3-D rotated anisotropic diffusion problems
   (7-point), assembled as one block-diagonal batch.
2. `sweep_labels`: for every (threshold, weight) pair of a grid, one batched
   BoomerAMG setup on the whole batch and one persistent batched PCG solve
   (FP32 V-cycle, l1-Jacobi); the per-system cost is
   operator complexity x (iterations + setup_cycles), setup_cycles being the
   time of a setup in PCG iterations (`calibrate_setup_cycles` measures it on
   the GPU for a problem of the size the model will serve).  Each system's
   label is its cheapest pair.
3. `train`: every row of a system is a sample (its 16 stencil features ->
   the system's label); full-batch Adam on the BF16 tensor-core MLP kernels.
4. `LearnedSolver.solve`: BoomerAMG with the model (threshold from the finest
   level's rows, weight per level) inside FP64 PCG with the FP32 cycle; the
   judge runs the first `judge_iters` iterations with the learned and with
   the default parameters and keeps the learned ones only when they are not
   worse: by convergence factor (`judge="factor"`) or by estimated time
   (`judge="time"`: measured setup time + measured time per iteration x the
   iterations the factor predicts to the tolerance).
"""
import ctypes as C

import numpy as np

from . import BatchedPCG, BoomerAMG, IJMatrix, IJVector, Krylov, check, lib
from . import problems as G

THETAS = (0.25, 0.35, 0.5, 0.65, 0.8)
WEIGHTS = (0.6, 0.8, 1.0, 1.2)
SETUP_CYCLES = 8.0
DEFAULT_THETA = 0.25
DEFAULT_WEIGHT = 1.0


def nparam():
    n = C.c_int()
    lib().HYPRE_GB300_MLPNumParams(C.byref(n))
    return n.value


def init_params(seed=0):
    """He-style initialisation; the output bias starts at the default parameters."""
    rng = np.random.default_rng(seed)
    W1 = rng.standard_normal((64, 16)) * np.sqrt(2.0 / 16)
    W2 = rng.standard_normal((64, 64)) * np.sqrt(2.0 / 64)
    W3 = rng.standard_normal((2, 64)) * np.sqrt(1.0 / 64) * 0.1
    p = np.concatenate([W1.ravel(), np.zeros(64), W2.ravel(), np.zeros(64), W3.ravel(),
                        np.array([DEFAULT_THETA, DEFAULT_WEIGHT])])
    assert len(p) == nparam()
    return p.astype(np.float32)


def _dev():
    import torch
    return torch.device("cuda", torch.cuda.current_device())


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def features(A):
    """Row features (n x 16 BF16, device) of an assembled IJMatrix."""
    import torch
    X = torch.empty((A.n, 16), dtype=torch.bfloat16, device=_dev())
    check(lib().HYPRE_GB300_MLPRowFeatures(A.par, _ptr(X)), "features")
    return X


def forward(X, params):
    """MLP outputs (n x 2 FP32, device)."""
    import torch
    P = torch.as_tensor(np.asarray(params, np.float32), device=_dev())
    out = torch.empty((X.shape[0], 2), dtype=torch.float32, device=_dev())
    check(lib().HYPRE_GB300_MLPForward(X.shape[0], _ptr(X), _ptr(P), _ptr(out)), "forward")
    _sync()
    return out


def gradient(X, T, params):
    """(loss, gradient) of 0.5 * mean |MLP(X) - T|^2 on the GPU."""
    import torch
    P = torch.as_tensor(np.asarray(params, np.float32), device=_dev())
    g = torch.empty(nparam(), dtype=torch.float32, device=_dev())
    loss = torch.empty(1, dtype=torch.float32, device=_dev())
    check(lib().HYPRE_GB300_MLPGradient(X.shape[0], _ptr(X), _ptr(T), _ptr(P), _ptr(g), _ptr(loss)), "gradient")
    _sync()
    return float(loss.item()), g.cpu().numpy()


def _sync():
    s = C.c_void_p()
    lib().HYPRE_GB300_GetStream(C.byref(s))
    import torch
    torch.cuda.synchronize()


def train(X, T, params=None, steps=300, lr=3e-3, seed=0, log=None):
    """Full-batch Adam; returns (params, loss history)."""
    import torch
    dev = _dev()
    P = torch.as_tensor(init_params(seed) if params is None else np.asarray(params, np.float32), device=dev).clone()
    m = torch.zeros_like(P)
    v = torch.zeros_like(P)
    g = torch.empty_like(P)
    loss = torch.empty(1, dtype=torch.float32, device=dev)
    L = lib()
    hist = []
    for k in range(1, steps + 1):
        check(L.HYPRE_GB300_MLPGradient(X.shape[0], _ptr(X), _ptr(T), _ptr(P), _ptr(g), _ptr(loss)), "gradient")
        check(L.HYPRE_GB300_MLPAdamStep(_ptr(P), _ptr(g), _ptr(m), _ptr(v), lr, k), "adam")
        if k == 1 or k % 25 == 0 or k == steps:
            _sync()
            hist.append((k, float(loss.item())))
            if log:
                log(k, hist[-1][1])
    _sync()
    return P.cpu().numpy(), hist


# --------------------------------------------------------------------------
# training problems and labels
# --------------------------------------------------------------------------
def make_problems(num, n=12, seed=0, eps_lo=1e-4, eps_hi=1.0):
    """`num` rotated anisotropic problems (n^3, 7-point) as one block-diagonal
    matrix; returns (I, J, V, offsets, eps, angles)."""
    rng = np.random.default_rng(seed)
    eps = np.exp(rng.uniform(np.log(eps_lo), np.log(eps_hi), size=num))
    ang = rng.uniform(0.0, 2.0 * np.pi, size=(num, 3))
    Is, Js, Vs = [], [], []
    off = np.zeros(num + 1, np.int64)
    nz = 0
    for k in range(num):
        I, J, V = G.rotated_aniso3d(n, float(eps[k]), ang[k])
        Is.append(I[:-1].astype(np.int64) + nz)
        Js.append(J.astype(np.int64) + off[k])
        Vs.append(V)
        off[k + 1] = off[k] + len(I) - 1
        nz += len(J)
    I = np.concatenate(Is + [np.array([nz])]).astype(np.int32)
    return I, np.concatenate(Js).astype(np.int32), np.concatenate(Vs), off.astype(np.int32), eps, ang


def calibrate_setup_cycles(A, bv, xv, prec=1, tol=1e-8, maxit=300):
    """Time of the default BoomerAMG setup over the time of one PCG iteration
    with its cycle, measured for A on the GPU: (ratio, setup seconds, seconds
    per iteration, iterations)."""
    import time
    amg = BoomerAMG(StrongThreshold=DEFAULT_THETA, RelaxType=18, RelaxWt=DEFAULT_WEIGHT, Tol=0.0, MaxIter=1)
    amg.set("CyclePrecision", prec)
    k = Krylov("pcg", tol=tol, maxit=maxit, amg=amg)
    xv.set(np.zeros(A.n))
    for _ in range(2):                       # the second run is the measured one
        xv.set(np.zeros(A.n))
        _sync()
        t0 = time.perf_counter()
        k.setup(A, bv, xv)
        _sync()
        t1 = time.perf_counter()
        k.solve(A, bv, xv)
        _sync()
        t2 = time.perf_counter()
    its = max(k.iterations(), 1)
    t_iter = (t2 - t1) / its
    return (t1 - t0) / t_iter, t1 - t0, t_iter, its


def sweep_labels(I, J, V, off, thetas=THETAS, weights=WEIGHTS, seed=22775, shape=None, setup_cycles=SETUP_CYCLES):
    """Per-system cost over the (threshold, weight) grid with the batched
    solver; returns (cost[nθ, nw, nsys], iterations[...], labels[nsys, 2], shape)."""
    n = len(I) - 1
    nsys = len(off) - 1
    A = IJMatrix(I, J, V)
    b = G.park_miller(n, seed) * 2.0 - 1.0
    bv = IJVector(n, b)
    xv = IJVector(n, np.zeros(n))
    cost = np.zeros((len(thetas), len(weights), nsys))
    its = np.zeros((len(thetas), len(weights), nsys), np.int32)
    for i, th in enumerate(thetas):
        for j, w in enumerate(weights):
            amg = BoomerAMG(StrongThreshold=th, RelaxType=18, RelaxWt=w, Tol=0.0, MaxIter=1)
            bp = BatchedPCG(amg, tol=1e-8, maxit=200, prec=1, shape=shape)
            bp.setup(A, off)
            xv.set(np.zeros(n))
            bp.solve(bv, xv)
            lib().HYPRE_ClearAllErrors()
            if shape is None:
                shape = bp.shape()
            it = bp.iterations()
            ok = bp.relres() < 1e-8
            its[i, j] = np.where(ok, it, 10 ** 6)
            cost[i, j] = bp.complexities() * (its[i, j] + setup_cycles)
            del bp, amg
    flat = cost.reshape(-1, nsys)
    best = np.argmin(flat, axis=0)
    labels = np.stack([np.asarray(thetas)[best // len(weights)], np.asarray(weights)[best % len(weights)]], 1)
    return cost, its, labels, shape


def row_targets(off, labels):
    """Per-row targets: every row of system s gets labels[s]."""
    sizes = np.diff(off)
    return np.repeat(labels, sizes, axis=0).astype(np.float32)


# --------------------------------------------------------------------------
# solving with the learned parameters and the judge
# --------------------------------------------------------------------------
def convergence_factor(hist):
    """Average reduction per iteration of a residual history."""
    h = np.asarray(hist)
    k = len(h) - 1
    if k < 1 or h[0] <= 0:
        return 1.0
    return float((h[-1] / h[0]) ** (1.0 / k))


class LearnedSolver:
    """FP64 PCG + BoomerAMG (FP32 cycle) with learned threshold and weights;
    reverts to the defaults when the learned setup converges more slowly over
    the first `judge_iters` iterations."""

    def __init__(self, params, judge_iters=4, tol=1e-8, maxit=200, prec=1, judge="factor"):
        self.params = np.asarray(params, np.float64)
        self.judge_iters = judge_iters
        self.tol = tol
        self.maxit = maxit
        self.prec = prec
        self.judge = judge
        self.default_factor = {}

    def estimate(self, f, t_setup, t_iter):
        """Estimated seconds to the tolerance: setup + iterations predicted by
        the convergence factor f times the measured time per iteration."""
        n = self.maxit if not (0.0 < f < 1.0) else min(self.maxit, int(np.ceil(np.log(self.tol) / np.log(f))))
        return t_setup + t_iter * n

    def _solver(self, learned):
        amg = BoomerAMG(StrongThreshold=DEFAULT_THETA, RelaxType=18, RelaxWt=DEFAULT_WEIGHT, Tol=0.0, MaxIter=1)
        amg.set("CyclePrecision", self.prec)
        if learned:
            check(lib().HYPRE_GB300_BoomerAMGSetLearnedModel(amg.h, self.params.ctypes.data), "model")
        return amg

    def factor(self, A, bv, xv, learned):
        """Setup + the first judge_iters PCG iterations from x = 0; returns
        (factor, amg, krylov) with the hierarchy kept for continuing."""
        import time
        warm = self.judge == "time"
        amg = self._solver(learned)
        k = Krylov("pcg", tol=self.tol, maxit=self.judge_iters, amg=amg)
        xv.set(np.zeros(A.n))
        if warm:
            # warm timings: a first setup and solve pay one-time costs (pool
            # growth, launch-shape tuning, the cycle's graph capture)
            k.setup(A, bv, xv)
        _sync()
        t0 = time.perf_counter()
        k.setup(A, bv, xv)
        _sync()
        t_setup = time.perf_counter() - t0
        if warm:
            k.solve(A, bv, xv)
            xv.set(np.zeros(A.n))
        _sync()
        t0 = time.perf_counter()
        k.solve(A, bv, xv)
        _sync()
        t_solve = time.perf_counter() - t0
        lib().HYPRE_ClearAllErrors()
        self.last_times = (t_setup, t_solve / max(k.iterations(), 1))
        return convergence_factor(k.history()), amg, k

    def solve(self, A, bv, xv, key=None):
        """Judge, then finish the solve (warm start from the judge's iterate)
        with the chosen parameters.  Returns a dict with the choice, the
        total iterations and both factors."""
        f_l, amg_l, k_l = self.factor(A, bv, xv, True)
        ts_l, ti_l = self.last_times
        it0 = k_l.iterations()
        x_l = xv.values()
        if key is not None and key in self.default_factor:
            (f_d, ts_d, ti_d), amg_d, k_d = self.default_factor[key], None, None
        else:
            f_d, amg_d, k_d = self.factor(A, bv, xv, False)
            ts_d, ti_d = self.last_times
            if key is not None:
                self.default_factor[key] = (f_d, ts_d, ti_d)
        est_l, est_d = self.estimate(f_l, ts_l, ti_l), self.estimate(f_d, ts_d, ti_d)
        use_learned = est_l <= est_d if self.judge == "time" else f_l <= f_d
        theta = C.c_double()
        w = np.zeros(32)
        if use_learned:
            lib().HYPRE_GB300_BoomerAMGGetLearnedParams(amg_l.h, C.byref(theta), w.ctypes.data, 32)
            amg, k = amg_l, k_l
            xv.set(x_l)
        else:
            if k_d is None:
                f_d, amg_d, k_d = self.factor(A, bv, xv, False)
            amg, k = amg_d, k_d
            it0 = k_d.iterations()
        done = it0 < self.judge_iters
        rc = 0
        if not done:
            lib().HYPRE_PCGSetMaxIter(k.h, self.maxit - it0)
            rc = k.solve(A, bv, xv)
            it0 += k.iterations()
        return dict(used="learned" if use_learned else "default", iterations=it0, rc=rc,
                    factor_learned=f_l, factor_default=f_d, estimate_learned=est_l, estimate_default=est_d,
                    theta=theta.value if use_learned else DEFAULT_THETA,
                    weights=w[: amg.num_levels()].tolist() if use_learned else None)
