"""Learned parameters: the BF16 tensor-core MLP kernels against the CPU
reference (forward outputs and training gradients), training on the GPU, and
what the trained model gains over the default parameters on held-out
problems (with the revert-to-defaults judge)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _data(n, seed):
    import torch
    from mlp_ref import bf16
    rng = np.random.default_rng(seed)
    X = bf16(rng.uniform(-1.0, 1.5, (n, 16)))
    T = rng.uniform(0.2, 1.2, (n, 2))
    Xd = torch.tensor(X, dtype=torch.bfloat16, device="cuda")
    Td = torch.tensor(T, dtype=torch.float32, device="cuda")
    return X, T, Xd, Td


@pytest.mark.parametrize("n", [16, 1000, 40000])
def test_mlp_forward_matches_cpu(gb, n):
    from hypre_gb300 import learned
    import mlp_ref
    X, T, Xd, Td = _data(n, 1)
    p = learned.init_params(3)
    p[-2:] = [0.3, 0.9]
    out = learned.forward(Xd, p).cpu().numpy()
    ref, _, _ = mlp_ref.forward(X, p.astype(np.float64))
    err = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    assert err < 5e-3, err


@pytest.mark.parametrize("n", [16, 999, 50000])
def test_mlp_gradient_matches_cpu(gb, n):
    """GPU gradient of the MSE loss against the CPU reference, per parameter block."""
    from hypre_gb300 import learned
    import mlp_ref
    X, T, Xd, Td = _data(n, 2)
    p = learned.init_params(5)
    loss, g = learned.gradient(Xd, Td, p)
    loss_r, g_r = mlp_ref.gradient(X, T, p.astype(np.float64))
    assert abs(loss - loss_r) <= 2e-3 * abs(loss_r)
    k = 0
    for name, shape in mlp_ref.SIZES:
        m = int(np.prod(shape))
        a, b = g[k:k + m], g_r[k:k + m]
        err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        assert err < 2e-2, (name, err)
        k += m


def test_training_reduces_loss(gb):
    """Full-batch Adam on the GPU fits a smooth function of the features."""
    import torch
    from hypre_gb300 import learned
    rng = np.random.default_rng(4)
    n = 20000
    X = rng.uniform(0, 1, (n, 16))
    T = np.stack([0.2 + 0.6 * X[:, 3], 0.5 + 0.5 * X[:, 7] * X[:, 8]], 1)
    Xd = torch.tensor(X, dtype=torch.bfloat16, device="cuda")
    Td = torch.tensor(T, dtype=torch.float32, device="cuda")
    p, hist = learned.train(Xd, Td, steps=300, lr=3e-3)
    assert hist[-1][1] < 0.1 * hist[0][1]
    out = learned.forward(Xd, p).cpu().numpy()
    assert np.sqrt(np.mean((out - T) ** 2)) < 0.05


def test_learned_gain_over_defaults(gb):
    """Train on a sweep of small rotated anisotropic problems; on held-out
    problems the learned parameters (with the judge) need no more work than
    the defaults, and less on average."""
    from hypre_gb300 import learned
    I, J, V, off, eps, ang = learned.make_problems(160, n=10, seed=7)
    cost, its, labels, shape = learned.sweep_labels(I, J, V, off)
    A = gb.IJMatrix(I, J, V)
    X = learned.features(A)
    import torch
    T = torch.tensor(learned.row_targets(off, labels), device="cuda")
    p, hist = learned.train(X, T, steps=300, lr=3e-3)
    assert hist[-1][1] < hist[0][1]
    solver = learned.LearnedSolver(p, judge_iters=4)
    Ih, Jh, Vh, offh, epsh, angh = learned.make_problems(8, n=20, seed=99)
    ratio = []
    for s in range(8):
        a, b = offh[s], offh[s + 1]
        Ii = Ih[a:b + 1] - Ih[a]
        Js = Jh[Ih[a]:Ih[b]] - a
        Vs = Vh[Ih[a]:Ih[b]]
        n = b - a
        As = gb.IJMatrix(Ii, Js, Vs)
        rhs = np.random.default_rng(s).uniform(-1, 1, n)
        bv, xv = gb.IJVector(n, rhs), gb.IJVector(n, np.zeros(n))
        res = solver.solve(As, bv, xv)
        import scipy.sparse as sp
        r = rhs - sp.csr_matrix((Vs, Js, Ii), shape=(n, n)) @ xv.values()
        assert np.linalg.norm(r) / np.linalg.norm(rhs) < 1e-8
        # default run for the comparison
        amg = gb.BoomerAMG(StrongThreshold=0.25, RelaxType=18, Tol=0.0, MaxIter=1)
        amg.set("CyclePrecision", 1)
        k = gb.Krylov("pcg", tol=1e-8, maxit=200, amg=amg)
        xv.set(np.zeros(n))
        k.setup(As, bv, xv)
        k.solve(As, bv, xv)
        ratio.append(res["iterations"] / max(k.iterations(), 1))
        print(f"held-out {s}: eps {epsh[s]:.2e} learned {res['used']} theta {res['theta']:.3f} "
              f"its {res['iterations']} (default {k.iterations()}) factors {res['factor_learned']:.3f} "
              f"vs {res['factor_default']:.3f}")
        assert res["factor_learned"] <= res["factor_default"] or res["used"] == "default"
    print("label distribution (theta, weight):", np.unique(labels, axis=0, return_counts=True))
    print("mean iteration ratio learned/default:", np.mean(ratio))
    assert np.mean(ratio) <= 1.0 + 1e-12
    # the time judge keeps the set with the smaller estimated time, and the
    # solve still reaches the tolerance
    tjudge = learned.LearnedSolver(p, judge_iters=4, judge="time")
    for s in range(2):
        a, b = offh[s], offh[s + 1]
        Ii = Ih[a:b + 1] - Ih[a]
        Js = Jh[Ih[a]:Ih[b]] - a
        Vs = Vh[Ih[a]:Ih[b]]
        n = b - a
        As = gb.IJMatrix(Ii, Js, Vs)
        rhs = np.random.default_rng(50 + s).uniform(-1, 1, n)
        bv, xv = gb.IJVector(n, rhs), gb.IJVector(n, np.zeros(n))
        res = tjudge.solve(As, bv, xv)
        assert (res["used"] == "learned") == (res["estimate_learned"] <= res["estimate_default"])
        import scipy.sparse as sp
        r = rhs - sp.csr_matrix((Vs, Js, Ii), shape=(n, n)) @ xv.values()
        assert np.linalg.norm(r) / np.linalg.norm(rhs) < 1e-8
