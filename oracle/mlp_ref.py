"""CPU reference of the learned-parameter MLP (16 -> 64 -> 64 -> 2, ReLU).

TEST INFRASTRUCTURE ONLY: the gradient check of the GPU training kernels
compares against this.  It emulates the GPU's BF16 roundings -- features,
weights, hidden activations and the backpropagated signals are rounded to
BF16 where the GPU feeds them to the tensor cores -- and accumulates in FP64,
so the remaining difference is the FP32 accumulation order on the GPU.  The
parameter layout is the library's: W1[64][16] b1[64] W2[64][64] b2[64]
W3[2][64] b3[2].
"""
import numpy as np

IN, H, OUT = 16, 64, 2
SIZES = [("W1", (H, IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (OUT, H)), ("b3", (OUT,))]
NPARAM = sum(int(np.prod(s)) for _, s in SIZES)


def bf16(x):
    """Round float values to BF16 (round to nearest even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    out, k = {}, 0
    for name, shape in SIZES:
        m = int(np.prod(shape))
        out[name] = np.asarray(p[k:k + m], dtype=np.float64).reshape(shape)
        k += m
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SIZES])


def _id(x):
    return np.asarray(x, dtype=np.float64)


def forward(X, p, rounding=True):
    """X: n x 16 features (already BF16 values); returns (O, H1, H2) as the GPU
    forms them (rounding=False: the same network in exact FP64)."""
    r = bf16 if rounding else _id
    w = unpack(p)
    W1, W2, W3 = r(w["W1"]), r(w["W2"]), r(w["W3"])
    H1 = r(np.maximum(X @ W1.T + w["b1"], 0.0))
    H2 = r(np.maximum(H1 @ W2.T + w["b2"], 0.0))
    O = H2 @ W3.T + w["b3"]
    return O, H1, H2


def gradient(X, T, p, rounding=True):
    """Mean squared error 0.5 * mean over rows of |O - T|^2 (per output pair) and its
    gradient with the GPU's BF16 roundings of dO, dH2, dH1 (rounding=False: exact)."""
    r = bf16 if rounding else _id
    n = X.shape[0]
    w = unpack(p)
    W2, W3 = r(w["W2"]), r(w["W3"])
    O, H1, H2 = forward(X, p, rounding)
    D = O - T
    loss = 0.5 * np.sum(D * D) / n
    dO = r(D / n)
    dH2 = r((dO @ W3) * (H2 > 0))
    dH1 = r((dH2 @ W2) * (H1 > 0))
    g = {"W3": dO.T @ H2, "b3": dO.sum(0), "W2": dH2.T @ H1, "b2": dH2.sum(0), "W1": dH1.T @ X, "b1": dH1.sum(0)}
    return loss, pack(g)


def init_params(seed=0):
    """He-style random initialisation (the library's training starts from this)."""
    rng = np.random.default_rng(seed)
    d = {"W1": rng.standard_normal((H, IN)) * np.sqrt(2.0 / IN), "b1": np.zeros(H),
         "W2": rng.standard_normal((H, H)) * np.sqrt(2.0 / H), "b2": np.zeros(H),
         "W3": rng.standard_normal((OUT, H)) * np.sqrt(1.0 / H), "b3": np.zeros(OUT)}
    return pack(d)
