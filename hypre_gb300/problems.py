"""Seeded problem generators (host numpy), CSR with the diagonal first and the
off-diagonals in ascending column order -- the row layout the reference's
generators and IJ assembly produce.

  laplace(kind, nx, ny, nz)       7-point (diag 6) / 27-point (diag 26) Laplacian,
                                  reference GenerateLaplacian / GenerateLaplacian27pt
                                  (src/parcsr_ls/par_laplace.c, par_laplace_27pt.c)
  fv_diffusion(n, seed, ...)      7-point finite-volume diffusion on n^3 cells,
                                  log-normal cell coefficients times 10^{-4,0,+4}
                                  on random blocks, harmonic-mean face coefficients,
                                  Dirichlet boundaries (no reference generator)
  aniso2d(n, eps)                 -eps*u_xx - u_yy, 5-point, Dirichlet
  rotated_aniso3d(n, eps, angles) 7-point discretisation of div(K grad u) with
                                  K = Q diag(1, eps, eps) Q^T (diagonal part of K,
                                  the 2-D analogue being GenerateRotate7pt)
  rhs(n, seed)                    2*PM-1 uniform[-1,1] from the Park-Miller
                                  sequence, scaled to unit 2-norm (the
                                  reference driver's right-hand side)
"""
import numpy as np


def _assemble(n, cols, vals, mask):
    """cols/vals: (n, k) with column 0 the diagonal and the rest in ascending
    column order; mask selects present entries."""
    cnt = mask.sum(axis=1)
    I = np.zeros(n + 1, np.int64)
    np.cumsum(cnt, out=I[1:])
    J = cols[mask].astype(np.int32)
    V = vals[mask].astype(np.float64)
    return I.astype(np.int32), J, V


def laplace(kind, nx, ny, nz):
    n = nx * ny * nz
    idx = np.arange(n, dtype=np.int64)
    ix = idx % nx
    iy = (idx // nx) % ny
    iz = idx // (nx * ny)
    offs = []
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                m = abs(dx) + abs(dy) + abs(dz)
                if m == 0 or (kind == 7 and m != 1):
                    continue
                offs.append((dx, dy, dz))
    k = len(offs) + 1
    cols = np.zeros((n, k), np.int64)
    vals = np.zeros((n, k))
    mask = np.zeros((n, k), bool)
    cols[:, 0] = idx
    vals[:, 0] = 26.0 if kind == 27 else 6.0
    mask[:, 0] = True
    for t, (dx, dy, dz) in enumerate(offs, start=1):
        jx, jy, jz = ix + dx, iy + dy, iz + dz
        ok = (jx >= 0) & (jx < nx) & (jy >= 0) & (jy < ny) & (jz >= 0) & (jz < nz)
        cols[:, t] = jx + nx * (jy + ny * jz)
        vals[:, t] = -1.0
        mask[:, t] = ok
    return _assemble(n, cols, vals, mask)


def _face_matrix(n3, Tx, Ty, Tz, Bx0, Bx1, By0, By1, Bz0, Bz1):
    """7-point matrix from face transmissibilities (shape (n,n,n-1) etc.) and
    Dirichlet boundary terms added to the diagonal."""
    n = n3
    N = n ** 3
    idx = np.arange(N).reshape(n, n, n)   # [z, y, x]
    diag = np.zeros((n, n, n))
    diag[:, :, :-1] += Tx; diag[:, :, 1:] += Tx
    diag[:, :-1, :] += Ty; diag[:, 1:, :] += Ty
    diag[:-1, :, :] += Tz; diag[1:, :, :] += Tz
    diag[:, :, 0] += Bx0; diag[:, :, -1] += Bx1
    diag[:, 0, :] += By0; diag[:, -1, :] += By1
    diag[0, :, :] += Bz0; diag[-1, :, :] += Bz1
    cols = np.zeros((N, 7), np.int64)
    vals = np.zeros((N, 7))
    mask = np.zeros((N, 7), bool)
    cols[:, 0] = idx.ravel(); vals[:, 0] = diag.ravel(); mask[:, 0] = True

    def put(t, shift_axis, sgn, T):
        c = np.zeros((n, n, n), np.int64)
        v = np.zeros((n, n, n))
        m = np.zeros((n, n, n), bool)
        sl_to = [slice(None)] * 3
        sl_from = [slice(None)] * 3
        if sgn < 0:
            sl_to[shift_axis] = slice(1, None)
            sl_from[shift_axis] = slice(0, -1)
        else:
            sl_to[shift_axis] = slice(0, -1)
            sl_from[shift_axis] = slice(1, None)
        c[tuple(sl_to)] = idx[tuple(sl_from)]
        v[tuple(sl_to)] = -T
        m[tuple(sl_to)] = True
        cols[:, t] = c.ravel(); vals[:, t] = v.ravel(); mask[:, t] = m.ravel()

    put(1, 0, -1, Tz)   # z-1
    put(2, 1, -1, Ty)   # y-1
    put(3, 2, -1, Tx)   # x-1
    put(4, 2, +1, Tx)   # x+1
    put(5, 1, +1, Ty)   # y+1
    put(6, 0, +1, Tz)   # z+1
    return _assemble(N, cols, vals, mask)


def fv_diffusion(n, seed=0, sigma=2.0, block=8, jump=4.0):
    rng = np.random.default_rng(seed)
    kappa = np.exp(sigma * rng.standard_normal((n, n, n)))
    nb = (n + block - 1) // block
    expo = rng.integers(-1, 2, size=(nb, nb, nb)).astype(np.float64) * jump
    fac = 10.0 ** expo
    fac = np.repeat(np.repeat(np.repeat(fac, block, 0), block, 1), block, 2)[:n, :n, :n]
    kappa = kappa * fac
    hm = lambda a, b: 2.0 * a * b / (a + b)
    Tx = hm(kappa[:, :, :-1], kappa[:, :, 1:])
    Ty = hm(kappa[:, :-1, :], kappa[:, 1:, :])
    Tz = hm(kappa[:-1, :, :], kappa[1:, :, :])
    return _face_matrix(n, Tx, Ty, Tz, 2 * kappa[:, :, 0], 2 * kappa[:, :, -1], 2 * kappa[:, 0, :],
                        2 * kappa[:, -1, :], 2 * kappa[0, :, :], 2 * kappa[-1, :, :])


def rotated_aniso3d(n, eps, angles):
    """K = Q diag(1, eps, eps) Q^T, Q from Euler angles (a, b, c); the 7-point
    operator uses the diagonal of K as the three axis diffusivities."""
    a, b, c = angles
    ca, sa, cb, sb, cc, sc = np.cos(a), np.sin(a), np.cos(b), np.sin(b), np.cos(c), np.sin(c)
    Rz1 = np.array([[ca, -sa, 0], [sa, ca, 0], [0, 0, 1]])
    Ry = np.array([[cb, 0, sb], [0, 1, 0], [-sb, 0, cb]])
    Rz2 = np.array([[cc, -sc, 0], [sc, cc, 0], [0, 0, 1]])
    Q = Rz1 @ Ry @ Rz2
    K = Q @ np.diag([1.0, eps, eps]) @ Q.T
    kx, ky, kz = K[0, 0], K[1, 1], K[2, 2]
    Tx = np.full((n, n, n - 1), kx)
    Ty = np.full((n, n - 1, n), ky)
    Tz = np.full((n - 1, n, n), kz)
    return _face_matrix(n, Tx, Ty, Tz, kx, kx, ky, ky, kz, kz)


def aniso2d(n, eps):
    N = n * n
    idx = np.arange(N)
    ix, iy = idx % n, idx // n
    cols = np.zeros((N, 5), np.int64)
    vals = np.zeros((N, 5))
    mask = np.zeros((N, 5), bool)
    cols[:, 0] = idx; vals[:, 0] = 2.0 * eps + 2.0; mask[:, 0] = True
    cols[:, 1] = idx - n; vals[:, 1] = -1.0; mask[:, 1] = iy > 0
    cols[:, 2] = idx - 1; vals[:, 2] = -eps; mask[:, 2] = ix > 0
    cols[:, 3] = idx + 1; vals[:, 3] = -eps; mask[:, 3] = ix < n - 1
    cols[:, 4] = idx + n; vals[:, 4] = -1.0; mask[:, 4] = iy < n - 1
    return _assemble(N, cols, vals, mask)


def park_miller(n, seed):
    """First n draws of the reference's Park-Miller generator (random.c),
    as doubles in (0, 1), computed by jump-ahead in blocks."""
    m = 2147483647
    a = 16807
    out = np.empty(n, np.int64)
    s = max(1, min(seed, m - 1))
    # sequential in chunks: x_{k+1} = a x_k mod m, vectorised by powers of a
    chunk = 4096
    pw = np.empty(chunk, np.int64)
    p = 1
    for k in range(chunk):
        p = (p * a) % m
        pw[k] = p
    x = s
    for start in range(0, n, chunk):
        cnt = min(chunk, n - start)
        out[start:start + cnt] = (pw[:cnt] * x) % m
        x = int(out[start + cnt - 1])
    return out.astype(np.float64) / m


def rhs(n, seed=22775, normalise=True):
    b = 2.0 * park_miller(n, seed) - 1.0
    if normalise:
        s = 0.0
        # sequential dot for a bit-identical norm with the reference's serial sum
        s = float(np.add.reduce(b * b)) if n > 100000 else sum((b * b).tolist())
        b = b * (1.0 / np.sqrt(s))
    return b


def aniso2d_batch(num, nmin=16, nmax=128, eps_lo=1e-3, eps_hi=1.0, seed=0):
    """Block-diagonal matrix of `num` independent 2-D anisotropic 5-point
    problems (-eps d_xx - d_yy on n x n grids), n uniform in [nmin, nmax],
    eps log-uniform in [eps_lo, eps_hi]; returns (I, J, V, offsets, sizes, eps)."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(nmin, nmax + 1, size=num)
    eps = np.exp(rng.uniform(np.log(eps_lo), np.log(eps_hi), size=num))
    Is, Js, Vs = [], [], []
    off = np.zeros(num + 1, np.int64)
    nnz_off = 0
    for k in range(num):
        I, J, V = aniso2d(int(ns[k]), float(eps[k]))
        N = len(I) - 1
        Is.append(I[:-1].astype(np.int64) + nnz_off)
        Js.append(J.astype(np.int64) + off[k])
        Vs.append(V)
        off[k + 1] = off[k] + N
        nnz_off += len(J)
    I = np.concatenate(Is + [np.array([nnz_off])]).astype(np.int32)
    J = np.concatenate(Js).astype(np.int32)
    V = np.concatenate(Vs)
    return I, J, V, off.astype(np.int32), ns, eps
