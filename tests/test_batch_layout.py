"""Host-side checks of the batched solver's layout (CPU): the block-diagonal
batch generator, and the invariant the persistent kernel relies on -- BoomerAMG
on a block-diagonal matrix keeps every level block diagonal with each system's
coarse rows contiguous, at the offsets given by counting its C points."""
import numpy as np

from hypre_gb300 import problems as G


def test_batch_generator_blocks():
    I, J, V, off, ns, eps = G.aniso2d_batch(12, nmin=4, nmax=9, seed=2)
    assert off[0] == 0 and off[-1] == len(I) - 1
    assert np.array_equal(np.diff(off), ns.astype(np.int64) ** 2)
    assert np.all((eps >= 1e-3) & (eps <= 1.0))
    for s in range(12):
        rows = range(off[s], off[s + 1])
        cols = np.concatenate([J[I[r]:I[r + 1]] for r in rows])
        assert cols.min() >= off[s] and cols.max() < off[s + 1]


def test_block_diagonal_hierarchy(oracle_mod):
    O = oracle_mod
    I, J, V, off, ns, eps = G.aniso2d_batch(20, nmin=5, nmax=20, seed=3)
    H = O.Hierarchy(I, J, V, O.default_params(strong_threshold=0.25))
    offs = [off.astype(np.int64)]
    for l in range(H.num_levels - 1):
        cf = H.cf(l)
        o = offs[-1]
        nxt = np.zeros_like(o)
        for s in range(len(o) - 1):
            nxt[s + 1] = nxt[s] + np.count_nonzero(cf[o[s]:o[s + 1]] > 0)
        Pi, Pj, _, nc = H.csr("P", l)
        assert nxt[-1] == nc
        for s in range(len(o) - 1):
            for r in range(o[s], o[s + 1]):
                c = Pj[Pi[r]:Pi[r + 1]]
                assert np.all((c >= nxt[s]) & (c < nxt[s + 1]))
        Ai, Aj, _, _ = H.csr("A", l + 1)
        for s in range(len(nxt) - 1):
            for r in range(nxt[s], nxt[s + 1]):
                c = Aj[Ai[r]:Ai[r + 1]]
                assert np.all((c >= nxt[s]) & (c < nxt[s + 1]))
        offs.append(nxt)
