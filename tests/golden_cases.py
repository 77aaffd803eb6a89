"""Golden fixtures written by tests/golden/make_golden.py from the reference
library (compiled from its own sources) and the checks that compare a
hierarchy -- the oracle's or the GPU's -- against them."""
import glob
import hashlib
import json
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def case_names():
    """BoomerAMG setup + solve fixtures."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz"))
                  if not os.path.basename(p).startswith("mm_"))


def matmat_names():
    """Sparse-product fixtures (C = A*A from HYPRE_ParCSRMatrixMatmat)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "mm_*.npz")))


def load(name):
    d = dict(np.load(os.path.join(GOLDEN_DIR, name + ".npz")))
    d["case"] = json.loads(str(d["case"]))
    return d


def matrix(c, O, g=None):
    """The case's matrix (I, J, V): the reference generators' stencils, or,
    for a generated case, the rows the reference driver was given (stored in
    the record g as in_i, in_j, in_v)."""
    if "gen" not in c:
        return O.stencil(c["kind"], *c["n"])
    if g is not None and "in_i" in g:
        return g["in_i"], g["in_j"], g["in_v"]
    return generate(c)


def generate(c):
    """A seeded project generator ("gen": "fv" finite-volume diffusion on n^3
    cells, "aniso" 2-D anisotropic 5-point with eps, "diag" a diagonal matrix
    with entries from 1 to 3 (no strong couplings), "zerodiag" the 7-point
    Laplacian on n^3 with the diagonal of every row i = 5 mod 11 set to zero,
    so that interpolation rows meet a zero diagonal)."""
    from hypre_gb300 import problems as P
    if c["gen"] == "fv":
        return P.fv_diffusion(c["n"][0], seed=c.get("seed", 0))
    if c["gen"] == "diag":
        n = c["n"][0]
        return (np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32), np.linspace(1.0, 3.0, n))
    if c["gen"] == "zerodiag":
        n = c["n"][0]
        I, J, V = P.laplace(7, n, n, n)
        rows = np.repeat(np.arange(len(I) - 1), np.diff(I))
        V = np.where((J == rows) & (rows % 11 == 5), 0.0, V)
        return I, J, V
    return P.aniso2d(c["n"][0], c["eps"])


def oracle_params(c):
    """or_amg_params keyword arguments of a golden case."""
    p = dict(strong_threshold=c["th"], max_row_sum=c["mxrs"], p_max_elmts=c["Pmx"],
             trunc_factor=c.get("tr", 0.0), agg_num_levels=c.get("agg_nl", 0),
             agg_interp_type=c.get("agg_interp", 4), relax_down=c.get("rlx_down", c["rlx"]),
             relax_up=c.get("rlx_up", c["rlx"]), relax_coarse=9, max_coarse_size=c["coarse_th"],
             relax_weight=c.get("w", 1.0), interp_type=c.get("interptype", 6))
    if "cheby_order" in c:
        p["cheby_order"] = c["cheby_order"]
    if "agg_Pmx" in c:
        p["agg_p_max_elmts"] = c["agg_Pmx"]
    if "agg_P12_mx" in c:
        p["agg_p12_max_elmts"] = c["agg_P12_mx"]
    if "relax_order" in c:
        p["relax_order"] = c["relax_order"]
    if "cycle_type" in c:
        p["cycle_type"] = c["cycle_type"]
    if "fcycle" in c:
        p["fcycle"] = c["fcycle"]
    if "ns" in c:
        p["num_sweeps"] = c["ns"]
    if "rel_change" in c:
        p["pcg_rel_change"] = c["rel_change"]
    if "ow" in c:
        p["outer_weight"] = c["ow"]
    if "max_levels" in c:
        p["max_levels"] = c["max_levels"]
    return p


def amg_params(c):
    """HYPRE_BoomerAMGSet* values of a golden case."""
    p = dict(StrongThreshold=c["th"], MaxRowSum=c["mxrs"], PMaxElmts=c["Pmx"], TruncFactor=c.get("tr", 0.0),
             AggNumLevels=c.get("agg_nl", 0), RelaxType=c["rlx"], MaxCoarseSize=c["coarse_th"],
             RelaxWt=c.get("w", 1.0), InterpType=c.get("interptype", 6))
    cyc = [(c[k], part) for k, part in (("rlx_down", 1), ("rlx_up", 2)) if k in c]
    if cyc:
        p["CycleRelaxType"] = cyc
    if c.get("agg_nl", 0):
        p["AggInterpType"] = c.get("agg_interp", 4)
    if "agg_Pmx" in c:
        p["AggPMaxElmts"] = c["agg_Pmx"]
    if "agg_P12_mx" in c:
        p["AggP12MaxElmts"] = c["agg_P12_mx"]
    if "relax_order" in c:
        p["RelaxOrder"] = c["relax_order"]
    if "cycle_type" in c:
        p["CycleType"] = c["cycle_type"]
    if "fcycle" in c:
        p["FCycle"] = c["fcycle"]
    if "ns" in c:
        p["NumSweeps"] = c["ns"]
    if "ow" in c:
        p["OuterWt"] = c["ow"]
    if "max_levels" in c:
        p["MaxLevels"] = c["max_levels"]
    if "cheby_order" in c:
        p["ChebyOrder"] = c["cheby_order"]
    return p


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def check_array(g, key, a, rtol=0.0):
    """a against the golden record key: exact for integers; floats exact when
    rtol is 0, else to rtol relative (checksums and a seeded sample for the
    large cases)."""
    a = np.asarray(a)
    if key in g:
        ref = g[key]
        assert a.shape == ref.shape, f"{key}: {a.shape} vs {ref.shape}"
        if ref.dtype == np.int32 or rtol == 0.0:
            assert np.array_equal(a, ref), f"{key} differs"
        else:
            np.testing.assert_allclose(a, ref, rtol=rtol, atol=0, err_msg=key)
        return
    if ("sha256:" + key) in g:
        assert len(a) == int(g["len:" + key]), f"{key} length"
        assert _digest(a.astype(np.int32)) == str(g["sha256:" + key]), f"{key} digest"
        return
    if ("sum:" + key) in g:
        idx = g["sample_idx:" + key]
        if rtol == 0.0:
            assert np.array_equal(a[idx], g["sample:" + key]), f"{key} sample"
        else:
            np.testing.assert_allclose(a[idx], g["sample:" + key], rtol=rtol, atol=0, err_msg=key)
        np.testing.assert_allclose(np.sum(np.abs(a)), float(g["abssum:" + key]), rtol=max(rtol, 1e-13), atol=0,
                                   err_msg=key + " abs checksum")
        return
    raise KeyError(key)


def has(g, key):
    return key in g or ("sha256:" + key) in g or ("sum:" + key) in g


def check_hierarchy(g, num_levels, csr, cf, l1, cheby=None, value_rtol=0.0, cheby_rtol=0.0):
    """Compares a hierarchy given by accessor functions with the golden case:
    csr(which, level) -> (I, J, V), cf(level), l1(level), cheby(level, order) ->
    (coefs, (max_eig, min_eig), ds)."""
    c = g["case"]
    assert num_levels == int(g["nlev"][0]), "number of levels"
    for l in range(num_levels):
        I, J, V = csr("A", l)
        check_array(g, f"A{l}_i", I)
        check_array(g, f"A{l}_j", J)
        check_array(g, f"A{l}_v", V, value_rtol)
        if has(g, f"L1_{l}"):
            check_array(g, f"L1_{l}", l1(l), value_rtol)
        if l < num_levels - 1:
            I, J, V = csr("P", l)
            check_array(g, f"P{l}_i", I)
            check_array(g, f"P{l}_j", J)
            check_array(g, f"P{l}_v", V, value_rtol)
            check_array(g, f"CF{l}", cf(l))
            if has(g, f"S{l}_i"):
                I, J, _ = csr("S", l)
                check_array(g, f"S{l}_i", I)
                check_array(g, f"S{l}_j", J)
        if cheby is not None and has(g, f"CHEB_COEF{l}"):
            co, eig, ds = cheby(l, c["cheby_order"])
            check_array(g, f"CHEB_DS{l}", ds)
            check_array(g, f"CHEB_EIG{l}", np.array(eig), cheby_rtol)
            check_array(g, f"CHEB_COEF{l}", co, cheby_rtol * 10)
