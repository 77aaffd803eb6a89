"""Generates the golden fixtures in this directory from the reference library
itself.

The reference's serial CPU BoomerAMG path is compiled from its own sources by
oracle/ref/Makefile into oracle/_ref/<machine>/amg_ref_dump (a driver that builds the
7/27-point Laplacian, runs BoomerAMG-PCG or -FlexGMRES through the public API
and dumps every level of the hierarchy).  This script runs it single-threaded
on each case below and stores what the tests compare against:

* small cases: every array of the hierarchy (A, P, S, CF, l1 norms,
  Chebyshev data), the residual history, the solution;
* large cases: SHA-256 digests of the integer arrays, checksums and a seeded
  sample of the floating-point arrays, the full residual history;
* sparse products (mm_*): C = A*A from the reference's
  HYPRE_ParCSRMatrixMatmat, with the IJ-assembled A it was given and, for
  generated matrices, the rows as they were put (in_i, in_j, in_v).

Usage (needs the reference sources, so it runs only where they are present):
    make -C oracle/ref REF=<reference>/src
    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DUMP = os.path.join(ROOT, "oracle", "_ref", os.uname().machine, "amg_ref_dump")
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402  (read_records, stencils)
sys.path.insert(0, os.path.join(ROOT, "tests"))

# name -> settings (the keys map one to one onto amg_ref_dump's options)
CASES = {
    "lap7_10_pcg_l1jacobi": dict(kind=7, n=(10, 10, 10), th=0.25, mxrs=1.0, Pmx=4, rlx=18, coarse_th=9, solver=1,
                                 full=True),
    "lap7_50_pcg_l1jacobi": dict(kind=7, n=(50, 50, 50), th=0.25, mxrs=1.0, Pmx=4, rlx=18, coarse_th=100, solver=1,
                                 full=False),
    "lap7_16x12x10_trunc": dict(kind=7, n=(16, 12, 10), th=0.25, mxrs=1.0, Pmx=3, tr=0.1, rlx=18, coarse_th=9,
                                solver=1, full=True),
    "lap27_12_agg_fgmres_gs": dict(kind=27, n=(12, 12, 12), th=0.5, mxrs=1.0, Pmx=4, agg_nl=1, agg_interp=6, rlx=11,
                                   coarse_th=9, solver=61, k=30, full=True),
    "lap7_16_agg2_pcg": dict(kind=7, n=(16, 16, 16), th=0.25, mxrs=1.0, Pmx=4, agg_nl=2, agg_interp=6, rlx=18,
                             coarse_th=9, solver=1, full=True),
    "lap27_24_agg_pcg_l1jacobi": dict(kind=27, n=(24, 24, 24), th=0.5, mxrs=1.0, Pmx=4, agg_nl=1, agg_interp=6,
                                      rlx=18, coarse_th=9, solver=1, full=False),
    "lap27_14_gs12_fgmres": dict(kind=27, n=(14, 14, 14), th=0.5, mxrs=1.0, Pmx=4, rlx=12, coarse_th=9, solver=61,
                                 k=30, full=True),
    "lap7_12_cheby3_pcg": dict(kind=7, n=(12, 12, 12), th=0.25, mxrs=1.0, Pmx=4, rlx=16, cheby_order=3, coarse_th=9,
                               solver=1, full=True),
    "lap27_10_cheby2_pcg": dict(kind=27, n=(10, 10, 10), th=0.25, mxrs=0.9, Pmx=4, rlx=16, cheby_order=2,
                                coarse_th=9, solver=1, full=True),
    # hybrid Gauss-Seidel: the reference's CPU defaults 13 down / 14 up (l1),
    # symmetric 6 and 8 (8 also weighted), forward 3 and backward 4
    "lap7_14_hgs13_14_pcg": dict(kind=7, n=(14, 14, 14), th=0.25, mxrs=1.0, Pmx=4, rlx=13, rlx_down=13, rlx_up=14,
                                 coarse_th=9, solver=1, full=True),
    "lap27_12_hgs6_pcg": dict(kind=27, n=(12, 12, 12), th=0.5, mxrs=1.0, Pmx=4, rlx=6, coarse_th=9, solver=1,
                              full=True),
    "lap7_12_hgs8_w08_pcg": dict(kind=7, n=(12, 12, 12), th=0.25, mxrs=1.0, Pmx=4, rlx=8, w=0.8, coarse_th=9,
                                 solver=1, full=True),
    "lap27_12_hgs3_fgmres": dict(kind=27, n=(12, 12, 12), th=0.5, mxrs=1.0, Pmx=4, rlx=3, coarse_th=9, solver=61,
                                 k=30, full=True),
    "lap7_13_agg_hgs4_fgmres": dict(kind=7, n=(13, 13, 13), th=0.25, mxrs=1.0, Pmx=4, agg_nl=1, agg_interp=6,
                                    rlx=4, coarse_th=9, solver=61, k=30, full=True),
    "lap27_30_hgs13_14_pcg": dict(kind=27, n=(30, 30, 30), th=0.5, mxrs=1.0, Pmx=4, rlx=13, rlx_down=13, rlx_up=14,
                                  coarse_th=9, solver=1, full=False),
    # the modified ("MM") interpolations: 16 extended, 17 extended+i, 18 extended+e
    "lap7_14_mm16_pcg": dict(kind=7, n=(14, 14, 14), th=0.25, mxrs=1.0, Pmx=4, interptype=16, rlx=18, coarse_th=9,
                             solver=1, full=True),
    "lap27_12_mm17_pcg": dict(kind=27, n=(12, 12, 12), th=0.5, mxrs=1.0, Pmx=4, interptype=17, rlx=18, coarse_th=9,
                              solver=1, full=True),
    "lap7_16_mm18_pcg": dict(kind=7, n=(16, 16, 16), th=0.25, mxrs=1.0, Pmx=4, interptype=18, rlx=18, coarse_th=9,
                             solver=1, full=True),
    "lap27_14_mm18_tr_pcg": dict(kind=27, n=(14, 14, 14), th=0.25, mxrs=0.9, Pmx=3, tr=0.1, interptype=18, rlx=18,
                                 coarse_th=9, solver=1, full=True),
    "lap27_30_mm18_pcg": dict(kind=27, n=(30, 30, 30), th=0.5, mxrs=1.0, Pmx=4, interptype=18, rlx=13, rlx_down=13,
                              rlx_up=14, coarse_th=9, solver=1, full=False),
    # direct interpolation (3), also on jumping coefficients and anisotropy
    "lap7_16_dir3_pcg": dict(kind=7, n=(16, 16, 16), th=0.25, mxrs=1.0, Pmx=4, interptype=3, rlx=18, coarse_th=9,
                             solver=1, full=True),
    "lap27_12_dir3_pcg": dict(kind=27, n=(12, 12, 12), th=0.5, mxrs=1.0, Pmx=4, interptype=3, rlx=18, coarse_th=9,
                              solver=1, full=True),
    "fv_12_dir3_pcg": dict(gen="fv", n=(12,), seed=3, th=0.25, mxrs=0.9, Pmx=4, interptype=3, rlx=18, coarse_th=9,
                           solver=1, full=True),
    # BAMG-direct (15): the reference's host path builds the direct interpolation
    "lap27_12_bamg15_pcg": dict(kind=27, n=(12, 12, 12), th=0.5, mxrs=1.0, Pmx=4, interptype=15, rlx=18, coarse_th=9,
                                solver=1, full=True),
    "aniso_40_dir3_tr_pcg": dict(gen="aniso", n=(40,), eps=0.001, th=0.25, mxrs=0.9, Pmx=3, tr=0.1, interptype=3,
                                 rlx=18, coarse_th=9, solver=1, full=True),
    "fv_12_mm18_pcg": dict(gen="fv", n=(12,), seed=4, th=0.25, mxrs=0.9, Pmx=4, interptype=18, rlx=18, coarse_th=9,
                           solver=1, full=True),
    # extended interpolation (14)
    "lap7_16_ext14_pcg": dict(kind=7, n=(16, 16, 16), th=0.25, mxrs=1.0, Pmx=4, interptype=14, rlx=18, coarse_th=9,
                              solver=1, full=True),
    "lap27_12_ext14_pcg": dict(kind=27, n=(12, 12, 12), th=0.5, mxrs=1.0, Pmx=4, interptype=14, rlx=18, coarse_th=9,
                               solver=1, full=True),
    "fv_14_ext14_tr_pcg": dict(gen="fv", n=(14,), seed=5, th=0.25, mxrs=0.9, Pmx=3, tr=0.1, interptype=14, rlx=18,
                               coarse_th=9, solver=1, full=True),
    # multipass interpolation on the aggressive levels (agg_interp_type 4, the
    # library default), with and without its truncation
    "lap27_16_agg4_pcg": dict(kind=27, n=(16, 16, 16), th=0.5, mxrs=1.0, Pmx=4, agg_nl=1, agg_interp=4, rlx=18,
                              coarse_th=9, solver=1, full=True),
    "lap7_20_agg4x2_pcg": dict(kind=7, n=(20, 20, 20), th=0.25, mxrs=1.0, Pmx=4, agg_nl=2, agg_interp=4, rlx=6,
                               coarse_th=9, solver=1, full=True),
    "lap7_18_agg4_pmx_fgmres": dict(kind=7, n=(18, 18, 18), th=0.25, mxrs=1.0, Pmx=4, agg_nl=1, agg_interp=4,
                                    agg_Pmx=4, rlx=3, coarse_th=9, solver=61, k=10, full=True),
    "fv_14_agg4_pcg": dict(gen="fv", n=(14,), seed=6, th=0.25, mxrs=0.9, Pmx=4, agg_nl=1, agg_interp=4, rlx=18,
                           coarse_th=9, solver=1, full=True),
    "aniso_48_agg4_pcg": dict(gen="aniso", n=(48,), eps=0.001, th=0.25, mxrs=0.9, Pmx=4, agg_nl=1, agg_interp=4,
                              agg_Pmx=3, rlx=18, coarse_th=9, solver=1, full=True),
    "zerodiag_14_agg4_fgmres": dict(gen="zerodiag", n=(14,), th=0.25, mxrs=1.0, Pmx=4, agg_nl=1, agg_interp=4, rlx=18,
                                    coarse_th=9, solver=61, k=10, full=True),
    # multipass interpolation in product form (agg_interp_type 8: each pass
    # block a scaled Q times the previous block; 9: Q times the previous block,
    # then scaled with the row's weak sum)
    "lap27_16_agg8_pcg": dict(kind=27, n=(16, 16, 16), th=0.5, mxrs=1.0, Pmx=4, agg_nl=1, agg_interp=8, rlx=18,
                              coarse_th=9, solver=1, full=True),
    "lap7_20_agg9x2_pcg": dict(kind=7, n=(20, 20, 20), th=0.25, mxrs=1.0, Pmx=4, agg_nl=2, agg_interp=9, rlx=18,
                               coarse_th=9, solver=1, full=True),
    "fv_14_agg8_pmx_pcg": dict(gen="fv", n=(14,), seed=7, th=0.25, mxrs=0.9, Pmx=4, agg_nl=1, agg_interp=8,
                               agg_Pmx=4, rlx=18, coarse_th=9, solver=1, full=True),
    "aniso_48_agg9_pcg": dict(gen="aniso", n=(48,), eps=0.001, th=0.25, mxrs=0.9, Pmx=4, agg_nl=1, agg_interp=9,
                              agg_Pmx=3, rlx=18, coarse_th=9, solver=1, full=True),
    "aniso_48_agg8_pcg": dict(gen="aniso", n=(48,), eps=0.001, th=0.25, mxrs=0.9, Pmx=4, agg_nl=1, agg_interp=8,
                              rlx=18, coarse_th=9, solver=1, full=True),
    # two-stage interpolation on the aggressive levels with the other first /
    # second stages: 5 modified extended / modified partial extended, 7
    # modified extended+e / modified partial extended+e, 1 extended+i /
    # partial extended+i
    "lap27_16_agg5_pcg": dict(kind=27, n=(16, 16, 16), th=0.5, mxrs=1.0, Pmx=4, agg_nl=1, agg_interp=5, rlx=18,
                              coarse_th=9, solver=1, full=True),
    "lap7_18_agg7_fgmres": dict(kind=7, n=(18, 18, 18), th=0.25, mxrs=1.0, Pmx=4, agg_nl=1, agg_interp=7, rlx=18,
                                coarse_th=9, solver=61, k=10, full=True),
    "fv_14_agg5x2_p12_pcg": dict(gen="fv", n=(14,), seed=8, th=0.25, mxrs=0.9, Pmx=4, agg_nl=2, agg_interp=5,
                                 agg_P12_mx=3, agg_Pmx=4, rlx=18, coarse_th=9, solver=1, full=True),
    "lap27_16_agg7_p12_pcg": dict(kind=27, n=(16, 16, 16), th=0.5, mxrs=1.0, Pmx=4, agg_nl=1, agg_interp=7,
                                  agg_P12_mx=4, rlx=18, coarse_th=9, solver=1, full=True),
    "lap7_20_agg1x2_pcg": dict(kind=7, n=(20, 20, 20), th=0.25, mxrs=1.0, Pmx=4, agg_nl=2, agg_interp=1, rlx=18,
                               coarse_th=9, solver=1, full=True),
    "lap27_16_agg3_pcg": dict(kind=27, n=(16, 16, 16), th=0.5, mxrs=1.0, Pmx=4, agg_nl=1, agg_interp=3, rlx=18,
                              coarse_th=9, solver=1, full=True),
    "fv_14_agg3x2_p12_pcg": dict(gen="fv", n=(14,), seed=12, th=0.25, mxrs=0.9, Pmx=4, agg_nl=2, agg_interp=3,
                                 agg_P12_mx=3, rlx=18, coarse_th=9, solver=1, full=True),
    "aniso_48_agg7_pcg": dict(gen="aniso", n=(48,), eps=0.001, th=0.25, mxrs=0.9, Pmx=4, agg_nl=1, agg_interp=7,
                              rlx=18, coarse_th=9, solver=1, full=True),
    # C/F relaxation (relax_order 1): C then F points on the way down, F then
    # C on the way up; l1-Jacobi with l1 norms over the row's own C/F class,
    # Jacobi, hybrid Gauss-Seidel (forward/backward/symmetric, l1, weighted),
    # two-stage Gauss-Seidel (which ignores the points, so it runs twice)
    "lap7_14_cf18_pcg": dict(kind=7, n=(14, 14, 14), th=0.25, mxrs=1.0, Pmx=4, rlx=18, relax_order=1, coarse_th=9,
                             solver=1, full=True),
    "lap27_16_agg4_cf18_pcg": dict(kind=27, n=(16, 16, 16), th=0.5, mxrs=1.0, Pmx=4, agg_nl=1, agg_interp=4, rlx=18,
                                   relax_order=1, coarse_th=9, solver=1, full=True),
    "fv_12_cf7_w07_fgmres": dict(gen="fv", n=(12,), seed=9, th=0.25, mxrs=0.9, Pmx=4, rlx=7, w=0.7, relax_order=1,
                                 coarse_th=9, solver=61, k=30, full=True),
    "lap7_12_cf6_pcg": dict(kind=7, n=(12, 12, 12), th=0.25, mxrs=1.0, Pmx=4, rlx=6, relax_order=1, coarse_th=9,
                            solver=1, full=True),
    "lap27_12_cf13_14_fgmres": dict(kind=27, n=(12, 12, 12), th=0.5, mxrs=1.0, Pmx=4, rlx=13, rlx_down=13, rlx_up=14,
                                    relax_order=1, coarse_th=9, solver=61, k=30, full=True),
    "lap7_13_cf11_fgmres": dict(kind=7, n=(13, 13, 13), th=0.25, mxrs=1.0, Pmx=4, rlx=11, relax_order=1,
                                coarse_th=9, solver=61, k=30, full=True),
    "aniso_40_cf8_w08_pcg": dict(gen="aniso", n=(40,), eps=0.001, th=0.25, mxrs=0.9, Pmx=4, rlx=8, w=0.8,
                                 relax_order=1, coarse_th=9, solver=1, full=True),
    # W-cycles (cycle_type 2), F-cycles, two sweeps per relaxation
    "lap7_16_w_pcg": dict(kind=7, n=(16, 16, 16), th=0.25, mxrs=1.0, Pmx=4, rlx=18, cycle_type=2, coarse_th=9,
                          solver=1, full=True),
    "lap27_14_w_gs11_fgmres": dict(kind=27, n=(14, 14, 14), th=0.5, mxrs=1.0, Pmx=4, rlx=11, cycle_type=2,
                                   coarse_th=9, solver=61, k=30, full=True),
    "lap7_16_f_pcg": dict(kind=7, n=(16, 16, 16), th=0.25, mxrs=1.0, Pmx=4, rlx=18, fcycle=1, coarse_th=9, solver=1,
                          full=True),
    "fv_12_w_hgs6_ns2_pcg": dict(gen="fv", n=(12,), seed=10, th=0.25, mxrs=0.9, Pmx=4, rlx=6, cycle_type=2, ns=2,
                                 coarse_th=9, solver=1, full=True),
    "lap27_16_agg4_f_cheby_pcg": dict(kind=27, n=(16, 16, 16), th=0.5, mxrs=1.0, Pmx=4, agg_nl=1, agg_interp=4,
                                      rlx=16, cheby_order=2, fcycle=1, coarse_th=9, solver=1, full=True),
    "lap7_14_w_cf18_amg": dict(kind=7, n=(14, 14, 14), th=0.25, mxrs=1.0, Pmx=4, rlx=18, cycle_type=2,
                               relax_order=1, coarse_th=9, solver=0, precond=0, full=True),
    # PCG's relative-change test (x must also stop changing)
    # SSOR / hybrid Gauss-Seidel with an outer weight (SetOuterWt)
    "lap7_12_hgs6_ow09_pcg": dict(kind=7, n=(12, 12, 12), th=0.25, mxrs=1.0, Pmx=4, rlx=6, ow=0.9, coarse_th=9,
                                  solver=1, full=True),
    "lap27_12_hgs8_w08_ow12_pcg": dict(kind=27, n=(12, 12, 12), th=0.5, mxrs=1.0, Pmx=4, rlx=8, w=0.8, ow=1.2,
                                       coarse_th=9, solver=1, full=True),
    "lap7_16_relchg_pcg": dict(kind=7, n=(16, 16, 16), th=0.25, mxrs=1.0, Pmx=4, rlx=18, rel_change=1, coarse_th=9,
                               solver=1, full=True),
    "fv_12_relchg_pcg": dict(gen="fv", n=(12,), seed=11, th=0.25, mxrs=0.9, Pmx=4, rlx=18, rel_change=1,
                             coarse_th=9, solver=1, full=True),
    # edge cases: no strong couplings (coarsening stops at once, the single
    # level is above max_coarse_size and relaxes instead of a direct solve),
    # a level cap that leaves a large coarsest level, a matrix within
    # max_coarse_size (direct solve only)
    "diag_2000_pcg": dict(gen="diag", n=(2000,), th=0.25, mxrs=0.9, Pmx=4, rlx=18, coarse_th=9, solver=1, full=True),
    # the smallest systems: one unknown, and a 1-D pair (two 7-point cells)
    "diag_1_pcg": dict(gen="diag", n=(1,), th=0.25, mxrs=0.9, Pmx=4, rlx=18, coarse_th=9, solver=1, full=True),
    "lap7_2x1x1_fgmres": dict(kind=7, n=(2, 1, 1), th=0.25, mxrs=1.0, Pmx=4, rlx=18, coarse_th=9, solver=61, k=5,
                              full=True),
    "lap27_12_ml2_pcg": dict(kind=27, n=(12, 12, 12), th=0.5, mxrs=1.0, Pmx=4, rlx=18, coarse_th=9, max_levels=2,
                             solver=1, full=True),
    "lap27_12_ml2_hgs6_pcg": dict(kind=27, n=(12, 12, 12), th=0.5, mxrs=1.0, Pmx=4, rlx=6, coarse_th=9, max_levels=2,
                                  solver=1, full=True),
    "lap7_2_pcg": dict(kind=7, n=(2, 2, 2), th=0.25, mxrs=1.0, Pmx=4, rlx=18, coarse_th=9, solver=1, full=True),
    # BoomerAMG as the solver (V-cycles in place on (b, x) until the relative
    # residual is below tol)
    "lap7_16_amg_l1jac": dict(kind=7, n=(16, 16, 16), th=0.25, mxrs=1.0, Pmx=4, rlx=18, coarse_th=9, solver=0,
                              precond=0, full=True),
    "lap27_12_amg_hgs3": dict(kind=27, n=(12, 12, 12), th=0.5, mxrs=1.0, Pmx=4, rlx=3, coarse_th=9, solver=0,
                              precond=0, full=True),
    "lap27_14_agg_amg_gs11": dict(kind=27, n=(14, 14, 14), th=0.5, mxrs=1.0, Pmx=4, agg_nl=1, agg_interp=6, rlx=11,
                                  coarse_th=9, solver=0, precond=0, full=True),
    "lap27_48_agg4_pcg": dict(kind=27, n=(48, 48, 48), th=0.5, mxrs=1.0, Pmx=4, agg_nl=1, agg_interp=4, rlx=18,
                              coarse_th=9, solver=1, full=False),
    "lap27_40_ext14_pcg": dict(kind=27, n=(40, 40, 40), th=0.5, mxrs=1.0, Pmx=4, interptype=14, rlx=18, coarse_th=9,
                               solver=1, full=False),
}


def dump_args(c, out):
    if "gen" in c:
        import golden_cases as GC
        I, J, V = GC.generate(c)
        mat = out + ".csr"
        with open(mat, "wb") as f:
            np.array([len(I) - 1, len(J)], np.int32).tofile(f)
            np.asarray(I, np.int32).tofile(f); np.asarray(J, np.int32).tofile(f)
            np.asarray(V, np.float64).tofile(f)
        a = [DUMP, "-mat", mat]
    else:
        a = [DUMP, "-lap%d" % c["kind"]] + [str(v) for v in c["n"]]
    for key in ("th", "mxrs", "Pmx", "tr", "interptype", "agg_nl", "agg_interp", "agg_Pmx", "agg_P12_mx", "max_levels", "precond", "rlx", "rlx_down", "rlx_up", "relax_order", "cycle_type", "fcycle", "ns", "rel_change", "ow", "w",
                "coarse_th", "solver", "k", "cheby_order"):
        if key in c:
            a += ["-" + key, str(c[key])]
    return a + ["-tol", "1e-8", "-rlx_coarse", "9", "-o", out]


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def sample_idx(n, k=512, seed=7):
    if n <= k:
        return np.arange(n)
    return np.sort(np.random.default_rng(seed).choice(n, k, replace=False))


def make(name, c):
    tmp = os.path.join("/tmp", "golden_%s.bin" % name)
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(dump_args(c, tmp), capture_output=True, text=True, env=env, check=True)
    rec = O.read_records(tmp)
    os.unlink(tmp)
    out = {"case": np.array(json.dumps({k: v for k, v in c.items() if k != "full"})),
           "dump_stdout": np.array(r.stdout)}
    if "gen" in c:
        # the rows the driver was given: the generators use numpy's exp, whose
        # last bits differ between machines
        import golden_cases as GC
        I, J, V = GC.generate(c)
        out.update(in_i=np.asarray(I, np.int32), in_j=np.asarray(J, np.int32), in_v=np.asarray(V, np.float64))
    for key in ("iters", "final_relres", "nlev", "lev_rows", "lev_nnz", "relres", "resnorms"):
        if key in rec:
            out[key] = rec[key]
    for key, v in rec.items():
        if key in out or key in ("t_setup", "t_solve"):
            continue
        if c["full"]:
            out[key] = v
        elif v.dtype == np.int32:
            out["sha256:" + key] = np.array(digest(v))
            out["len:" + key] = np.array(len(v))
        else:
            idx = sample_idx(len(v))
            out["sum:" + key] = np.array(float(np.sum(v)))
            out["abssum:" + key] = np.array(float(np.sum(np.abs(v))))
            out["sample_idx:" + key] = idx.astype(np.int64)
            out["sample:" + key] = v[idx]
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print("%-28s levels %d iters %d  %6.1f KB" % (name, int(rec["nlev"][0]), int(rec["iters"][0]),
                                                  os.path.getsize(path) / 1024))


# Sparse products C = A*A through HYPRE_ParCSRMatrixMatmat (full arrays of the
# IJ-assembled A and of C).  "gen" cases write A to a binary CSR file first.
MATMAT = {
    "mm_lap7_10": dict(kind=7, n=(10, 10, 10)),
    "mm_lap27_9x8x7": dict(kind=27, n=(9, 8, 7)),
    "mm_lap9pt2d_16": dict(gen="9pt2d", n=16),
    "mm_empty_rows": dict(gen="empty_rows", n=6),
    "mm_random_300": dict(gen="random", n=300),
}


def _gen_matrix(c):
    """Host CSR (I, J, V) of a generated matrix (rows as given; IJ assembly
    moves each row's diagonal first)."""
    from hypre_gb300 import problems as P
    if c["gen"] == "9pt2d":
        I, J, V = P.laplace(27, c["n"], c["n"], 1)
        V = np.where(J == np.repeat(np.arange(len(I) - 1), np.diff(I)), 8.0, V)
        return I, J, V
    if c["gen"] == "empty_rows":
        I, J, V = P.laplace(7, c["n"], c["n"], c["n"])
        n = len(I) - 1
        keep = np.ones(n, bool)
        keep[[0, 7, 50, 51, 100, n - 1]] = False
        rows = np.repeat(np.arange(n), np.diff(I))
        m = keep[rows]
        cnt = np.where(keep, np.diff(I), 0)
        I2 = np.zeros(n + 1, np.int32)
        np.cumsum(cnt, out=I2[1:])
        return I2, J[m].astype(np.int32), V[m]
    rng = np.random.default_rng(5)
    n = c["n"]
    rows = []
    for i in range(n):
        k = int(rng.integers(0, 9))
        cols = rng.choice(n, k, replace=False)
        if rng.random() < 0.8 and i not in cols:
            cols = np.append(cols, i)
        rows.append(cols)
    I = np.zeros(n + 1, np.int32)
    np.cumsum([len(r) for r in rows], out=I[1:])
    J = np.concatenate(rows).astype(np.int32)
    V = rng.standard_normal(len(J))
    return I, J, V


def make_matmat(name, c):
    tmp = os.path.join("/tmp", "golden_%s.bin" % name)
    args = [DUMP, "-matmat", "-o", tmp]
    inp = {}
    if "gen" in c:
        I, J, V = _gen_matrix(c)
        inp = {"in_i": I.astype(np.int32), "in_j": J.astype(np.int32), "in_v": V.astype(np.float64)}
        mat = os.path.join("/tmp", "golden_%s.csr" % name)
        with open(mat, "wb") as f:
            np.array([len(I) - 1, len(J)], np.int32).tofile(f)
            I.astype(np.int32).tofile(f); J.astype(np.int32).tofile(f); V.astype(np.float64).tofile(f)
        args += ["-mat", mat]
    else:
        args += ["-lap%d" % c["kind"]] + [str(v) for v in c["n"]]
    r = subprocess.run(args, capture_output=True, text=True, env=dict(os.environ, OMP_NUM_THREADS="1"),
                       check=True)
    rec = O.read_records(tmp)
    os.unlink(tmp)
    out = {"case": np.array(json.dumps(c)), "dump_stdout": np.array(r.stdout)}
    for key in ("A0_i", "A0_j", "A0_v", "C0_i", "C0_j", "C0_v"):
        out[key] = rec[key]
    out.update(inp)      # the rows as put (one SetValues per row after SetRowSizes)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print("%-28s A nnz %d, C nnz %d  %6.1f KB" % (name, len(rec["A0_j"]), len(rec["C0_j"]),
                                                  os.path.getsize(path) / 1024))


def main():
    if not os.path.exists(DUMP):
        sys.exit("build the reference dumper first: make -C oracle/ref REF=<reference>/src")
    only = set(sys.argv[1:])          # case names to remake (default: all)
    for name, c in CASES.items():
        if not only or name in only:
            make(name, c)
    for name, c in MATMAT.items():
        if not only or name in only:
            make_matmat(name, c)


if __name__ == "__main__":
    main()
