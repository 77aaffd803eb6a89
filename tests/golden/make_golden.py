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
  sample of the floating-point arrays, the full residual history.

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

from oracle import oracle as O  # noqa: E402  (only read_records)

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
}


def dump_args(c, out):
    a = [DUMP, "-lap%d" % c["kind"]] + [str(v) for v in c["n"]]
    for key in ("th", "mxrs", "Pmx", "tr", "agg_nl", "agg_interp", "rlx", "coarse_th", "solver", "k", "cheby_order"):
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


def main():
    if not os.path.exists(DUMP):
        sys.exit("build the reference dumper first: make -C oracle/ref REF=<reference>/src")
    for name, c in CASES.items():
        make(name, c)


if __name__ == "__main__":
    main()
