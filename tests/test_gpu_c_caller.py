"""A C program written against the reference's API (tests/c_caller/amg_pcg.c:
IJ assembly row by row, BoomerAMG as the PCG preconditioner through
HYPRE_PtrToSolverFcn pointers, as in src/examples/ex5.c:342-400) is compiled
with gcc against include/HYPRE_gb300.h, linked with -lHYPRE_gb300 and run.  On
the 50^3 7-point Laplacian with the first configuration's settings it must
print the reference library's own result for the same system: the iteration
count and final relative residual of the golden fixture lap7_50_pcg_l1jacobi
(13 iterations, 3.539986e-09)."""
import os
import subprocess

import pytest

import golden_cases as G

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_c_caller_matches_reference(gb, tmp_path):
    libdir = os.path.dirname(gb.lib()._name)
    exe = str(tmp_path / "amg_pcg")
    subprocess.run(["gcc", "-std=gnu11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c_caller", "amg_pcg.c"), "-L", libdir, "-lHYPRE_gb300", "-lm",
                    "-Wl,-rpath," + libdir, "-o", exe], check=True)
    r = subprocess.run([exe, "50"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    words = r.stdout.split()
    its, rel = int(words[words.index("iterations") + 1]), words[words.index("relres") + 1]
    g = G.load("lap7_50_pcg_l1jacobi")
    assert its == int(g["iters"][0]) == 13
    assert rel == "%.6e" % float(g["final_relres"][0]) == "3.539986e-09", rel
