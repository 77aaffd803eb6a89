"""CPU tests of the C-ABI library: it loads without a GPU and exports every
function include/HYPRE_gb300.h declares (no compute calls)."""
import ctypes
import os
import subprocess

import pytest

import hypre_gb300 as gb


def _lib_built():
    return os.path.exists(gb.LIB_PATH)


def test_header_declares_reference_api():
    syms = gb.header_symbols()
    for must in ("HYPRE_IJMatrixCreate", "HYPRE_IJMatrixSetValues", "HYPRE_IJMatrixAssemble",
                 "HYPRE_BoomerAMGCreate", "HYPRE_BoomerAMGSetup", "HYPRE_BoomerAMGSolve",
                 "HYPRE_ParCSRPCGCreate", "HYPRE_ParCSRPCGSolve", "HYPRE_PCGSetPrecond",
                 "HYPRE_ParCSRFlexGMRESCreate", "HYPRE_FlexGMRESSetKDim", "HYPRE_ParCSRMatrixMatvec"):
        assert must in syms


@pytest.mark.skipif(not _lib_built(), reason="library not built")
def test_library_exports_every_declared_symbol():
    L = ctypes.CDLL(gb.LIB_PATH)
    missing = [s for s in gb.header_symbols() if not hasattr(L, s)]
    assert not missing, missing


@pytest.mark.skipif(not _lib_built(), reason="library not built")
def test_library_has_no_torch_or_oracle_dependency():
    out = subprocess.run(["nm", "-D", "--undefined-only", gb.LIB_PATH], capture_output=True, text=True).stdout
    assert "torch" not in out and "or_" not in out.split()
    ldd = subprocess.run(["ldd", gb.LIB_PATH], capture_output=True, text=True).stdout
    assert "liboracle" not in ldd and "libtorch" not in ldd and "HYPRE_ref" not in ldd


def test_build_targets_sm_103a_only():
    from hypre_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


@pytest.mark.skipif(not _lib_built(), reason="library not built")
def test_no_unresolved_internal_symbols():
    out = subprocess.run(["nm", "-D", "--undefined-only", gb.LIB_PATH], capture_output=True, text=True).stdout
    bad = [l for l in out.splitlines() if " gb_" in l or " HYPRE_" in l]
    assert not bad, bad
