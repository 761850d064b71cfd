"""The C-ABI library loads without a GPU and exports every function that
include/*.h declares; host-only entry points work on the CPU."""
import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(\w+)\s*\([^;]*\)\s*;", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("InitGpuWorkspace", "PrepareGpuMesh", "RunGpuResidual", "RunGpuResidualJacobian",
              "FormFunctionFEMGpu", "FormJacobianFEMGpu"):
        assert n in names


def test_library_exports_every_declared_symbol():
    from biofem.gpu import LIB_PATH, load_library, EXPORTS
    lib = load_library()
    out = subprocess.run(["nm", "-D", "--defined-only", str(LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (\w+)$", out, flags=re.M))
    for n in declared_functions():
        assert n in exported, n
        assert hasattr(lib, n)
    assert set(EXPORTS) == set(declared_functions())


def test_errors_are_petsc_codes_without_gpu():
    from biofem.gpu import load_library
    lib = load_library()
    lib.RunGpuResidual.argtypes = [ctypes.c_void_p] * 3
    assert lib.RunGpuResidual(None, None, None) == 85   # PETSC_ERR_ARG_NULL
    assert b"null" in lib.BiofemGpuLastError()
