"""Build recipe for biofem-ia_gb300/lib/libbiofem_gpu.so (sm_103a).

nvcc compiles the CUDA translation units for exactly one target,
-gencode arch=compute_103a,code=sm_103a; g++ compiles the host-only C++.
Objects are built in parallel and linked into one shared library with the
C-ABI declared in include/biofem_gpu.h.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
PKG = HERE.parent
ROOT = PKG.parent
LIB_DIR = PKG / "lib"
LIB = LIB_DIR / "libbiofem_gpu.so"
OBJ_DIR = LIB_DIR / "obj"
CUDA_SOURCES = ["kernels.cu", "bridge.cu", "noalloc.cu", "solver.cu", "amg.cu"]
CXX_SOURCES = ["topology.cpp", "serve.cpp", "amg_setup.cpp", "formats.cpp"]
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-pthread"]


def nvcc() -> str:
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    return str(cand) if cand.exists() else "nvcc"


def _deps() -> list[Path]:
    return [HERE / s for s in CUDA_SOURCES + CXX_SOURCES] + list(HERE.glob("*.h")) + list(HERE.glob("*.cuh")) \
        + [ROOT / "include" / "biofem_gpu.h"]


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> Path:
    if LIB.exists() and not force and not ptxas_info:
        t = LIB.stat().st_mtime
        if all(p.stat().st_mtime <= t for p in _deps()):
            return LIB
    OBJ_DIR.mkdir(parents=True, exist_ok=True)

    def compile_one(src: str) -> Path:
        obj = OBJ_DIR / (Path(src).stem + ".o")
        if src.endswith(".cu"):
            cmd = [nvcc(), *GENCODE, *NVCC_FLAGS, "-c", str(HERE / src), "-o", str(obj)]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
        else:
            cuda_inc = Path(nvcc()).resolve().parent.parent / "include"
            cmd = ["g++", *CXX_FLAGS, "-I", str(cuda_inc), "-c", str(HERE / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compiling {src} failed:\n{r.stdout}\n{r.stderr}")
        if ptxas_info or verbose:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=4) as ex:
        objs = list(ex.map(compile_one, CUDA_SOURCES + CXX_SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *GENCODE, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart", "-Xcompiler", "-pthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"linking failed:\n{r.stdout}\n{r.stderr}")
    tmp.replace(LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
