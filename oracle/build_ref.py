"""Build recipe for oracle/_ref/libbiofem_ref.so, oracle/_ref/libbiofem_ref_dyn.so
and oracle/_ref/ref_cuda_kernel.cubin (TEST INFRASTRUCTURE ONLY).

libbiofem_ref.so compiles the reference's own, unmodified hot-path C files
where they lie (``<reference>/src/{active_strain,math,bending,io,external}.c``)
together with the petsc-lite shim (oracle/petsc_lite/) and the np = 1 driver
(oracle/ref_driver.c).  libbiofem_ref_dyn.so adds the reference's src/main.c
(FDynamic, xAccVel; its ``main`` renamed) and src/material.c (Mass, Damp); the
driver is compiled with -DREF_DRIVER_WITH_MAIN so that main.c's globals are
the ones used, and every external that main.c names but the dynamic term
never calls (SNES, DMPlex setup, LV mesh loaders, CUDA / Kokkos bridges, ...)
is resolved by an abort stub generated here from the linker's list of
undefined references.  ref_cuda_kernel.cubin is the device code of the
reference's own GPU kernels (src/cuda_kernel.cu: SubdivGeomKernel_,
MetricTensorKernel_, ...) compiled unmodified for sm_103a against the
petsc-lite headers; being device code only, it loads on any host
(oracle/ref_cuda.py).  The results are the checkers that pin the restated
oracle and generate tests/golden/.  They are built only where the reference
sources exist; nothing on the product path links them.

The reference root is BIOFEM_REFERENCE_ROOT if set, else /root/reference.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
REFERENCE = Path(os.environ.get("BIOFEM_REFERENCE_ROOT", "/root/reference"))
OUT_DIR = HERE / "_ref"
LIB = OUT_DIR / "libbiofem_ref.so"
LIB_DYN = OUT_DIR / "libbiofem_ref_dyn.so"
CUBIN = OUT_DIR / "ref_cuda_kernel.cubin"
REF_SOURCES = ["active_strain.c", "math.c", "bending.c", "io.c", "external.c"]
DYN_SOURCES = ["main.c", "material.c"]
# -ffp-contract=off keeps every multiply and add separately rounded, so the
# reference build and the restated oracle agree bit for bit on any host.
CFLAGS = ["-O2", "-ffp-contract=off", "-fPIC", "-w", "-std=gnu11"]


def available() -> bool:
    return (REFERENCE / "src" / "active_strain.c").is_file()


def _inc() -> list[str]:
    return ["-I", str(HERE / "petsc_lite"), "-iquote", str(REFERENCE / "include")]


def _compile(src: Path, obj: Path, extra: list[str], verbose: bool) -> Path:
    cmd = ["gcc", "-c", *CFLAGS, *extra, *_inc(), str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return obj


def _stale(lib: Path, deps: list[Path]) -> bool:
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> Path | None:
    """Compile libbiofem_ref.so; returns its path, or None without the reference."""
    if not available():
        return None
    srcs = [REFERENCE / "src" / s for s in REF_SOURCES]
    srcs += [HERE / "petsc_lite" / "petsc_lite.c", HERE / "ref_driver.c"]
    deps = srcs + list((HERE / "petsc_lite").glob("*.h"))
    if not force and not _stale(LIB, deps):
        return LIB
    OUT_DIR.mkdir(exist_ok=True)
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(lambda s: _compile(s, OUT_DIR / (s.stem + ".o"), [], verbose), srcs))
    subprocess.run(["gcc", "-shared", "-o", str(LIB), *map(str, objs), "-lm"], check=True)
    for o in objs:
        o.unlink()
    return LIB


def build_dyn(force: bool = False, verbose: bool = False) -> Path | None:
    """Compile libbiofem_ref_dyn.so (the hot path plus main.c and material.c);
    returns its path, or None without the reference."""
    if not available():
        return None
    srcs = [REFERENCE / "src" / s for s in REF_SOURCES + DYN_SOURCES]
    srcs += [HERE / "petsc_lite" / "petsc_lite.c", HERE / "ref_driver.c"]
    deps = srcs + list((HERE / "petsc_lite").glob("*.h"))
    if not force and not _stale(LIB_DYN, deps):
        return LIB_DYN
    OUT_DIR.mkdir(exist_ok=True)
    work = OUT_DIR / "dyn_obj"
    work.mkdir(exist_ok=True)

    def one(src: Path) -> Path:
        extra = []
        if src.name == "main.c":
            extra = ["-Dmain=biofem_reference_main_unused"]
        elif src.name == "ref_driver.c":
            extra = ["-DREF_DRIVER_WITH_MAIN"]
        return _compile(src, work / (src.stem + ".o"), extra, verbose)

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(one, srcs))
    # the externals nothing here defines: ask the linker, then stub them
    probe = subprocess.run(["gcc", "-shared", "-Wl,--no-undefined", "-o", str(work / "probe.so"), *map(str, objs),
                            "-lm"], capture_output=True, text=True)
    missing = sorted(set(re.findall(r"undefined reference to `([A-Za-z_][A-Za-z0-9_]*)'", probe.stderr)))
    stub = work / "abort_stubs.c"
    with open(stub, "w") as f:
        f.write("/* generated by oracle/build_ref.py: externals the dynamic term never calls */\n")
        f.write("#include <stdio.h>\n#include <stdlib.h>\n")
        for name in missing:
            f.write(f"int {name}(void) {{ fprintf(stderr, \"oracle/_ref: {name} is off the dynamic path\\n\"); "
                    f"abort(); }}\n")
    stub_o = _compile(stub, work / "abort_stubs.o", [], verbose)
    subprocess.run(["gcc", "-shared", "-Wl,--no-undefined", "-o", str(LIB_DYN), *map(str, objs), str(stub_o),
                    "-lm"], check=True)
    for o in list(objs) + [stub_o, stub, work / "probe.so"]:
        if o.exists():
            o.unlink()
    work.rmdir()
    return LIB_DYN


def build_cuda(force: bool = False, verbose: bool = False) -> Path | None:
    """Compile the reference's src/cuda_kernel.cu (device code) into
    ref_cuda_kernel.cubin for sm_103a; returns its path, or None without the
    reference sources or nvcc."""
    src = REFERENCE / "src" / "cuda_kernel.cu"
    if not src.is_file():
        return None
    deps = [src, REFERENCE / "include" / "cuda_bridge.h", REFERENCE / "include" / "variables.h"]
    deps += list((HERE / "petsc_lite").glob("*.h"))
    if not force and not _stale(CUBIN, [d for d in deps if d.exists()]):
        return CUBIN
    OUT_DIR.mkdir(exist_ok=True)
    cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-w",
           "-I", str(HERE / "petsc_lite"), "-I", str(REFERENCE / "include"), str(src), "-o", str(CUBIN)]
    if verbose:
        print(" ".join(cmd))
    try:
        subprocess.run(cmd, check=True)
    except FileNotFoundError:
        return None
    return CUBIN


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose=True)
    print(p if p else "reference sources not present; nothing built")
    p = build_dyn(force="--force" in sys.argv, verbose=True)
    print(p if p else "reference sources not present; nothing built")
    p = build_cuda(force="--force" in sys.argv, verbose=True)
    print(p if p else "reference CUDA sources or nvcc not present; nothing built")
