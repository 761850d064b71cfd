"""Build recipe for oracle/_ref/libbiofem_ref.so (TEST INFRASTRUCTURE ONLY).

Compiles the reference's own, unmodified hot-path C files where they lie
(``/root/reference/src/{active_strain,math,bending,io,external}.c``) together
with the petsc-lite shim (oracle/petsc_lite/) and the np = 1 driver
(oracle/ref_driver.c).  The result is the checker that pins the restated oracle
and generates tests/golden/.  It is built only where the reference sources
exist; nothing on the product path links it.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
REFERENCE = Path("/root/reference")
OUT_DIR = HERE / "_ref"
LIB = OUT_DIR / "libbiofem_ref.so"
REF_SOURCES = ["active_strain.c", "math.c", "bending.c", "io.c", "external.c"]
# -ffp-contract=off keeps every multiply and add separately rounded, so the
# reference build and the restated oracle agree bit for bit on any host.
CFLAGS = ["-O2", "-ffp-contract=off", "-fPIC", "-w", "-std=gnu11"]


def available() -> bool:
    return (REFERENCE / "src" / "active_strain.c").is_file()


def build(force: bool = False, verbose: bool = False) -> Path | None:
    """Compile libbiofem_ref.so; returns its path, or None without the reference."""
    if not available():
        return None
    srcs = [REFERENCE / "src" / s for s in REF_SOURCES]
    srcs += [HERE / "petsc_lite" / "petsc_lite.c", HERE / "ref_driver.c"]
    deps = srcs + list((HERE / "petsc_lite").glob("*.h"))
    if LIB.exists() and not force:
        t = LIB.stat().st_mtime
        if all(p.stat().st_mtime <= t for p in deps):
            return LIB
    OUT_DIR.mkdir(exist_ok=True)
    inc = ["-I", str(HERE / "petsc_lite"), "-iquote", str(REFERENCE / "include")]
    objs = []

    def compile_one(src: Path) -> Path:
        obj = OUT_DIR / (src.stem + ".o")
        cmd = ["gcc", "-c", *CFLAGS, *inc, str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, srcs))
    cmd = ["gcc", "-shared", "-o", str(LIB), *map(str, objs), "-lm"]
    subprocess.run(cmd, check=True)
    for o in objs:
        o.unlink()
    return LIB


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose=True)
    print(p if p else "reference sources not present; nothing built")
