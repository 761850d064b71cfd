"""Build recipe for oracle/_build/liboracle.so (TEST INFRASTRUCTURE ONLY).

The restated oracle (oracle/oracle.cpp) is plain C++ with no dependencies; it
builds on any host with g++ (this container and the GPU host alike).
-ffp-contract=off keeps its FP64 results identical across x86-64 and aarch64
(no fused multiply-adds) and bitwise equal to the reference build.
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "liboracle.so"
SRC = HERE / "oracle.cpp"
FLAGS = ["-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c++17", "-fopenmp"]


def build(force: bool = False, verbose: bool = False) -> Path:
    if LIB.exists() and not force and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    OUT_DIR.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["g++", *FLAGS, str(SRC), "-o", str(tmp)]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    tmp.replace(LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
