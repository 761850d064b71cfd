"""Converged load step of C1 from the restated oracle (GPU-independent):
Newton with the oracle's exact sparse Jacobian and a direct solve, to
||R|| <= 1e-10 ||R0||.  Writes tests/golden/C1_newton.npz.

    python tests/golden/make_newton_golden.py
"""
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "biofem-ia_gb300"))

from biofem import configs  # noqa: E402
from oracle.pyoracle import Oracle  # noqa: E402


def main(name="C1"):
    w = {"C1": configs.C1}[name]
    m = w.build_mesh()
    o = Oracle().setup(m, w, configs.MU, configs.BULK, configs.H0)
    o.set_threads(8)
    topo = o.topology()
    x0 = w.initial_x(m, topo.xyz0_full)
    t = time.time()
    x, hist = o.newton(x0, topo, verbose=True)
    print(f"{len(hist) - 1} Newton iterations, {time.time() - t:.1f} s, |R| {hist[0]:.3e} -> {hist[-1]:.3e}")
    np.savez_compressed(Path(__file__).parent / f"{w.name}_newton.npz", x0=x0, x=x, rhist=np.array(hist))


if __name__ == "__main__":
    main()
