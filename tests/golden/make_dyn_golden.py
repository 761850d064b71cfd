"""Generate tests/golden/dyn_*.npz: the reference's own dynamic term.

Run where the reference sources exist (oracle/build_ref.py compiles
oracle/_ref/libbiofem_ref_dyn.so: the hot-path files plus the reference's
src/main.c and src/material.c, driven by oracle/ref_driver.c):

    python tests/golden/make_dyn_golden.py

For a free-edged flat membrane and a clamped geodesic LV cap, one seeded state
(x, xn, xnm1, xd, xdd) per case, the fixture stores what the reference's own
code returns:
  * FDynamic (main.c:1157-1364) for Newmark (gamma 0.6, damped) and central
    differences (damped), on the path of an active-strain run (the DMPlex
    context initialised, main.c:326-331) and, for comparison, on the serial
    path (every triangle, ghost and bridging ones included);
  * xAccVel (main.c:1367-1412) on both paths.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "biofem-ia_gb300"))

from biofem import configs  # noqa: E402
from oracle.pyoracle import RefOracle  # noqa: E402

OUT = Path(__file__).resolve().parent
CASES = {
    "dyn_flat_6x5": (configs.small(6, 5, index=93, pressure=0.0), False),
    "dyn_lv_f2": (configs.LVWorkload("lv_f2", 2, index=94), True),
}
DT, RHO, DAMPF = 2e-3, 1.3, 7.0
SCHEMES = {"newmark": (0, 0.6), "central": (1, 0.5)}


def make(name, w, clamp):
    m = w.build_mesh()
    ref = RefOracle(dyn=True).setup(m, w, configs.MU, configs.BULK, configs.H0, clamp=clamp)
    t = ref.topology()
    x = w.initial_x(m, t.xyz0_full)
    rng = np.random.default_rng(95)
    n = x.size
    st = dict(x=x + 1e-3 * rng.standard_normal(n), xn=x + 1e-3 * rng.standard_normal(n),
              xnm1=x + 1e-3 * rng.standard_normal(n), xd=rng.standard_normal(n), xdd=rng.standard_normal(n))
    out = dict(st)
    out["clamp"] = np.array(int(clamp))
    out["consts"] = np.array([DT, RHO, DAMPF])
    for tag, (ti, G) in SCHEMES.items():
        ref.set_dynamics(DT, RHO, G, DAMPF, ti, 1)
        for path, dm in (("dmplex", True), ("serial", False)):
            out[f"Fdyn_{tag}_{path}"] = ref.fdynamic(st["x"], st["xn"], st["xnm1"], st["xd"], st["xdd"], dmplex=dm)
            xd, xdd = ref.xaccvel(st["x"], st["xn"], st["xd"], st["xdd"], dmplex=dm)
            out[f"xd_{tag}_{path}"] = xd
            out[f"xdd_{tag}_{path}"] = xdd
        out[f"gamma_{tag}"] = np.array(G)
    np.savez_compressed(OUT / f"{name}.npz", **out)
    print(name, m.n_elmt, "triangles")


if __name__ == "__main__":
    for name, (w, clamp) in CASES.items():
        make(name, w, clamp)
