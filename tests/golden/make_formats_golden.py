"""Generate tests/golden/formats_*.npz: the reference's own on-disk output.

Run where the reference sources exist (oracle/build_ref.py compiles them with
the driver oracle/ref_driver.c):

    python tests/golden/make_formats_golden.py

For one seeded state of a small flat membrane and of the geodesic LV cap the
reference writes, through its own io.c functions:
  * LocationOut checkpoints on the DMPlex path (raw big-endian, original-vertex
    order) and on the serial path (VecView records), io.c:1272-1376;
  * the Output surface VTK file, io.c:540-964 (Fint / Fext from its own residual
    at x, Fdyn and the velocity given, Init's nodal mass);
  * UpdateElementThickness and the Write3DShellVTK file, active_strain.c:2198,
    io.c:983-1064.
The fixture keeps the inputs, the reference's Fint / Fext / thickness, the
SHA-256 of every file and the text of the VTK files.
"""
from __future__ import annotations

import hashlib
import json
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "biofem-ia_gb300"))

from biofem import configs  # noqa: E402
from oracle.pyoracle import RefOracle  # noqa: E402

OUT = Path(__file__).resolve().parent
CASES = {
    "formats_flat_6x5": (configs.small(6, 5, activation="random", index=90, pressure=1e-3), False),
    "formats_lv_f2": (configs.LVWorkload("lv_f2", 2, index=91), True),
}
RHO = 1.1
TI = 7


def files_of(d: Path) -> dict:
    return {p.name: p.read_bytes() for p in sorted(d.iterdir())}


def make(name, w, lv):
    m = w.build_mesh()
    ref = RefOracle().setup(m, w, configs.MU, configs.BULK, configs.H0)
    t = ref.topology()
    x = w.initial_x(m, t.xyz0_full)
    rng = np.random.default_rng(92)
    n = x.size
    state = dict(x=x, xn=x + 1e-3 * rng.standard_normal(n), xd=rng.standard_normal(n), xdd=rng.standard_normal(n))
    Fdyn = 1e-2 * rng.standard_normal(n)
    R, Fint, Fext = ref.residual(x, want_parts=True)
    data = dict(Fdyn=Fdyn, Fint=Fint, Fext=Fext, **state)
    hashes = {}
    with tempfile.TemporaryDirectory(prefix="fmt") as tmp:
        for tag, dmplex in (("ckpt_vertex", True), ("ckpt_vec", False)):
            d = Path(tmp) / tag
            d.mkdir()
            ref.location_out(str(d), TI, state["x"], state["xn"], state["xd"], state["xdd"], ibi=0, dmplex=dmplex)
            back = ref.location_in(str(d), TI, ibi=0, dmplex=dmplex)
            for k in back:
                assert np.array_equal(back[k], state[k]), (tag, k)
            for fn, b in files_of(d).items():
                hashes[f"{tag}/{fn}"] = hashlib.sha256(b).hexdigest()
        d = Path(tmp) / "vtk"
        d.mkdir()
        ref.output_vtk(str(d), TI, x, Fdyn, state["xd"], RHO, lv=lv)
        th = ref.thickness(x, str(d), TI)
        data["thickness"] = th
        for fn, b in files_of(d).items():
            hashes[f"vtk/{fn}"] = hashlib.sha256(b).hexdigest()
            data[f"text/{fn}"] = np.frombuffer(b, dtype=np.uint8)
    meta = dict(case=name, lv=lv, rho=RHO, ti=TI, n_v=m.n_v, n_elmt=m.n_elmt, n_ghosts=ref.n_ghosts,
                workload=w.name, index=w.index, sha256=hashes)
    data["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(OUT / f"{name}.npz", **data)
    print(name, m.n_v, m.n_elmt, sorted(hashes))


def workload_of(name):
    return CASES[name][0]


if __name__ == "__main__":
    for name, (w, lv) in CASES.items():
        make(name, w, lv)
