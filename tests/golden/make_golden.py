"""Generate tests/golden/*.npz from the reference's own C code.

Run where the reference sources exist (they are compiled by
oracle/build_ref.py into oracle/_ref/libbiofem_ref.so):

    python tests/golden/make_golden.py

Each fixture holds the workload parameters (flat sheets, LV caps, cone
discs with one extraordinary vertex, a closed sphere), the reference topology tables
(GlobalGhostInit/IrrVer/Patch output), the SNES iterate x and the reference
residual R, Fint and Fext for that x, plus per-element stress / C33 / geometry
for a few sample elements.  Larger meshes store checksums and a strided
sample of R instead of full arrays to keep fixtures small (C2 with --c2,
the full-size ellipsoid C4 with --c4).
"""
from __future__ import annotations

import hashlib
import json
import sys
from dataclasses import replace
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "biofem-ia_gb300"))

from biofem import configs  # noqa: E402
from oracle.pyoracle import RefOracle  # noqa: E402

OUT = Path(__file__).resolve().parent


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def workload_dict(w) -> dict:
    extra = dict(dead_load=w.dead_load, iso_act=w.iso_act) if (w.dead_load or w.iso_act) else {}
    if isinstance(w, configs.SphereWorkload):
        return dict(kind="sphere", name=w.name, freq=w.freq, index=w.index, n_qp=w.n_qp, c33_iters=w.c33_iters,
                    pressure=w.pressure, lambda_a=w.lambda_a, jitter=w.jitter, disp_rel=w.disp_rel,
                    mu=configs.MU, bulk=configs.BULK, h0=configs.H0, **extra)
    if isinstance(w, configs.ConeWorkload):
        return dict(kind="cone", name=w.name, valence=w.valence, rings=w.rings, index=w.index, n_qp=w.n_qp,
                    c33_iters=w.c33_iters, pressure=w.pressure, z_sigma=w.z_sigma, disp_rel=w.disp_rel,
                    mu=configs.MU, bulk=configs.BULK, h0=configs.H0, **extra)
    if isinstance(w, configs.CappedLVWorkload):
        return dict(kind="capped", name=w.name, n_phi=w.n_phi, n_theta=w.n_theta, apex_vertex=w.apex_vertex,
                    clamp=w.clamp, index=w.index, n_qp=w.n_qp, c33_iters=w.c33_iters, pressure=w.pressure,
                    jitter=w.jitter, disp_rel=w.disp_rel, mu=configs.MU, bulk=configs.BULK, h0=configs.H0, **extra)
    if isinstance(w, configs.LVWorkload):
        return dict(kind="lv", name=w.name, freq=w.freq, index=w.index, n_qp=w.n_qp, c33_iters=w.c33_iters,
                    pressure=w.pressure, lambda_a=w.lambda_a, nflip=w.nflip, jitter=w.jitter,
                    mu=configs.MU, bulk=configs.BULK, h0=configs.H0, **extra)
    return dict(name=w.name, nx=w.nx, ny=w.ny, n_qp=w.n_qp, c33_iters=w.c33_iters, pressure=w.pressure,
                z_sigma=w.z_sigma, activation=w.activation, lambda_a=w.lambda_a, disp_rel=w.disp_rel,
                index=w.index, mu=configs.MU, bulk=configs.BULK, h0=configs.H0, **extra)


def make(w, full: bool, sample_elems=(0, 1, 5, 17)):
    m = w.build_mesh()
    ref = RefOracle().setup(m, w, configs.MU, configs.BULK, configs.H0)
    t = ref.topology()
    x = w.initial_x(m, t.xyz0_full)
    R, Fi, Fe = ref.residual(x, want_parts=True)
    meta = workload_dict(w)
    meta.update(n_v=m.n_v, n_elmt=m.n_elmt, n_ghosts=ref.n_ghosts,
                sha_patch=sha(t.patch), sha_ire=sha(t.ire), sha_val=sha(t.val), sha_irv=sha(t.irv),
                sha_gtri=sha(t.gtri), sha_R=sha(R), norm_R=float(np.linalg.norm(R)),
                norm_Fint=float(np.linalg.norm(Fi)), norm_Fext=float(np.linalg.norm(Fe)))
    data = dict(meta=np.array(json.dumps(meta)))
    if full:
        data.update(patch=t.patch, ire=t.ire, val=t.val, irv=t.irv, gtri=t.gtri, xyz0_full=t.xyz0_full,
                    dA0=t.dA0, x=x, R=R, Fint=Fi, Fext=Fe)
        S, C33, G = [], [], []
        for ec in sample_elems:
            s, c, g = ref.elem_state(ec, w.n_qp)
            S.append(s); C33.append(c); G.append(g)
        # irregular samples too
        irr = list(np.nonzero(t.ire)[0][:4])
        if m.n_elmt_base > 0:                       # apex-cap triangles
            irr += [m.n_elmt_base, m.n_elmt - 1]
        for ec in irr:
            s, c, g = ref.elem_state(int(ec), w.n_qp)
            S.append(s); C33.append(c); G.append(g)
        data.update(sample_elems=np.array(list(sample_elems) + [int(e) for e in irr], np.int32),
                    sample_S=np.array(S), sample_C33=np.array(C33), sample_geom=np.array(G))
    else:
        stride = 97
        data.update(R_idx=np.arange(0, R.size, stride, dtype=np.int64), R_sample=R[::stride],
                    ire=t.ire, val=t.val)
    path = OUT / f"{w.name}.npz"
    np.savez_compressed(path, **data)
    print(f"wrote {path} ({path.stat().st_size/1024:.1f} KiB)  |R|={meta['norm_R']:.6e}")


CASES_FULL = [
    configs.small(6, 5),
    configs.small(9, 7, activation="uniform", lambda_a=0.8, index=11),
    configs.small(12, 8, n_qp=5, c33_iters=1, index=12, pressure=1e-3),
    configs.small(10, 6, n_qp=2, c33_iters=4, activation="random", index=13),
    configs.C1,
    # truncated ellipsoid caps: interior valence 5/7 and jagged-rim irregular patches
    configs.LVWorkload("lv_f3", 3, index=40),
    configs.LVWorkload("lv_f4_q5", 4, index=41, n_qp=5, c33_iters=2, pressure=5e-4),
    # the dead-load pressure (SurfaceConstNormalPressure) and the isotropic active gradient (-cart_fib_act 0)
    replace(configs.small(8, 7, index=14, pressure=2e-3, dead_load=1), name="flat_8x7_dead_load"),
    replace(configs.small(9, 6, index=15, activation="random", iso_act=1), name="flat_9x6_isotropic"),
    configs.LVWorkload("lv_f3_iso_dead", 3, index=42, iso_act=1, dead_load=1),
    # one interior vertex of valence 3, 8 and 10: the one-step subdivision at its
    # smallest valence (rows overwriting rows) and up to the 16-node patch
    configs.cone(3),
    configs.cone(8, n_qp=4),
    configs.cone(10),
    # a closed surface: no boundary ring, no ghost nodes, nothing clamped
    configs.SphereWorkload("sphere_f5", 5, index=70),
    # apex-cap triangles (ibm->n_elmt_base): a fan over the apex ring, and a
    # fan from an apex node with the apex ring clamped
    configs.capped(10, 5),
    configs.capped(12, 6, True, clamp=True, n_qp=4),
]

if __name__ == "__main__":
    only = [a for a in sys.argv[1:] if not a.startswith("--")]
    for w in CASES_FULL:
        if not only or w.name in only:
            make(w, full=True)
    if "--c2" in sys.argv:
        make(configs.C2, full=False)
    if "--c4" in sys.argv:   # the reference's O(N^2) Patch() on 200k triangles: tens of minutes
        make(configs.C4, full=False)
