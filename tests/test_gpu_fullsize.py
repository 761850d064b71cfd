"""Parity at the full workload sizes: the device residual and tangent of C2
(98,304 triangles), C4 (the 200,614-triangle truncated ellipsoid with
valence-5/7 vertices) and C3 (1,572,864 triangles, 6 thickness points)
against the oracle evaluated on the whole mesh (its O(N) topology scans, the
reference's tables bit for bit; OpenMP over elements), and C4's residual
against the reference build's own strided sample
(tests/golden/C4_lv_ellipsoid.npz, tests/golden/make_golden.py --c4).

C3 runs two extensions of the reference's formulation (the exact basis
tables and the tangential thickness metric; at h ~ h0/10 the reference's
four-decimal tables and its a3,alpha fold the thickness points), so its
oracle is the restated oracle with the same switches: the builder's
formulation, not the reference's algebra.

Tolerances:
  residual   ||R - R_o||_2 <= 1e-10 ||R_o||_2 and max |R - R_o| <= 1e-12 max |Fint_o|
             (FP32-bulk float-float: 1e-10 max |Fint_o|); C4: 1e-9 ||R_o||_2 and
             1e-8 max |Fint_o| -- its reference-state residual is the small
             imbalance of prestressed element forces, and on its strongly bent
             patches (C33 down to 0.36 at the outer thickness point) the
             device's closed-form stress and the oracle's loops round apart by
             up to ~1e-9 of the force scale (measured 2.0e-10 of ||R||, 1.2e-9
             of max |Fint|);
  tangent    FP64: ||K v - J v||_2 <= 1e-9 ||J v||_2 on the real rows (J v the
             oracle's exact dual-number derivative); FP32-bulk: 2e-5 (C2, C3),
             5e-4 (C4, whose distorted and extraordinary patches carry the
             largest FP32 rounding; the measured error is printed).
"""
import json
import os

import numpy as np
import pytest

from biofem import configs
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

THREADS = max(1, os.cpu_count() or 1)


def oracle_on(w, m):
    from oracle.pyoracle import Oracle
    o = Oracle().set_fast_topology(True)
    try:
        o.setup(m, w, configs.MU, configs.BULK, configs.H0)
    finally:
        o.set_fast_topology(False)
    o.set_threads(THREADS)
    return o


def check_case(w, tol32, tolR=1e-10, tolF=1e-12):
    from biofem.gpu import GpuShell, BIOFEM_FP32_BULK
    m = w.build_mesh()
    o = oracle_on(w, m)
    s64 = GpuShell(m, w, configs.MU, configs.BULK, configs.H0)
    t = s64.topology()
    assert np.array_equal(t["patch"], o.topology().patch)
    x = w.initial_x(m, t["xyz0_full"])
    v = np.random.default_rng(8).standard_normal(x.size)
    Ro, Jv = o.jvp(x, v)
    fint = np.abs(o.residual_parts(x)[1]).max()
    R, K = s64.form_jacobian(x)
    errR = np.linalg.norm(R - Ro) / np.linalg.norm(Ro)
    real = slice(0, 3 * m.n_v)
    Kv = s64.to_scipy(K) @ v
    errK = np.linalg.norm((Kv - Jv)[real]) / np.linalg.norm(Jv[real])
    s64.close()
    s32 = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, precision=BIOFEM_FP32_BULK)
    R32, K32 = s32.form_jacobian(x)
    Kv32 = s32.to_scipy(K32) @ v
    errK32 = np.linalg.norm((Kv32 - Jv)[real]) / np.linalg.norm(Jv[real])
    errR32 = np.linalg.norm(R32 - Ro) / np.linalg.norm(Ro)
    s32.close()
    print(f"{w.name}: R {errR:.2e}, K v FP64 {errK:.2e}; FP32-bulk R {errR32:.2e}, K v {errK32:.2e}")
    assert errR <= tolR, errR
    assert np.abs(R - Ro).max() <= tolF * fint
    assert errK <= 1e-9, errK
    assert errR32 <= tolR, errR32
    assert np.abs(R32 - Ro).max() <= max(tolF, 1e-10) * fint
    assert errK32 <= tol32, errK32
    return m, x, R


def test_C2_full_tangent_against_oracle():
    check_case(configs.C2, 2e-5)


def test_C4_full_against_oracle_and_reference_sample():
    m, x, R = check_case(configs.C4, 5e-4, tolR=1e-9, tolF=1e-8)
    d = np.load(GOLDEN / "C4_lv_ellipsoid.npz")
    meta = json.loads(str(d["meta"]))
    ref = d["R_sample"]   # the reference state: the fixture's iterate
    assert np.linalg.norm(R[d["R_idx"]] - ref) <= 1e-9 * np.linalg.norm(ref)
    assert abs(np.linalg.norm(R) - meta["norm_R"]) <= 1e-9 * meta["norm_R"]


def test_C3_full_against_oracle_with_the_same_extensions():
    check_case(configs.C3, 2e-5)
