"""GPU parity: the sm_103a residual and tangent against the oracle / golden
fixtures, through the C-ABI (libbiofem_gpu.so).

Tolerances (FP64 plain path):
  residual   ||R_gpu - R_ref||_2 <= 1e-10 * ||R_ref||_2 and per-entry
             |R_gpu - R_ref| <= 1e-12 * max|Fint| + 4 d_ulp (rounding of the
             closed-form stress vs the reference's 3^6 / 3^8 loops, and of fused
             multiply-add), d_ulp = the largest change of the oracle residual
             when x moves by one rounding (x (1 + 2^-52 z), z ~ N(0, 1), three
             draws): the residual's own rounding floor, which exceeds
             1e-12 max|Fint| where stiff rows carry little net force;
  tangent    ||K v - J v||_2 <= 1e-9 * ||J v||_2 on the non-ghost rows, where
             J v is the exact (dual-number) directional derivative of the
             oracle residual; ghost rows of K are identity.
"""
import json

import numpy as np
import pytest

from conftest import GOLDEN, golden_case
from biofem import configs
from biofem.configs import Workload

pytestmark = pytest.mark.gpu

FULL = sorted(p for p in GOLDEN.glob("*.npz") if "R" in np.load(p))


def load_case(path):
    return golden_case(path)


def shell_for(m, w):
    from biofem.gpu import GpuShell
    return GpuShell(m, w, configs.MU, configs.BULK, configs.H0)


def rounding_floor(o, x):
    """Largest change of the oracle residual under a one-rounding relative
    perturbation of x (three seeded draws)."""
    R0 = o.residual(x)
    rng = np.random.default_rng(17)
    return max(np.abs(o.residual(x * (1.0 + 2.0 ** -52 * rng.standard_normal(x.size))) - R0).max()
               for _ in range(3))


@pytest.mark.parametrize("path", FULL, ids=lambda p: p.stem)
def test_residual_matches_reference_golden(path, oracle_lib):
    w, meta, d = load_case(path)
    m = w.build_mesh()
    sh = shell_for(m, w)
    t = sh.topology()
    assert np.array_equal(t["patch"], d["patch"])
    R = sh.form_function(d["x"])
    Rref = d["R"]
    err = np.linalg.norm(R - Rref)
    assert err <= 1e-10 * np.linalg.norm(Rref), (err, np.linalg.norm(Rref))
    floor = rounding_floor(oracle_lib.setup(m, w, meta["mu"], meta["bulk"], meta["h0"]), d["x"])
    assert np.abs(R - Rref).max() <= 1e-12 * np.abs(d["Fint"]).max() + 4 * floor
    sh.close()


def test_residual_is_deterministic():
    w = configs.C1
    m = w.build_mesh()
    sh = shell_for(m, w)
    x = w.initial_x(m, sh.topology()["xyz0_full"])
    x = x + 1e-4 * np.random.default_rng(0).standard_normal(x.size)
    R1 = sh.form_function(x)
    R2 = sh.form_function(x)
    _, K1 = sh.form_jacobian(x)
    _, K2 = sh.form_jacobian(x)
    assert np.array_equal(R1, R2) and np.array_equal(K1, K2)
    sh.close()


@pytest.mark.parametrize("wl", [configs.small(8, 6, index=40), configs.small(9, 7, activation="random", index=41, n_qp=4, c33_iters=2),
                                configs.small(12, 8, activation="uniform", lambda_a=0.85, index=42, pressure=1e-3, n_qp=5, c33_iters=1),
                                configs.small(10, 8, activation="random", index=44, n_qp=6, pressure=1e-4),
                                configs.small(11, 8, activation="random", index=45, n_qp=6, basis=1),
                                configs.small(12, 9, index=46, basis=1, tnormal=1, pressure=1e-3),
                                configs.LVWorkload("lv_f4", 4, index=47),
                                configs.small(8, 7, index=48, pressure=2e-3, dead_load=1),
                                configs.small(9, 6, activation="random", index=49, iso_act=1),
                                configs.LVWorkload("lv_f3", 3, index=50, iso_act=1, dead_load=1),
                                configs.cone(3), configs.cone(9, n_qp=5), configs.cone(10),
                                configs.SphereWorkload("sphere_f6", 6, index=71),
                                configs.capped(10, 5), configs.capped(12, 6, True, clamp=True, n_qp=4),
                                configs.capped(16, 8, True, pressure=2e-3),
                                configs.SphereWorkload("sphere_f4_holed", 4, index=72, drop=(5, 200)),
                                configs.C1],
                         ids=lambda w: w.name + ("_exact" if w.basis else "") + ("_tnormal" if w.tnormal else "")
                         + ("_dead" if w.dead_load else "") + ("_iso" if w.iso_act else ""))
def test_tangent_matches_oracle_directional_derivative(wl, oracle_lib):
    m = wl.build_mesh()
    o = oracle_lib.setup(m, wl, configs.MU, configs.BULK, configs.H0)
    sh = shell_for(m, wl)
    x = wl.initial_x(m, sh.topology()["xyz0_full"])
    rng = np.random.default_rng(5)
    h = 1.0 / wl.nx if hasattr(wl, "nx") else m.meta["hmean"]
    x[: 3 * m.n_v] += 1e-3 * h * rng.standard_normal(3 * m.n_v)
    R, K = sh.form_jacobian(x)
    Rres = sh.form_function(x)
    assert np.array_equal(R, Rres)  # the tangent pass returns the same residual
    Ks = sh.to_scipy(K)
    ghost = np.zeros(sh.n_dof, bool)
    ghost[3 * m.n_v:] = True
    for k in range(3):
        v = rng.standard_normal(sh.n_dof)
        Ro, Jv = o.jvp(x, v)
        Kv = Ks @ v
        assert np.linalg.norm(Kv[~ghost] - Jv[~ghost]) <= 1e-9 * np.linalg.norm(Jv[~ghost])
        np.testing.assert_array_equal(Kv[ghost], v[ghost])
    np.testing.assert_allclose(R, Ro, rtol=0, atol=1e-12 * max(1e-30, np.abs(Ro).max()) + 1e-17
                               + 4 * rounding_floor(o, x))
    sh.close()


def test_tangent_dense_small_mesh(oracle_lib):
    w = configs.small(5, 4, index=43)
    m = w.build_mesh()
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0)
    sh = shell_for(m, w)
    x = w.initial_x(m, sh.topology()["xyz0_full"])
    J = o.jacobian_dense(x)
    _, K = sh.form_jacobian(x)
    Kd = sh.to_scipy(K).toarray()
    nreal = 3 * m.n_v
    scale = np.abs(J[:nreal, :nreal]).max()
    assert np.abs(Kd[:nreal, :nreal] - J[:nreal, :nreal]).max() <= 1e-10 * scale
    # ghost columns are folded into real columns: the oracle's J has none
    assert not J[:nreal, nreal:].any() and not Kd[:nreal, nreal:].any()
    np.testing.assert_array_equal(Kd[nreal:, nreal:], np.eye(sh.n_dof - nreal))
    sh.close()


def test_residual_C2_sample_matches_reference():
    """C2 (98,304 triangles, 3 qp, 3 C33 iterations): strided sample of the
    reference residual stored in the fixture."""
    d = np.load(GOLDEN / "C2_flat_256x192.npz")
    meta = json.loads(str(d["meta"]))
    w = configs.C2
    m = w.build_mesh()
    sh = shell_for(m, w)
    x = w.initial_x(m, sh.topology()["xyz0_full"])
    R = sh.form_function(x)
    Rs = R[d["R_idx"]]
    ref = d["R_sample"]
    assert np.linalg.norm(Rs - ref) <= 1e-10 * np.linalg.norm(ref)
    assert abs(np.linalg.norm(R) - meta["norm_R"]) <= 1e-10 * meta["norm_R"]
    sh.close()


def test_kinematic_checks_C1():
    """Known answers: x = X and no activation gives the reference-state
    residual of the reference (not exactly 0: its truncated basis tables make
    the flat-state curvature 1e-4-sized); clamped rows are x - X exactly."""
    w = Workload("kat", 16, 12, z_sigma=0.0, activation="uniform", lambda_a=1.0, pressure=0.0, index=44)
    m = w.build_mesh()
    sh = shell_for(m, w)
    X = sh.topology()["xyz0_full"].reshape(-1)
    R = sh.form_function(X)
    bn = m.bnodes
    assert np.all(R[3 * bn] == 0.0)
    d = np.zeros_like(X)
    d[3 * bn[0]] = 1e-3
    R2 = sh.form_function(X + d)
    assert R2[3 * bn[0]] == pytest.approx(1e-3, rel=0, abs=1e-18)
    sh.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32_bulk"])
def test_host_call_into_pinned_buffers(precision):
    """RunGpuResidualJacobian with page-locked host buffers: the row assembly
    writes K straight into the mapped buffer; R and K equal the pageable-buffer
    call bitwise."""
    import torch
    from biofem.gpu import GpuShell
    w = configs.small(10, 8, activation="random", index=48, pressure=300.0)   # max|Fext| > 1: R and K scaled
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, precision=precision)
    x = w.initial_x(m, sh.topology()["xyz0_full"])
    R, K = sh.form_jacobian(x)
    hx = torch.tensor(x).pin_memory()
    hR = torch.empty(sh.n_dof, dtype=torch.float64).pin_memory()
    kdt = torch.float64 if precision == 0 else torch.float32
    hK = torch.full((9 * sh.nnzb,), float("nan"), dtype=kdt).pin_memory()
    sh.residual_jacobian_host_ptrs(hx.data_ptr(), hR.data_ptr(), hK.data_ptr())
    np.testing.assert_array_equal(hR.numpy(), R)
    np.testing.assert_array_equal(hK.numpy().reshape(K.shape), K)
    sh.close()


def test_node_ids_beyond_the_reference_sentinel_on_the_device():
    """R and K of a mesh whose node ids all sit at 10^6 and above (the
    reference's 1000000 sentinel among them) equal the small mesh's, shifted:
    the same element and summation order, so bit for bit."""
    import copy
    pad = 1_000_000
    w = configs.small(8, 6, index=96, pressure=1e-3)
    m = w.build_mesh()
    m2 = copy.deepcopy(m)
    m2.xyz0 = np.vstack([np.zeros((pad, 3)), m.xyz0])
    m2.tri = (m.tri + pad).astype(np.int32)
    m2.bnodes = (m.bnodes + pad).astype(np.int32)
    sh, sh2 = shell_for(m, w), shell_for(m2, w)
    x = w.initial_x(m, sh.topology()["xyz0_full"])
    x2 = np.concatenate([np.zeros(3 * pad), x])
    R, K = sh.form_jacobian(x)
    R2, K2 = sh2.form_jacobian(x2)
    np.testing.assert_array_equal(R2[3 * pad:], R)
    v = np.random.default_rng(97).standard_normal(x.size)
    Kv = sh.to_scipy(K) @ v
    Kv2 = sh2.to_scipy(K2) @ np.concatenate([np.zeros(3 * pad), v])
    np.testing.assert_array_equal(Kv2[3 * pad:], Kv)
    sh.close()
    sh2.close()
