"""FP32-bulk form: the residual runs on the FP32 pipe in float-float
numbers (about 48 significant bits); the tangent (subdivision basis, tangent
vectors, curvature, df/dy, K values) in FP32 on patch-local shifted
coordinates.

Stated tolerances for the FP32-bulk form:
  ||R32 - R_o||_2 <= 1e-10 ||R_o||_2  (R_o the oracle's FP64 residual; the
                                       FP32-bulk form's budget is 1e-6),
  ||K32 - K64||_F <= 2e-5 ||K64||_F,  ||K32 v - J v||_2 <= 2e-5 ||J v||_2
(J v = exact dual-number directional derivative of the oracle residual).
"""
import numpy as np
import pytest

from biofem import configs

pytestmark = pytest.mark.gpu


def pair(w):
    from biofem.gpu import GpuShell, BIOFEM_FP32_BULK
    m = w.build_mesh()
    s64 = GpuShell(m, w, configs.MU, configs.BULK, configs.H0)
    s32 = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, precision=BIOFEM_FP32_BULK)
    return m, s64, s32


@pytest.mark.parametrize("w", [configs.C1, configs.small(12, 9, activation="random", index=70, pressure=1e-3),
                               configs.cone(10), configs.capped(12, 6, True),
                               configs.SphereWorkload("sphere_f4_holed", 4, index=72, drop=(5, 200)), configs.C2],
                         ids=lambda w: w.name)
def test_fp32_bulk_tangent_error(w, oracle_lib):
    m, s64, s32 = pair(w)
    t = s64.topology()
    x = w.initial_x(m, t["xyz0_full"])
    R64, K64 = s64.form_jacobian(x)
    R32, K32 = s32.form_jacobian(x)
    assert K32.dtype == np.float32
    frob = np.linalg.norm(K32.astype(np.float64) - K64) / np.linalg.norm(K64)
    assert frob <= 2e-5, frob
    o = oracle_lib.setup_given_topology(m, w, t, configs.MU, configs.BULK, configs.H0)
    o.set_threads(8)
    v = np.random.default_rng(11).standard_normal(x.size)
    Ro, Jv = o.jvp(x, v)
    nreal = 3 * m.n_v
    errR32 = np.linalg.norm(R32 - Ro) / np.linalg.norm(Ro)
    assert errR32 <= 1e-10, errR32                    # float-float residual against the FP64 oracle
    assert np.linalg.norm(R64 - Ro) <= 1e-10 * np.linalg.norm(Ro)
    Kv = s32.to_scipy(K32) @ v
    assert np.linalg.norm(Kv[:nreal] - Jv[:nreal]) <= 2e-5 * np.linalg.norm(Jv[:nreal])
    Kv64 = s64.to_scipy(K64) @ v                      # the FP64 tangent at full size, against the oracle
    assert np.linalg.norm(Kv64[:nreal] - Jv[:nreal]) <= 1e-9 * np.linalg.norm(Jv[:nreal])
    s64.close()
    s32.close()


def test_fp32_bulk_is_deterministic():
    w = configs.small(16, 12, index=71)
    m, s64, s32 = pair(w)
    x = w.initial_x(m, s64.topology()["xyz0_full"])
    _, K1 = s32.form_jacobian(x)
    _, K2 = s32.form_jacobian(x)
    assert np.array_equal(K1, K2)
    s64.close()
    s32.close()
