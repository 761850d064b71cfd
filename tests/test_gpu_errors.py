"""Device-side error paths, made on the host: a NaN coordinate makes CC3333
fail its |CC3333| > 1e-14 test (ModElemC33, active_strain.c:1676) inside the
element kernels, which set the status word the host turns into
PETSC_ERR_FP (72); the handle stays usable and the next call is clean.  No
kernel faults, traps or waits on this path."""
import numpy as np
import pytest

from biofem import configs
from biofem.gpu import BiofemError, GpuShell

pytestmark = pytest.mark.gpu

W = configs.small(8, 6, activation="random", index=99, pressure=1e-3)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32_bulk"])
def test_nan_state_reports_fp_error_and_recovers(precision):
    m = W.build_mesh()
    sh = GpuShell(m, W, configs.MU, configs.BULK, configs.H0, precision=precision)
    x = W.initial_x(m, sh.topology()["xyz0_full"])
    R0 = sh.form_function(x)
    _, K0 = sh.form_jacobian(x)
    bad = x.copy()
    bad[3 * (m.n_v // 2) + 2] = np.nan
    for call in (sh.form_function, sh.form_jacobian, sh.residual_parts, sh.element_thickness):
        with pytest.raises(BiofemError) as e:
            call(bad)
        assert e.value.code == 72
        # the status word was cleared: the same handle gives the clean results again
        np.testing.assert_array_equal(sh.form_function(x), R0)
    _, K1 = sh.form_jacobian(x)
    np.testing.assert_array_equal(K1, K0)
    sh.close()


def test_newton_from_nan_state_stops():
    m = W.build_mesh()
    sh = GpuShell(m, W, configs.MU, configs.BULK, configs.H0)
    x = W.initial_x(m, sh.topology()["xyz0_full"])
    bad = x.copy()
    bad[5] = np.nan
    with pytest.raises(BiofemError) as e:    # refused at the initial residual
        sh.newton(bad, max_newton=3)
    assert e.value.code == 72
    x1, st = sh.newton(x, rtol=1e-10)   # a clean solve on the same handle afterwards
    assert st["converged"] and np.isfinite(x1).all()
    sh.close()
