"""GPU side of the on-disk formats: the force parts and wall thickness the
VTK writers print, and checkpoint / restart of the device time loop.

Tolerances: Fint, Fext, Fdyn per entry within 1e-11 of max|F| against the
oracle (Fint keeps the clamped rows, where R holds x - X instead: their large
internal forces carry the closed-form vs loop rounding, ~1.5e-12 of max|F|); thickness within 1e-12 relative of the
reference's UpdateElementThickness (fixture); a restart from either
checkpoint layout continues bit-identically to the uninterrupted run.
"""
import json

import numpy as np
import pytest

from conftest import GOLDEN
from biofem import configs, io
from biofem.gpu import BIOFEM_CKPT_VEC, BIOFEM_CKPT_VERTEX_ORDER, GpuShell

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dyn", [False, True], ids=["static", "newmark_damped"])
@pytest.mark.parametrize("w", [configs.small(9, 7, activation="random", index=93, pressure=1e-3),
                               configs.LVWorkload("lv_f4", 4, index=94)], ids=lambda w: w.name)
def test_residual_parts_match_oracle(w, dyn, oracle_lib):
    m = w.build_mesh()
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0)
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0)
    x = w.initial_x(m, sh.topology()["xyz0_full"])
    if dyn:
        rng = np.random.default_rng(95)
        st = dict(xn=x + 1e-3 * rng.standard_normal(x.size), xd=rng.standard_normal(x.size),
                  xdd=rng.standard_normal(x.size))
        for side in (o, sh):
            side.set_dynamics(2e-3, 1.2, 0.5, 3.0, 0, 1)
            side.set_dynamic_state(**st)
    R, Fi, Fe, Fd = sh.residual_parts(x)
    Ro, Fio, Feo, Fdo = o.residual_parts(x)
    nr = 3 * m.n_v
    np.testing.assert_array_equal(R, sh.form_function(x))
    for a, b in ((Fi, Fio), (Fe, Feo), (Fd, Fdo)):
        scale = max(np.abs(b[:nr]).max(), 1e-300)
        assert np.abs(a[:nr] - b[:nr]).max() <= 1e-11 * scale
        assert not a[nr:].any()
    assert (np.abs(Fd).max() > 0) == dyn
    if dyn:
        o.set_dynamics(None)
    sh.close()


@pytest.mark.parametrize("path", sorted(GOLDEN.glob("formats_*.npz")), ids=lambda p: p.stem)
def test_element_thickness_matches_reference(path):
    d = np.load(path)
    meta = json.loads(str(d["meta"]))
    w = (configs.small(6, 5, activation="random", index=90, pressure=1e-3) if meta["case"] == "formats_flat_6x5"
         else configs.LVWorkload("lv_f2", 2, index=91))
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0)
    th = sh.element_thickness(d["x"])
    np.testing.assert_allclose(th, d["thickness"], rtol=1e-12, atol=0)
    sh.close()


@pytest.mark.parametrize("layout", [BIOFEM_CKPT_VERTEX_ORDER, BIOFEM_CKPT_VEC], ids=["vertex_order", "vec"])
def test_restart_continues_bitwise(layout, tmp_path):
    from biofem.dynamics import Activation, Dynamics, time_loop
    w = configs.small(8, 6, activation="random", index=96, pressure=1e-3, disp_rel=0.0)
    m = w.build_mesh()
    dyn = Dynamics(dt=5e-3, rho=1.0, dampfactor=2.0, damping=1)
    act = Activation(0.12, ramp_type=2, T=0.02)
    kw = dict(rtol=1e-10, max_newton=30)
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0)
    x0 = w.initial_x(m, sh.topology()["xyz0_full"])
    x_full, _ = time_loop(sh, m, x0, dyn, act, 4, **kw)
    s_full = sh.dynamic_state()
    sh.close()
    # 2 steps, LocationOut at ti = 2, a fresh handle, LocationIn, 2 more steps
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0)
    x2, _ = time_loop(sh, m, x0, dyn, act, 2, **kw)
    io.checkpoint(sh, tmp_path, 2, x2, layout=layout)
    sh.close()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0)
    dyn.apply(sh)
    xr = io.restart(sh, tmp_path, 2)
    np.testing.assert_array_equal(xr, x2)
    x4, _ = time_loop(sh, m, xr, dyn, act, 2, tistart=2, reset_state=False, **kw)
    np.testing.assert_array_equal(x4, x_full)
    s = sh.dynamic_state()
    for k in ("xn", "xd", "xdd"):
        np.testing.assert_array_equal(s[k], s_full[k])
    sh.close()


def test_step_writer_files(tmp_path):
    from biofem.dynamics import Activation, Dynamics, time_loop
    w = configs.LVWorkload("lv_f3", 3, index=97)
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0)
    x0 = w.initial_x(m, sh.topology()["xyz0_full"])
    dyn = Dynamics(dt=5e-3, rho=1.0)
    act = Activation(0.1, ramp_type=1)
    wr = io.StepWriter(sh, m, tmp_path, act, dyn.dt, 3, dyn.rho, configs.H0, tiout=2, shell3d=True, fib=True)
    parts = {}
    x, rec = time_loop(sh, m, x0, dyn, act, 3, pre_update=lambda ti, x: (parts.__setitem__(ti, sh.residual_parts(x)),
                                                                         wr.pre_update(ti, x)),
                       on_step=wr.on_step, rtol=1e-10)
    assert wr.written == [1, 3]
    for ti in (0, 2):
        text = (tmp_path / f"surface00_{ti + 1:05d}.vtk").read_text().splitlines()
        k = text.index("VECTORS Fint float")
        Fint = np.array([[float(v) for v in ln.split()] for ln in text[k + 1: k + 1 + m.n_v]])
        np.testing.assert_allclose(Fint.ravel(), parts[ti][1][: 3 * m.n_v], rtol=0, atol=6e-7)
        k = text.index("VECTORS Fdyn float")
        Fdyn = np.array([[float(v) for v in ln.split()] for ln in text[k + 1: k + 1 + m.n_v]])
        np.testing.assert_allclose(Fdyn.ravel(), parts[ti][3][: 3 * m.n_v], rtol=0, atol=6e-7)
        assert "VECTORS nfib float" in text
        assert (tmp_path / f"shell3d00_{ti + 1:05d}.vtk").exists()
    sh.close()
