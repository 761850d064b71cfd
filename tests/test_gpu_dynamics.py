"""GPU parity of the dynamic term (FDynamic / xAccVel, main.c:1157-1412) and
of the time loop, through the C-ABI, against the oracle.

Tolerances (FP64):
  residual   per entry |R_gpu - R_ref| <= 1e-12 max|R_ref| (the static part's
             bound; the inertial sum is the same triangle-order sum);
  tangent    ||K v - J v|| <= 1e-9 ||J v|| on the non-ghost rows, J v the
             oracle's exact directional derivative;
  state      xAccVel is elementwise: 1e-12 relative;
  time loop  three Newton-converged steps (rtol 1e-10): displacements within
             1e-7 of the displacement norm.
"""
import numpy as np
import pytest

from biofem import configs

pytestmark = pytest.mark.gpu

CASES = [configs.small(9, 7, activation="random", index=80, pressure=1e-3),
         configs.LVWorkload("lv_f4", 4, index=81)]
MODES = [(0, 0, 0.5), (0, 1, 0.6), (1, 1, 0.5)]


def setup_pair(w, oracle_lib, precision=0):
    from biofem.gpu import GpuShell
    m = w.build_mesh()
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0)
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, precision=precision)
    x = w.initial_x(m, sh.topology()["xyz0_full"])
    return m, o, sh, x


def random_state(x, seed):
    rng = np.random.default_rng(seed)
    return dict(xn=x + 1e-3 * rng.standard_normal(x.size), xnm1=x + 1e-3 * rng.standard_normal(x.size),
                xd=rng.standard_normal(x.size), xdd=rng.standard_normal(x.size))


@pytest.mark.parametrize("mode", MODES, ids=["newmark", "newmark_damped", "central_damped"])
@pytest.mark.parametrize("w", CASES, ids=lambda w: w.name)
def test_dynamic_residual_and_tangent_match_oracle(w, mode, oracle_lib):
    timeinteg, damping, G = mode
    m, o, sh, x = setup_pair(w, oracle_lib)
    dyn = (2e-3, 1.3, G, 7.0, timeinteg, damping)
    st = random_state(x, 82)
    for side in (o, sh):
        side.set_dynamics(*dyn)
        side.set_dynamic_state(**st)
    Ro = o.residual(x)
    R = sh.form_function(x)
    assert np.abs(R - Ro).max() <= 1e-12 * np.abs(Ro).max()
    R2, K = sh.form_jacobian(x)
    np.testing.assert_array_equal(R, R2)
    Ks = sh.to_scipy(K)
    ghost = np.zeros(sh.n_dof, bool)
    ghost[3 * m.n_v:] = True
    rng = np.random.default_rng(83)
    for _ in range(2):
        v = rng.standard_normal(sh.n_dof)
        _, Jv = o.jvp(x, v)
        Kv = Ks @ v
        assert np.linalg.norm(Kv[~ghost] - Jv[~ghost]) <= 1e-9 * np.linalg.norm(Jv[~ghost])
        np.testing.assert_array_equal(Kv[ghost], v[ghost])
    # xAccVel + shift on the device against the oracle
    sh.dynamic_update(x)
    o.dynamic_update(x)
    sg, so = sh.dynamic_state(), o.dynamic_state()
    for k in ("xn", "xnm1", "xd", "xdd"):
        np.testing.assert_allclose(sg[k], so[k], rtol=1e-12, atol=1e-12 * np.abs(so[k]).max())
    # switching the term off gives back the static residual
    sh.set_dynamics(None)
    o.set_dynamics(None)
    np.testing.assert_allclose(sh.form_function(x), o.residual(x), rtol=0, atol=1e-12 * np.abs(Ro).max())
    sh.close()


def test_dynamic_state_starts_at_the_reference(oracle_lib):
    w = CASES[1]
    m, o, sh, x = setup_pair(w, oracle_lib)
    sh.set_dynamics(1e-2, 1.0)
    s = sh.dynamic_state()
    X = sh.topology()["xyz0_full"].ravel()
    np.testing.assert_array_equal(s["xn"], X)
    np.testing.assert_array_equal(s["xnm1"], X)
    assert not s["xd"].any() and not s["xdd"].any()
    sh.close()


def test_element_gamma_matches_oracle(oracle_lib):
    w = CASES[0]
    m, o, sh, x = setup_pair(w, oracle_lib)
    g = 0.4 * np.asarray(m.gamma_scale) * (1 + 0.5 * np.sin(np.arange(m.n_elmt)))
    sh.set_element_gamma(g)
    o.set_element_gamma(g)
    Ro = o.residual(x)
    assert np.abs(sh.form_function(x) - Ro).max() <= 1e-12 * np.abs(Ro).max()
    sh.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32_bulk"])
def test_time_loop_matches_oracle(precision, oracle_lib):
    """Three Newmark steps with damping and a delayed half-sin^2 activation
    ramp: GPU time loop (device Newton) against the oracle's Newton + xAccVel."""
    from biofem.dynamics import Activation, Dynamics, time_loop
    w = configs.small(8, 6, activation="random", index=84, pressure=1e-3, disp_rel=0.0)
    m, o, sh, x0 = setup_pair(w, oracle_lib, precision)
    dyn = Dynamics(dt=5e-3, rho=1.0, newmark_gamma=0.5, dampfactor=2.0, damping=1)
    act = Activation(0.15, ramp_type=2, T=0.015)
    delay = 0.004 * (np.arange(m.n_elmt) % 3)
    n = 3
    xs = []
    xg, rec = time_loop(sh, m, x0, dyn, act, n, delay=delay, on_step=lambda ti, x, r: xs.append(x.copy()),
                        rtol=1e-10, max_newton=40)
    assert all(r.converged for r in rec), [r.stats for r in rec]
    topo = o.topology()
    o.set_dynamics(dyn.dt, dyn.rho, dyn.newmark_gamma, dyn.dampfactor, dyn.timeinteg, dyn.damping)
    x = x0.copy()
    for ti in range(n):
        o.set_element_gamma(act.element_gamma(ti, dyn.dt, n, m.gamma_scale, delay))
        x, hist = o.newton(x, topo, rtol=1e-10, max_it=40, jacobian_its=1)
        o.dynamic_update(x)
        u_ref = (x - x0)[: 3 * m.n_v]
        u_gpu = (xs[ti] - x0)[: 3 * m.n_v]
        assert np.linalg.norm(u_ref) > 0
        assert np.linalg.norm(u_gpu - u_ref) <= 1e-7 * np.linalg.norm(u_ref), (ti, np.linalg.norm(u_gpu - u_ref))
    sg, so = sh.dynamic_state(), o.dynamic_state()
    nr = 3 * m.n_v
    for k in ("xd", "xdd"):
        assert np.linalg.norm(sg[k][:nr] - so[k][:nr]) <= 1e-5 * np.linalg.norm(so[k][:nr]), k
    sh.close()


def test_dynamic_term_full_size_C2():
    """C2 (98,304 triangles): Fdyn is the lumped-mass Newmark form of an
    independent numpy statement (the real triangles, FDynamic's path in an
    active-strain run), and the tangent grows by exactly its diagonal on the
    free rows."""
    from biofem.gpu import GpuShell
    w = configs.C2
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0)
    topo = sh.topology()
    x = w.initial_x(m, topo["xyz0_full"])
    rng = np.random.default_rng(85)
    st = dict(xn=x + 1e-4 * rng.standard_normal(x.size), xd=rng.standard_normal(x.size),
              xdd=rng.standard_normal(x.size))
    _, K0 = sh.form_jacobian(x)
    dt, rho, G, c = 1e-3, 1.1, 0.55, 4.0
    sh.set_dynamics(dt, rho, G, c, 0, 1)
    sh.set_dynamic_state(**st)
    R, Fi, Fe, Fd = sh.residual_parts(x)
    X = topo["xyz0_full"]
    tri = topo["gtri"][: m.n_elmt]
    A = 0.5 * np.linalg.norm(np.cross(X[tri[:, 1]] - X[tri[:, 0]], X[tri[:, 2]] - X[tri[:, 0]]), axis=1)
    mass = np.zeros(X.shape[0])
    for k in range(3):
        np.add.at(mass, tri[:, k], rho * configs.H0 * A / 3)
    M = np.repeat(mass, 3)
    B = 0.25 * (G + 0.5) ** 2
    M1, M2, M3 = 1 / (B * dt * dt), 1 / (B * dt), 1 / (2 * B) - 1
    C1, C2, C3 = G / (B * dt), G / B - 1, dt * (G / (2 * B) - 1)
    fd = M * (M1 * (x - st["xn"]) - M2 * st["xd"] - M3 * st["xdd"]) \
        + c * M * (C1 * (x - st["xn"]) - C2 * st["xd"] - C3 * st["xdd"])
    nr = 3 * m.n_v
    np.testing.assert_allclose(Fd[:nr], fd[:nr], rtol=1e-9, atol=1e-12 * np.abs(fd[:nr]).max())
    _, K1 = sh.form_jacobian(x)
    v = rng.standard_normal(sh.n_dof)
    d = sh.to_scipy(K1) @ v - sh.to_scipy(K0) @ v
    kinds = np.zeros(sh.n_dof, bool)
    kinds[:nr] = True
    clamped = np.zeros(sh.n_dof, bool)
    for nb in m.bnodes[: m.n_bnodes[0]]:
        clamped[3 * nb: 3 * nb + 3] = True
    free = kinds & ~clamped
    expect = M * (M1 + c * C1) * v   # R is unscaled here: no pressure on C2 beyond 1e-4 (max|Fext| < 1)
    np.testing.assert_allclose(d[free], expect[free], rtol=1e-9, atol=1e-9 * np.abs(expect[free]).max())
    assert not d[~free].any()
    sh.close()
