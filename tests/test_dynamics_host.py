"""The dynamic term and time stepping on the CPU: the oracle's FDynamic and
xAccVel (main.c:1157-1412) against a direct numpy statement of the lumped-mass Newmark / central-difference forms,
Newmark's exactness on a constant acceleration, the activation ramps of
GammaOfTimeDelayed (active_strain.c:1156-1179), and the host logic of the time
loop.

Known answers:
  * the lumped corner mass of a node is sum over the real triangles with that
    corner of rho h0 A0 / 3 (FDynamic with the DMPlex context of an
    active-strain run, main.c:1178-1270);
  * Newmark with gamma = 1/2 (Beta = 1/4) reproduces x(t) = x0 + v0 t + a t^2/2
    exactly: one xAccVel from (x0, v0, a) with x(dt) gives back a and v0 + a dt;
  * ramp 1 peaks at T/2, ramp 2 at T, ramp 3 is 1/2 at its upstroke midpoint
    (times the decay factor), ramps 1 and 2 are 0 for t <= 0.
"""
import numpy as np
import pytest

from biofem import configs
from biofem.dynamics import Activation, Dynamics, StepRecord, time_loop


def newmark_consts(dt, G):
    B = 0.25 * (G + 0.5) ** 2
    return dict(M1=1 / (B * dt * dt), M2=1 / (B * dt), M3=1 / (2 * B) - 1, C1=G / (B * dt), C2=G / B - 1,
                C3=dt * (G / (2 * B) - 1), U2=(1 - G) * dt, U3=G * dt)


def lumped_mass(topo, n_dof, rho, h0, n_elmt):
    X = topo.xyz0_full
    tri = topo.gtri[:n_elmt]
    a = X[tri[:, 1]] - X[tri[:, 0]]
    b = X[tri[:, 2]] - X[tri[:, 0]]
    A = 0.5 * np.linalg.norm(np.cross(a, b), axis=1)
    m = np.zeros(n_dof // 3)
    for k in range(3):
        np.add.at(m, tri[:, k], rho * h0 * A / 3)
    return np.repeat(m, 3)


def free_rows(mesh, o, clamp=True):
    free = np.zeros(o.n_dof, bool)
    free[: 3 * mesh.n_v] = True
    if clamp:
        for nb in mesh.bnodes[: mesh.n_bnodes[0]]:
            free[3 * nb: 3 * nb + 3] = False
    return free


@pytest.fixture(scope="module")
def body(oracle_lib):
    w = configs.small(8, 6, index=70, pressure=0.0)
    m = w.build_mesh()
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0)
    topo = o.topology()
    x = w.initial_x(m, topo.xyz0_full)
    rng = np.random.default_rng(71)
    state = dict(xn=x + 1e-3 * rng.standard_normal(x.size), xnm1=x + 1e-3 * rng.standard_normal(x.size),
                 xd=rng.standard_normal(x.size), xdd=rng.standard_normal(x.size))
    yield w, m, o, topo, x, state
    o.set_dynamics(None)


@pytest.mark.parametrize("timeinteg,damping,G", [(0, 0, 0.5), (0, 1, 0.6), (1, 1, 0.5)],
                         ids=["newmark", "newmark_damped", "central_damped"])
def test_oracle_dynamic_term_is_the_lumped_mass_form(body, timeinteg, damping, G):
    w, m, o, topo, x, st = body
    rho, dt, c = 1.3, 2e-3, 7.0
    o.set_dynamics(None)
    R0 = o.residual(x)
    o.set_dynamics(dt, rho, G, c, timeinteg, damping)
    o.set_dynamic_state(**st)
    R1 = o.residual(x)
    M = lumped_mass(topo, o.n_dof, rho, configs.H0, m.n_elmt)
    C = c * M if damping else 0.0 * M
    k = newmark_consts(dt, G)
    if timeinteg == 0:
        fd = M * (k["M1"] * (x - st["xn"]) - k["M2"] * st["xd"] - k["M3"] * st["xdd"]) \
            + C * (k["C1"] * (x - st["xn"]) - k["C2"] * st["xd"] - k["C3"] * st["xdd"])
    else:
        fd = M * (x - 2 * st["xn"] + st["xnm1"]) / dt ** 2 + C * (x - st["xn"]) / dt
    free = free_rows(m, o)
    d = R1 - R0
    np.testing.assert_allclose(d[free], fd[free], rtol=1e-9, atol=1e-12 * np.abs(fd).max())
    assert not d[~free].any()   # clamped rows stay x - X, ghost rows 0
    # the exact Jacobian gains diag(M (M1 + c C1)) (or M / dt^2 + C / dt) on free rows
    v = np.random.default_rng(3).standard_normal(o.n_dof)
    o.set_dynamics(None)
    _, J0v = o.jvp(x, v)
    o.set_dynamics(dt, rho, G, c, timeinteg, damping)
    o.set_dynamic_state(**st)
    _, J1v = o.jvp(x, v)
    diag = (M * k["M1"] + C * k["C1"]) if timeinteg == 0 else (M / dt ** 2 + C / dt)
    np.testing.assert_allclose((J1v - J0v)[free], (diag * v)[free], rtol=1e-9, atol=1e-9 * np.abs(diag * v).max())


def test_oracle_state_starts_at_the_reference_and_xaccvel(body):
    w, m, o, topo, x, st = body
    dt, G = 1e-2, 0.55
    o.set_dynamics(dt, 1.0, G, 0.0, 0, 0)
    s0 = o.dynamic_state()
    X = topo.xyz0_full.ravel()
    np.testing.assert_array_equal(s0["xn"], X)
    np.testing.assert_array_equal(s0["xnm1"], X)
    assert not s0["xd"].any() and not s0["xdd"].any()
    o.set_dynamic_state(**st)
    o.dynamic_update(x)
    s1 = o.dynamic_state()
    k = newmark_consts(dt, G)
    a = k["M1"] * (x - st["xn"]) - k["M2"] * st["xd"] - k["M3"] * st["xdd"]
    v = st["xd"] + k["U2"] * st["xdd"] + k["U3"] * a
    real = slice(0, 3 * m.n_v)   # xAccVel with the DMPlex context: the real nodes
    np.testing.assert_allclose(s1["xdd"][real], a[real], rtol=1e-12, atol=1e-12 * np.abs(a).max())
    np.testing.assert_allclose(s1["xd"][real], v[real], rtol=1e-12, atol=1e-12 * np.abs(v).max())
    np.testing.assert_array_equal(s1["xdd"][3 * m.n_v:], st["xdd"][3 * m.n_v:])
    np.testing.assert_array_equal(s1["xd"][3 * m.n_v:], st["xd"][3 * m.n_v:])
    np.testing.assert_array_equal(s1["xn"], x)
    np.testing.assert_array_equal(s1["xnm1"], st["xn"])


def test_newmark_is_exact_for_constant_acceleration(body):
    w, m, o, topo, x, st = body
    dt = 1e-2
    o.set_dynamics(dt, 1.0, 0.5, 0.0, 0, 0)
    rng = np.random.default_rng(9)
    X = topo.xyz0_full.ravel()
    v0, a = rng.standard_normal(X.size), rng.standard_normal(X.size)
    o.set_dynamic_state(xn=X, xd=v0, xdd=a)
    real = slice(0, 3 * m.n_v)
    for step in range(1, 4):
        o.dynamic_update(X + v0 * (step * dt) + 0.5 * a * (step * dt) ** 2)
        s = o.dynamic_state()
        np.testing.assert_allclose(s["xdd"][real], a[real], rtol=0, atol=1e-8 * np.abs(a).max())
        np.testing.assert_allclose(s["xd"][real], (v0 + a * step * dt)[real], rtol=0, atol=1e-9 * np.abs(v0).max())


def test_per_element_gamma_equals_scalar_gamma_times_scale(oracle_lib):
    """gamma_e = gamma * gamma_scale_e passed per element gives the residual of
    the scalar-gamma body (ElemActDefGrad's product)."""
    w = configs.LVWorkload("lv_f3", 3, index=72)
    m = w.build_mesh()
    gam = 0.7
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0, gamma=gam)
    x = w.initial_x(m, o.topology().xyz0_full)
    R0 = o.residual(x)
    o.set_element_gamma(gam * np.asarray(m.gamma_scale))
    R1 = o.residual(x)
    np.testing.assert_array_equal(R0, R1)
    o.set_element_gamma(np.zeros(m.n_elmt))
    R2 = o.residual(x)
    assert np.linalg.norm(R2 - R0) > 1e-6 * np.linalg.norm(R0)


def test_activation_ramps():
    dt, n = 1e-3, 200
    T = n * dt
    assert Activation(0.3).at(17, dt, n) == 0.3
    r1 = Activation(0.3, 1)
    assert r1.at(0, dt, n) == 0.0 and r1.at(-3, dt, n) == 0.0
    assert abs(r1.at(n // 2, dt, n) - 0.3) < 1e-15
    assert abs(r1.at(n, dt, n)) < 1e-15
    r2 = Activation(0.3, 2, T=0.1)
    assert abs(r2.at(100, dt, n) - 0.3) < 1e-15
    g = [r2.at(i, dt, n) for i in range(101)]
    assert all(b >= a for a, b in zip(g, g[1:]))   # monotonic systole ramp
    r3 = Activation(0.3, 3, tau_up=0.01, tau_down=0.05, apd=0.2)
    t_up = 0.04
    phi_down = 1 / (1 + np.exp((t_up - (t_up + 0.2)) / 0.05))
    assert abs(r3.at(40, dt, n) - 0.3 * 0.5 * phi_down) < 1e-15
    g3 = [r3.at(i, dt, 1000) for i in range(1000)]
    k = int(np.argmax(g3))
    assert 40 < k < 240 and g3[-1] < 0.01 * max(g3)
    # delay shifts the clock per element
    d = np.array([0.0, 0.05, 0.2])
    ge = r1.at(100, dt, n, d)
    np.testing.assert_allclose(ge, [r1.at(100, dt, n), r1.at(50, dt, n), 0.0], rtol=0, atol=1e-15)
    np.testing.assert_array_equal(Activation(0.3, 1).element_gamma(100, dt, n, [1.0, 0.5, 2.0], d), ge * [1.0, 0.5, 2.0])
    with pytest.raises(ValueError):
        Activation(0.3, 4)


class FakeShell:
    """Records the calls the time loop makes; Newton fails on one step."""

    def __init__(self, fail_at):
        self.calls, self.fail_at, self.k = [], fail_at, 0

    def set_dynamics(self, *a):
        self.calls.append(("dyn", a))

    def set_element_gamma(self, g):
        self.calls.append(("gamma", float(np.mean(g))))

    def newton(self, x, **kw):
        from biofem.gpu import BiofemError
        self.k += 1
        self.calls.append(("newton", kw))
        if self.k == self.fail_at:
            e = BiofemError(44, "line search failed")
            e.stats = {"newton_its": 3}
            raise e
        return x + 1.0, {"newton_its": 2}

    def dynamic_update(self, x):
        self.calls.append(("update", float(x[0])))


def test_time_loop_host_logic():
    class M:
        gamma_scale = np.array([1.0, 1.0])
    sh = FakeShell(fail_at=2)
    seen = []
    x, rec = time_loop(sh, M, np.zeros(3), Dynamics(1e-3, 1.0), Activation(0.2, 2), 4,
                       on_step=lambda ti, x, r: seen.append((ti, x[0])), rtol=1e-9)
    kinds = [c[0] for c in sh.calls]
    assert kinds == ["dyn"] + ["gamma", "newton", "update"] * 4
    assert [r.converged for r in rec] == [True, False, True, True]
    # the failed step keeps the previous positions and still advances the state
    assert [s[1] for s in seen] == [1.0, 1.0, 2.0, 3.0]
    assert [c[1] for c in sh.calls if c[0] == "update"] == [1.0, 1.0, 2.0, 3.0]
    assert rec[0].gamma_mean == 0.0 and rec[3].gamma_mean > rec[2].gamma_mean > 0
    assert all(isinstance(r, StepRecord) for r in rec) and "error" in rec[1].stats
    assert sh.calls[2][1] == {"rtol": 1e-9}
