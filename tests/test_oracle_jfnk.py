"""The reference's own solver path restated on the oracle (Jacobian-free
Newton: matrix-free finite-difference J v, unpreconditioned GMRES(30),
backtracking) reaches the same root as the oracle's Newton with the exact
Jacobian: the converged state depends only on R."""
import numpy as np

from biofem import configs
from biofem.gpu import GpuShell


def test_jfnk_reaches_the_exact_newton_root(oracle_lib):
    w = configs.small(4, 3, activation="random", index=95, pressure=1e-3)
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, host_only=True)
    topo = sh.topology()
    sh.close()
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0)
    x0 = w.initial_x(m, topo["xyz0_full"])
    x_ref, hist = o.newton(x0, o.topology(), rtol=1e-10)
    assert hist[-1] <= 1e-10 * hist[0]
    x = x0.copy()
    r0 = np.linalg.norm(o.residual(x0))
    evals = 0
    for _ in range(20):
        x, R, st = o.jfnk_newton_step(x)
        evals += st["residual_evaluations"]
        assert st["gmres_its"] > 0 and st["residual_evaluations"] >= st["gmres_its"] + 2
        if np.linalg.norm(R) <= 1e-8 * r0:
            break
    assert np.linalg.norm(R) <= 1e-8 * r0
    nreal = 3 * m.n_v
    dx = x_ref[:nreal] - x0[:nreal]
    assert np.linalg.norm(x[:nreal] - x_ref[:nreal]) <= 1e-6 * np.linalg.norm(dx)
    assert evals > 20
