"""One quasi-static load step on the GPU (Newton + GMRES/block-Jacobi on the
assembled tangent) against the oracle's converged state.

tests/golden/C1_flat_32x24_newton.npz holds the oracle's converged C1 load
step (exact sparse Jacobian + direct solve, ||R|| <= 1e-10 ||R0||, made by
tests/golden/make_newton_golden.py).  The converged state depends only on R,
so the GPU solution must agree to the conditioning of the problem:
  ||x_gpu - x_oracle||_2 <= 1e-7 ||x_oracle - x0||_2.
"""
import numpy as np
import pytest

from conftest import GOLDEN
from biofem import configs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32_bulk"])
def test_newton_C1_matches_oracle(precision):
    from biofem.gpu import GpuShell
    d = np.load(GOLDEN / "C1_flat_32x24_newton.npz")
    w = configs.C1
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, precision=precision)
    x0 = w.initial_x(m, sh.topology()["xyz0_full"])
    np.testing.assert_array_equal(x0, d["x0"])
    x, st = sh.newton(x0, rtol=1e-10)
    assert st["converged"] == 1, st
    assert st["newton_its"] <= 8, st
    dx_ref = d["x"] - d["x0"]
    assert np.linalg.norm(x - d["x"]) <= 1e-7 * np.linalg.norm(dx_ref), (np.linalg.norm(x - d["x"]), st)
    R = sh.form_function(x)
    assert np.linalg.norm(R) <= 1e-10 * st["r0"] * 1.0001
    sh.close()


def test_newton_64x48_solution_is_a_root_of_the_oracle_residual(oracle_lib):
    from biofem.gpu import GpuShell
    w = configs.Workload("flat_64x48", 64, 48, z_sigma=1e-3, activation="smooth", index=80, pressure=2e-4)
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0)
    t = sh.topology()
    x0 = w.initial_x(m, t["xyz0_full"])
    x, st = sh.newton(x0, rtol=1e-10)
    assert st["converged"] == 1, st
    o = oracle_lib.setup_given_topology(m, w, t, configs.MU, configs.BULK, configs.H0)
    o.set_threads(8)
    R0 = o.residual(x0)
    R = o.residual(x)
    assert np.linalg.norm(R) <= 2e-10 * np.linalg.norm(R0), (np.linalg.norm(R), np.linalg.norm(R0), st)
    sh.close()


def test_multigrid_and_block_jacobi_reach_the_same_root():
    """The preconditioner changes the Krylov path, not the Newton root: both
    solves end within the stated tolerance of each other, and the multigrid
    solve takes several times fewer GMRES iterations.  Repeated multigrid
    solves are bitwise identical (deterministic setup and V-cycle)."""
    from biofem.gpu import GpuShell, BIOFEM_PC_AMG, BIOFEM_PC_BJACOBI
    w = configs.Workload("flat_48x36", 48, 36, z_sigma=1e-3, activation="smooth", index=81, pressure=3e-4)
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0)
    x0 = w.initial_x(m, sh.topology()["xyz0_full"])
    xa, sa = sh.newton(x0, rtol=1e-10, preconditioner=BIOFEM_PC_AMG)
    xa2, _ = sh.newton(x0, rtol=1e-10, preconditioner=BIOFEM_PC_AMG)
    xb, sb = sh.newton(x0, rtol=1e-10, preconditioner=BIOFEM_PC_BJACOBI)
    assert sa["converged"] == 1 and sb["converged"] == 1, (sa, sb)
    np.testing.assert_array_equal(xa, xa2)
    assert np.linalg.norm(xa - xb) <= 1e-7 * np.linalg.norm(xb - x0)
    assert 4 * sa["gmres_its_total"] <= sb["gmres_its_total"], (sa["gmres_its_total"], sb["gmres_its_total"])
    sh.close()


def test_eisenstat_walker_forcing_reaches_the_same_root():
    """Inexact Newton (Eisenstat-Walker forcing terms) stops every linear
    solve early; the Newton target ||R|| <= 1e-10 ||R0|| and the root stay the
    same, with fewer GMRES iterations in total."""
    from biofem.gpu import GpuShell
    w = configs.Workload("flat_48x36", 48, 36, z_sigma=1e-3, activation="smooth", index=82, pressure=3e-4)
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0)
    x0 = w.initial_x(m, sh.topology()["xyz0_full"])
    xf, sf = sh.newton(x0, rtol=1e-10, forcing=0)
    xe, se = sh.newton(x0, rtol=1e-10, forcing=1, max_newton=30)
    assert sf["converged"] == 1 and se["converged"] == 1, (sf, se)
    assert se["rfinal"] <= 1e-10 * se["r0"]
    assert np.linalg.norm(xe - xf) <= 1e-7 * np.linalg.norm(xf - x0)
    assert se["gmres_its_total"] < sf["gmres_its_total"], (se["gmres_its_total"], sf["gmres_its_total"])
    sh.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32_bulk"])
@pytest.mark.parametrize("pc", [0, 1], ids=["multigrid", "bjacobi"])
def test_device_gmres_step_matches_scipy_gmres(pc, precision):
    """The device Krylov solve against scipy's gmres, the stand-in for PETSc
    KSP: one Newton step without line search, linear tolerance 1e-11, solves
    the system scipy's gmres (block-Jacobi(3x3) preconditioned, same
    tolerance) solves on the same assembled tangent and residual.  With an
    FP32-bulk handle the tangent is its FP32 K and the device solve runs its
    matvec and projections in float-float arithmetic."""
    import scipy.sparse.linalg as spla
    from biofem.gpu import GpuShell
    w = configs.Workload("flat_40x30", 40, 30, z_sigma=1e-3, activation="smooth", index=83, pressure=3e-4)
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, precision=precision)
    x0 = w.initial_x(m, sh.topology()["xyz0_full"])
    R, K = sh.form_jacobian(x0)
    A = sh.to_scipy(K.astype(np.float64)).tocsr()
    nb = A.shape[0] // 3
    blocks = np.array([np.linalg.inv(A[3 * i:3 * i + 3, 3 * i:3 * i + 3].toarray()) for i in range(nb)])
    M = spla.LinearOperator(A.shape, matvec=lambda v: np.einsum("bij,bj->bi", blocks, v.reshape(-1, 3)).ravel())
    try:
        dx_ref, info = spla.gmres(A, -R, rtol=1e-11, atol=0.0, restart=30, maxiter=3000, M=M)
    except TypeError:   # scipy before 1.12 names the tolerance tol
        dx_ref, info = spla.gmres(A, -R, tol=1e-11, atol=0.0, restart=30, maxiter=3000, M=M)
    assert info == 0
    x1, st = sh.newton(x0, max_newton=1, rtol=1e-30, gmres_rtol=1e-11, line_search=0, preconditioner=pc)
    dx = x1 - x0
    assert st["gmres_relres_last"] <= 1.0001e-11, st
    # both solve the same system: true residuals in the assembled operator, and the two solutions
    rn = np.linalg.norm(R)
    assert np.linalg.norm(A @ dx + R) <= 1e-10 * rn, np.linalg.norm(A @ dx + R) / rn
    assert np.linalg.norm(A @ dx_ref + R) <= 1e-10 * rn
    assert np.linalg.norm(dx - dx_ref) <= 1e-6 * np.linalg.norm(dx_ref), np.linalg.norm(dx - dx_ref) / np.linalg.norm(dx_ref)
    sh.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32_bulk"])
def test_newton_capped_lv_is_a_root_of_the_oracle_residual(precision, oracle_lib):
    """A truncated spheroid closed at the apex by cap triangles around an
    apex node (n_elmt_base), base ring clamped (clamp_edge 1), activation on
    the strip: the device Newton root zeroes the oracle's residual on every
    free row (the oracle's rows are unclamped; the clamp only replaces the
    base rows by x - X)."""
    from biofem.gpu import GpuShell
    w = configs.capped(16, 8, True)
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, clamp_edge=1, precision=precision)
    t = sh.topology()
    x0 = w.initial_x(m, t["xyz0_full"])
    x, st = sh.newton(x0, rtol=1e-10, max_newton=30)
    assert st["converged"] == 1, st
    base = np.asarray(m.bnodes[m.n_bnodes[0]:])
    free = np.ones(3 * m.n_v, bool)
    free[(3 * base[:, None] + np.arange(3)).ravel()] = False
    X = np.asarray(t["xyz0_full"]).ravel()[: 3 * m.n_v]
    np.testing.assert_allclose(x[: 3 * m.n_v][~free], X[~free], rtol=0, atol=1e-14)   # the clamp: x = X
    o = oracle_lib.setup_given_topology(m, w, t, configs.MU, configs.BULK, configs.H0)
    R0 = o.residual(x0)[: 3 * m.n_v][free]
    R = o.residual(x)[: 3 * m.n_v][free]
    assert np.linalg.norm(R) <= 1e-9 * np.linalg.norm(R0), (np.linalg.norm(R), np.linalg.norm(R0), st)
    assert np.abs(x - x0)[: 3 * m.n_v].max() > 1e-2          # a large deformation, not a trivial root
    sh.close()
