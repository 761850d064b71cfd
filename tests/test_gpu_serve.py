"""Serving loop (ServeCreate / ServeSubmit / ServeWait): load-step requests of
different mesh sizes run concurrently on their own streams, admitted by slot
and HBM budget.

Every kernel on the path is deterministic (gather assembly, fixed-order
reductions whose grids depend only on the problem size), so a request's
result in the mix must equal the same request solved alone bit for bit:
tolerance 0.
"""
import numpy as np
import pytest

from biofem import configs

pytestmark = pytest.mark.gpu

NEWTON = dict(max_newton=5, rtol=1e-10)


def alone(w, precision):
    from biofem.gpu import GpuShell
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, precision=precision)
    x0 = w.initial_x(m, sh.topology()["xyz0_full"])
    x, st = sh.newton(x0, **NEWTON)
    sh.close()
    return m, x0, x, st


def test_serve_results_equal_alone():
    from biofem.gpu import Serve
    ws = [configs.serve_request(i, 8, 48) for i in range(10)]
    precs = [i % 2 for i in range(10)]
    ref = [alone(w, p) for w, p in zip(ws, precs)]
    srv = Serve(2 << 30, 4)
    tickets = [srv.submit(m, w, configs.MU, configs.BULK, configs.H0, x0, precision=p, **NEWTON)
               for w, p, (m, x0, _, _) in zip(ws, precs, ref)]
    for t, w, (_, _, x_alone, st_alone) in zip(tickets, ws, ref):
        x, st, times = srv.wait(t)
        assert times[0] <= times[1] <= times[2]
        assert st["newton_its"] == st_alone["newton_its"] and st["gmres_its_total"] == st_alone["gmres_its_total"], w
        np.testing.assert_array_equal(x, x_alone, err_msg=w.name)
    s = srv.stats()
    assert s["completed"] == 10 and s["active"] == 0 and s["queued"] == 0 and s["in_use"] == 0
    assert 2 <= s["peak_active"] <= 4, s
    srv.close()


def test_serve_admission_respects_budget():
    from biofem.gpu import Serve, BiofemError, estimate_bytes
    ws = [configs.serve_request(i, 24, 40) for i in range(20, 26)]
    meshes = [w.build_mesh() for w in ws]
    est = [estimate_bytes(m.n_v, m.n_elmt, m.n_ghosts) for m in meshes]
    budget = int(max(est) * 1.5)                  # never two of the largest at once
    srv = Serve(budget, 6)
    from biofem.gpu import GpuShell
    tickets = []
    for w, m in zip(ws, meshes):
        sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, host_only=True)
        x0 = w.initial_x(m, sh.topology()["xyz0_full"])
        sh.close()
        tickets.append(srv.submit(m, w, configs.MU, configs.BULK, configs.H0, x0, **NEWTON))
    for t in tickets:
        _, st, _ = srv.wait(t)
        assert st["newton_its"] >= 1
    s = srv.stats()
    assert s["peak_in_use"] <= budget and s["completed"] == len(ws), s
    big = configs.serve_request(99, 64, 65)
    mb = big.build_mesh()
    with pytest.raises(BiofemError) as e:
        srv.submit(mb, big, configs.MU, configs.BULK, configs.H0, np.zeros(mb.n_dof))
    assert e.value.code == 55
    srv.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32_bulk"])
def test_serve_estimate_covers_what_a_request_allocates(precision):
    """The admission estimate BiofemServeEstimateBytes must not undercount:
    for requests across the stream's size range, the device memory a handle
    holds after its load step (mesh arrays, GMRES work, multigrid hierarchy;
    GetGpuMeshInfo.device_bytes) stays below the estimate."""
    import ctypes
    from biofem.gpu import GpuShell, MeshInfo, estimate_bytes
    for i, (lo, hi) in enumerate([(16, 17), (40, 41), (96, 97), (200, 201)]):
        w = configs.serve_request(300 + i, lo, hi)
        m = w.build_mesh()
        sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, precision=precision)
        x0 = w.initial_x(m, sh.topology()["xyz0_full"])
        sh.newton(x0, max_newton=2, rtol=1e-10)
        info = MeshInfo()
        assert sh.lib.GetGpuMeshInfo(sh.handle, ctypes.byref(info)) == 0
        est = estimate_bytes(m.n_v, m.n_elmt, m.n_ghosts, precision)
        print(f"{w.name} prec {precision}: device {info.device_bytes / 2**20:.1f} MiB, estimate {est / 2**20:.1f} MiB")
        assert info.device_bytes <= est, (w.name, info.device_bytes, est)
        sh.close()
