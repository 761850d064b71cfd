"""RunGpuResidualNoAlloc: the residual for callers that cannot allocate
device memory at call time (a serving loop or host code working inside an
HBM budget it reserved up front, which must not have the library reach
cudaMalloc).  Its work arrays live in the library's fixed 8 MiB device
array instead of the mesh handle.

Checked through the C-ABI against the existing device entry point
RunGpuResidualDevice, with the residual tolerance of the other parity tests
(||R_a - R_b||_2 <= 1e-10 ||R_b||_2), on two calls in a row (the shared array
keeps the previous call's contents), and the size limit is enforced.
This file is collected last so that a stop-at-first-failure run has already
run every other test.
"""
import numpy as np
import pytest

from biofem import configs

pytestmark = pytest.mark.gpu


def _shell(w, precision=0):
    from biofem.gpu import GpuShell
    m = w.build_mesh()
    return m, GpuShell(m, w, configs.MU, configs.BULK, configs.H0, precision=precision)


def test_no_alloc_residual_matches_existing_entry_point_twice():
    torch = pytest.importorskip("torch")
    w = configs.C1
    m, sh = _shell(w)
    x = w.initial_x(m, sh.topology()["xyz0_full"])
    x[: 3 * m.n_v] += 1e-4 * np.random.default_rng(7).standard_normal(3 * m.n_v)
    dx = torch.tensor(x, device="cuda")
    ref = torch.empty_like(dx)
    sh.residual_device(dx.data_ptr(), ref.data_ptr(), 0)
    sh.sync(0)
    Rref = ref.cpu().numpy()
    for call in range(2):
        out = torch.full_like(dx, float("nan"))
        sh.residual_device_noalloc(dx.data_ptr(), out.data_ptr(), 0)
        sh.sync(0)
        R = out.cpu().numpy()
        assert np.isfinite(R).all(), call
        assert np.linalg.norm(R - Rref) <= 1e-10 * np.linalg.norm(Rref), call
    sh.close()


def test_no_alloc_residual_of_an_fp32_bulk_handle_is_its_residual():
    """An FP32-bulk handle's residual is the float-float kernel's; the
    no-allocation call runs the same kernel, so the two agree bit for bit."""
    torch = pytest.importorskip("torch")
    w = configs.C1
    m, sh = _shell(w, precision=1)
    x = w.initial_x(m, sh.topology()["xyz0_full"])
    dx = torch.tensor(x, device="cuda")
    ref = torch.empty_like(dx)
    sh.residual_device(dx.data_ptr(), ref.data_ptr(), 0)
    out = torch.full_like(dx, float("nan"))
    sh.residual_device_noalloc(dx.data_ptr(), out.data_ptr(), 0)
    sh.sync(0)
    assert torch.equal(out, ref)
    sh.close()


def test_no_alloc_residual_second_mesh_after_first():
    """A different (smaller) mesh after C1: stale contents of the shared
    array must not leak into the result."""
    torch = pytest.importorskip("torch")
    w = configs.small(9, 7, index=60, pressure=0.0)
    m, sh = _shell(w)
    x = w.initial_x(m, sh.topology()["xyz0_full"])
    dx = torch.tensor(x, device="cuda")
    ref = torch.empty_like(dx)
    sh.residual_device(dx.data_ptr(), ref.data_ptr(), 0)
    out = torch.empty_like(dx)
    for _ in range(2):
        sh.residual_device_noalloc(dx.data_ptr(), out.data_ptr(), 0)
    sh.sync(0)
    Rref = ref.cpu().numpy()
    assert np.linalg.norm(out.cpu().numpy() - Rref) <= 1e-10 * np.linalg.norm(Rref)
    sh.close()


def test_no_alloc_rejects_meshes_beyond_the_fixed_array():
    torch = pytest.importorskip("torch")
    from biofem.gpu import BiofemError
    w = configs.Workload("big", 128, 96, index=61)   # 24,576 triangles > limit
    m, sh = _shell(w)
    dx = torch.zeros(sh.n_dof, dtype=torch.float64, device="cuda")
    with pytest.raises(BiofemError) as ei:
        sh.residual_device_noalloc(dx.data_ptr(), dx.data_ptr(), 0)
    assert ei.value.code == 63 and "too large" in str(ei.value)
    sh.close()


def test_no_alloc_residual_reports_element_errors_through_sync():
    """A NaN coordinate makes CC3333 fail inside the element kernel; the
    no-allocation call reports it like the other device variants, through
    BiofemGpuSync (error 72), and the handle then gives the clean result."""
    torch = pytest.importorskip("torch")
    from biofem.gpu import BiofemError
    w = configs.small(8, 6, activation="random", index=62, pressure=1e-3)
    m, sh = _shell(w)
    x = w.initial_x(m, sh.topology()["xyz0_full"])
    dx = torch.tensor(x, device="cuda")
    ref = torch.empty_like(dx)
    sh.residual_device(dx.data_ptr(), ref.data_ptr(), 0)
    sh.sync(0)
    bad = x.copy()
    bad[3 * (m.n_v // 2) + 2] = np.nan
    dbad = torch.tensor(bad, device="cuda")
    out = torch.empty_like(dx)
    sh.residual_device_noalloc(dbad.data_ptr(), out.data_ptr(), 0)
    with pytest.raises(BiofemError) as ei:
        sh.sync(0)
    assert ei.value.code == 72
    sh.residual_device_noalloc(dx.data_ptr(), out.data_ptr(), 0)
    sh.sync(0)
    Rref = ref.cpu().numpy()
    assert np.linalg.norm(out.cpu().numpy() - Rref) <= 1e-10 * np.linalg.norm(Rref)
    sh.close()
