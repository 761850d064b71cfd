"""The reference's own GPU kernels (src/cuda_kernel.cu, compiled unmodified
into oracle/_ref/ref_cuda_kernel.cubin and launched as its Launch*Impl
functions launch them): their element geometry agrees with the oracle's on a
flat membrane and on an ellipsoid with irregular (valence 5/7) patches, so
the timing bench.py --impl reference reports is of the reference kernels
doing their real work."""
import numpy as np
import pytest

from biofem import configs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def kernels():
    from oracle import ref_cuda
    if not ref_cuda.available():
        pytest.skip("oracle/_ref/ref_cuda_kernel.cubin not built (reference sources absent at build time)")
    return ref_cuda.RefCudaKernels()


@pytest.mark.parametrize("which", ["flat", "lv"])
def test_reference_geometry_kernel_matches_the_oracle(kernels, oracle_lib, which):
    import torch
    w = configs.small(12, 9, index=90) if which == "flat" else configs.LVWorkload("lv_f2", 2, index=91)
    m = w.build_mesh()
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0)
    t = o.topology()
    x = w.initial_x(m, t.xyz0_full)
    theta = np.polynomial.legendre.leggauss(w.n_qp)[0]
    b = kernels.prepare(m, t, x, t.xyz0_full.ravel(), w.n_qp, configs.H0, theta)
    sp = torch.cuda.current_stream().cuda_stream
    kernels.subdiv_geom(b, "ref", sp)
    kernels.subdiv_geom(b, "cur", sp)
    kernels.metric_tensor(b, sp)
    torch.cuda.synchronize()
    assert int((b["status"] != 0).sum()) == 0
    assert int((b["mstatus"] != 0).sum()) == 0
    geom = b["geom_cur"].cpu().numpy().reshape(m.n_elmt, 24)
    ref = np.array([o.elem_state(x, e, w.n_qp)[2].ravel() for e in range(m.n_elmt)])
    scale = np.abs(ref).max(axis=1, keepdims=True)
    assert np.abs(geom - ref).max() <= 1e-12 * scale.max()
    if which == "lv":
        assert int((t.ire != 0).sum()) > 0     # irregular patches were exercised
    # MetricTensorKernel_ keeps a3 = n as the third covariant basis vector
    basis = b["basis_cur"].cpu().numpy().reshape(m.n_elmt, w.n_qp, 18)
    np.testing.assert_array_equal(basis[:, :, 6:9], np.repeat(geom[:, None, 6:9], w.n_qp, axis=1))
