"""The CPU baseline bench.py reports beside the device numbers: the oracle's
element samples (residual alone, and residual + exact element tangent) run,
the residual sample's checksum does not depend on the thread count, and an
element range outside the mesh is refused."""
import ctypes

import numpy as np

import bench
from biofem import configs
from biofem.gpu import GpuShell


def _setup():
    w = configs.C1
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, host_only=True)
    topo = sh.topology()
    sh.close()
    return w, m, topo, w.initial_x(m, topo["xyz0_full"])


def test_residual_sample_is_deterministic_and_positive():
    w, m, topo, x = _setup()
    from oracle.pyoracle import Oracle
    o = Oracle().setup_given_topology(m, w, topo, configs.MU, configs.BULK, configs.H0)
    xc = np.ascontiguousarray(x)
    sums = []
    for threads in (1, 3):
        chk = ctypes.c_double()
        assert o.lib.oracle_r_sample(xc.ctypes.data_as(ctypes.c_void_p), 100, 612, threads, ctypes.byref(chk)) == 0
        sums.append(chk.value)
    assert sums[0] == sums[1] and np.isfinite(sums[0]) and sums[0] != 0.0
    chk = ctypes.c_double()
    assert o.lib.oracle_r_sample(xc.ctypes.data_as(ctypes.c_void_p), 5, m.n_elmt + 1, 1, ctypes.byref(chk)) == 63
    rate, secs, n = bench.cpu_rk(w, m, topo, x, 256, 2, residual_only=True)
    assert n == 256 and rate > 0 and secs > 0
    rate_k, secs_k, n_k = bench.cpu_rk(w, m, topo, x, 64, 2)
    assert n_k == 64 and rate_k > 0
