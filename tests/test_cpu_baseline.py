"""The CPU baseline bench.py reports beside the device numbers: the oracle's
element samples (residual alone, and residual + exact element tangent) run,
the residual sample's checksum does not depend on the thread count, an
element range outside the mesh is refused, and the reference arm sets the
oracle up by its own table builders without the GPU library."""
import ctypes
import subprocess
import sys
from pathlib import Path

import numpy as np

import bench
from biofem import configs
from biofem.gpu import GpuShell

ROOT = Path(__file__).resolve().parents[1]


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
    rate, secs, n = bench.cpu_rk(o, m.n_elmt, x, 256, 2, residual_only=True)
    assert n == 256 and rate > 0 and secs > 0
    rate_k, secs_k, n_k = bench.cpu_rk(o, m.n_elmt, x, 64, 2, steps=2)
    assert n_k == 64 and rate_k > 0


_PROBE = r"""
import sys, numpy as np
sys.path[:0] = [{root!r}, {pkg!r}]
import bench
from biofem import configs
w = configs.C1
m = w.build_mesh()
o = bench.cpu_oracle(w, m)
t = o.topology()
np.savez({out!r}, patch=t.patch, ire=t.ire, val=t.val, irv=t.irv, gtri=t.gtri)
maps = open('/proc/self/maps').read()
print('GPU_LIB_LOADED' if 'libbiofem_gpu' in maps else 'CLEAN')
"""


def test_reference_arm_oracle_needs_no_gpu_library(tmp_path):
    """bench.py --impl reference times the oracle set up by its own builders:
    the process never maps libbiofem_gpu.so, and the tables it builds are the
    host builder's."""
    out = tmp_path / "topo.npz"
    code = _PROBE.format(root=str(ROOT), pkg=str(ROOT / "biofem-ia_gb300"), out=str(out))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip().splitlines()[-1] == "CLEAN"
    _, m, topo, _ = _setup()
    got = np.load(out)
    for k in ("patch", "ire", "val", "irv"):
        np.testing.assert_array_equal(got[k], np.asarray(topo[k]).reshape(got[k].shape), err_msg=k)
    np.testing.assert_array_equal(got["gtri"][:m.n_elmt], np.asarray(topo["gtri"])[:m.n_elmt])
