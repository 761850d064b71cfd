"""The PETSc adapter of biofem-ia_gb300/petsc/ -- gpu_snes.c (the SNES residual
and Jacobian callbacks over the C-ABI, the Jacobian an assembled SeqBAIJ(3)
matrix whose storage the library fills directly) and gpu_prepare.c (the
reference's FE -> mesh description) -- compiled against the petsc-lite shim
(oracle/petsc_lite), whose SeqBAIJ Mat keeps each 3x3 block column by column as
PETSc's SeqBAIJ storage does (a[k bs^2 + c bs + r]).

CPU: the adapter against a stand-in library (tests/fake_biofem_gpu.c) with
non-symmetric blocks: the SeqBAIJ product J v must equal the row-major K v, so
the block orientation is right; and GpuSnesPrepareFE fed the reference's own
FE (reference build) must pass on the mesh arrays and options unchanged.
GPU: the adapter and the library's FormFunctionFEMGpu / FormJacobianFEMGpu
against the oracle's residual and exact J v."""
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from biofem import configs

ROOT = Path(__file__).resolve().parents[1]
LITE = ROOT / "oracle" / "petsc_lite"
INC = ["-I", str(LITE), "-I", str(ROOT / "include"), "-I", str(ROOT / "biofem-ia_gb300" / "petsc")]
CFLAGS = ["-O2", "-std=gnu11", "-w"]


def _gcc():
    g = shutil.which("gcc")
    if g is None:
        pytest.skip("gcc not available")
    return g


def write_case(path, mesh, w, x=None, v=None, clamp_edge=0, precision=0, n_dof=None):
    with open(path, "wb") as f:
        f.write(np.array([mesh.n_v, mesh.n_elmt, mesh.n_edge, int(mesh.n_bnodes.sum()), w.n_qp, w.c33_iters,
                          clamp_edge, precision], np.int32).tobytes())
        f.write(np.array([configs.MU, configs.BULK, configs.H0, 1.0, w.pressure]).tobytes())
        f.write(np.ascontiguousarray(mesh.tri, np.int32).tobytes())
        f.write(np.ascontiguousarray(mesh.xyz0, np.float64).tobytes())
        f.write(np.ascontiguousarray(mesh.n_bnodes, np.int32).tobytes())
        f.write(np.ascontiguousarray(mesh.bnodes, np.int32).tobytes())
        f.write(np.ascontiguousarray(mesh.fib, np.float64).tobytes())
        f.write(np.ascontiguousarray(mesh.gamma_scale, np.float64).tobytes())
        if x is not None:
            f.write(np.array([n_dof], np.int32).tobytes())
            f.write(np.ascontiguousarray(x, np.float64).tobytes())
            f.write(np.ascontiguousarray(v, np.float64).tobytes())


def build_harness(tmp, libdir, libname):
    exe = tmp / "adapter_harness"
    subprocess.run([_gcc(), *CFLAGS, *INC, str(ROOT / "tests" / "petsc_adapter_harness.c"),
                    str(ROOT / "biofem-ia_gb300" / "petsc" / "gpu_snes.c"), str(LITE / "petsc_lite.c"),
                    "-L", str(libdir), f"-l{libname}", f"-Wl,-rpath,{libdir}", "-lm", "-o", str(exe)], check=True)
    return exe


def build_fake(tmp):
    so = tmp / "libfakebiofem.so"
    subprocess.run([_gcc(), *CFLAGS, "-shared", "-fPIC", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "fake_biofem_gpu.c"), "-o", str(so)], check=True)
    return so


def run_harness(exe, case, tmp, n_dof, env=None):
    out = tmp / "out.bin"
    r = subprocess.run([str(exe), str(case), str(out)], capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stderr
    return np.fromfile(out).reshape(4, n_dof)


def test_adapter_block_orientation_with_stand_in_library(tmp_path):
    w = configs.small(4, 3, index=80)
    m = w.build_mesh()
    nt = m.n_v + int(m.n_bnodes.sum())
    n_dof = 3 * nt
    build_fake(tmp_path)
    exe = build_harness(tmp_path, tmp_path, "fakebiofem")
    rng = np.random.default_rng(81)
    x, v = rng.standard_normal(n_dof), rng.standard_normal(n_dof)
    write_case(tmp_path / "case.bin", m, w, x, v, n_dof=n_dof)
    R, Jv, R2, Kv = run_harness(exe, tmp_path / "case.bin", tmp_path, n_dof)
    np.testing.assert_array_equal(R, 2 * x - 1)
    np.testing.assert_array_equal(R2, R)
    # the stand-in's K, row-major: block (i, j), entry (a, b) = 100 i + 10 j + 3 a + b + 0.5
    K = np.zeros((n_dof, n_dof))
    for i in range(nt):
        for j in (i - 1, i, i + 1):
            if 0 <= j < nt:
                K[3 * i:3 * i + 3, 3 * j:3 * j + 3] = 100 * i + 10 * j + np.arange(9).reshape(3, 3) + 0.5
    np.testing.assert_allclose(Kv, K @ v, rtol=1e-14, atol=0)
    np.testing.assert_array_equal(Jv, Kv)        # SeqBAIJ storage read column by column = K
    assert np.abs(Jv - (K.T @ v)).max() > 1.0    # and not its transpose


def test_adapter_prepare_passes_the_reference_fe_through(tmp_path):
    """GpuSnesPrepareFE reads the reference's own FE (IBMNodes + act_data,
    built by the reference's code in the reference build) and must hand the
    library exactly the mesh arrays and options of that FE."""
    from oracle import build_ref
    if not build_ref.available():
        pytest.skip("reference sources not present")
    ref_so = build_ref.build()
    build_fake(tmp_path)
    exe = tmp_path / "prepare_harness"
    subprocess.run([_gcc(), *CFLAGS, *INC, "-iquote", str(build_ref.REFERENCE / "include"),
                    str(ROOT / "tests" / "petsc_prepare_harness.c"),
                    str(ROOT / "biofem-ia_gb300" / "petsc" / "gpu_prepare.c"),
                    str(ROOT / "biofem-ia_gb300" / "petsc" / "gpu_snes.c"),
                    "-L", str(tmp_path), "-lfakebiofem", str(ref_so), f"-Wl,-rpath,{tmp_path}:{ref_so.parent}",
                    "-lm", "-o", str(exe)], check=True)
    w = configs.LVWorkload("lv_f2", 2, index=82)
    m = w.build_mesh()
    write_case(tmp_path / "case.bin", m, w, clamp_edge=0)
    dump = tmp_path / "dump.bin"
    r = subprocess.run([str(exe), str(tmp_path / "case.bin")], capture_output=True, text=True,
                       env=dict(os.environ, BIOFEM_FAKE_DUMP=str(dump)))
    assert r.returncode == 0, r.stderr
    b = dump.read_bytes()
    hdr = np.frombuffer(b, np.int32, 11)
    o = 44
    rv = np.frombuffer(b, np.float64, 5, o)
    o += 40
    ne, nv, ned, sb = m.n_elmt, m.n_v, m.n_edge, int(m.n_bnodes.sum())

    def take(dt, n):
        nonlocal o
        a = np.frombuffer(b, dt, n, o)
        o += a.nbytes
        return a
    np.testing.assert_array_equal(hdr, [nv, ne, ned, sb, w.n_qp, w.c33_iters, 0, 0, 0, 0, 1])   # COL_MAJOR
    np.testing.assert_array_equal(rv, [configs.MU, configs.BULK, configs.H0, 1.0, w.pressure])
    np.testing.assert_array_equal(take(np.int32, 3 * ne), m.tri.ravel())
    np.testing.assert_array_equal(take(np.float64, 3 * nv), m.xyz0.ravel())
    np.testing.assert_array_equal(take(np.int32, ned), m.n_bnodes)
    np.testing.assert_array_equal(take(np.int32, sb), m.bnodes)
    np.testing.assert_array_equal(take(np.float64, 3 * ne), np.asarray(m.fib).ravel())
    np.testing.assert_array_equal(take(np.float64, ne), m.gamma_scale)
    assert take(np.int32, 1)[0] == 0                                   # ibm->n_elmt_base


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32_bulk"])
def test_gpu_adapter_and_exports_against_the_oracle(tmp_path, oracle_lib, precision):
    """The SNES callbacks through PETSc-shaped Vec / SeqBAIJ Mat and the
    library's FormFunctionFEMGpu / FormJacobianFEMGpu, called from C, give the
    oracle's residual and exact J v."""
    from biofem.gpu import load_library, LIB_PATH
    load_library()
    w = configs.small(10, 8, activation="random", index=83, pressure=2e-3)
    m = w.build_mesh()
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0)
    t = o.topology()
    x = w.initial_x(m, t.xyz0_full)
    v = np.random.default_rng(84).standard_normal(x.size)
    Ro, Jo = o.jvp(x, v)
    exe = build_harness(tmp_path, LIB_PATH.parent, "biofem_gpu")
    write_case(tmp_path / "case.bin", m, w, x, v, precision=precision, n_dof=x.size)
    R, Jv, R2, Kv = run_harness(exe, tmp_path / "case.bin", tmp_path, x.size)
    np.testing.assert_array_equal(R2, R)
    assert np.linalg.norm(R - Ro) <= 1e-10 * np.linalg.norm(Ro)
    real = slice(0, 3 * m.n_v)
    tol = 1e-9 if precision == 0 else 1e-5
    assert np.linalg.norm((Jv - Jo)[real]) <= tol * np.linalg.norm(Jo[real])
    np.testing.assert_allclose(Jv, Kv, rtol=0, atol=1e-14 * np.abs(Kv).max())
