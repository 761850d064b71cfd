"""Host-side input checks of PrepareGpuMesh / BuildHostMesh: every bad
parameter or mesh is refused with a PETSc-style code before any device work
(62 PETSC_ERR_ARG_WRONG, 63 PETSC_ERR_ARG_OUTOFRANGE), as the reference's
PetscCheck calls do; no CUDA call is made (host-only handles)."""
import copy
import dataclasses

import pytest

from biofem import configs
from biofem.gpu import BiofemError, GpuShell

W = configs.small(6, 5, index=98)


def build(mesh, w, **kw):
    h0 = kw.pop("h0", configs.H0)
    sh = GpuShell(mesh, w, configs.MU, configs.BULK, h0, host_only=True, **kw)
    sh.close()


@pytest.fixture(scope="module")
def mesh():
    return W.build_mesh()


@pytest.mark.parametrize("change,kw,code", [
    (dict(n_qp=7), {}, 63), (dict(n_qp=0), {}, 63), (dict(c33_iters=0), {}, 62),
    ({}, dict(h0=0.0), 62), ({}, dict(h0=float("nan")), 62), ({}, dict(precision=5), 62),
    ({}, dict(clamp_edge=9), 63), (dict(basis=4), {}, 62), (dict(tnormal=2), {}, 62)],
    ids=["n_qp7", "n_qp0", "c33_0", "h0_0", "h0_nan", "precision", "clamp_ring", "basis", "tnormal"])
def test_bad_parameters(mesh, change, kw, code):
    with pytest.raises(BiofemError) as e:
        build(mesh, dataclasses.replace(W, **change), **kw)
    assert e.value.code == code


def test_bad_meshes(mesh):
    cases = []
    m = copy.deepcopy(mesh); m.tri = m.tri.copy(); m.tri[3, 1] = mesh.n_v + 5; cases.append((m, 63))
    m = copy.deepcopy(mesh); m.tri = m.tri.copy(); m.tri[3, 1] = -1; cases.append((m, 63))
    m = copy.deepcopy(mesh); m.bnodes = m.bnodes.copy(); m.bnodes[0] = mesh.n_v + 1; cases.append((m, 63))
    m = copy.deepcopy(mesh); m.tri = m.tri[:0]; m.fib = m.fib[:0]; m.gamma_scale = m.gamma_scale[:0]; cases.append((m, 62))
    for m, code in cases:
        with pytest.raises(BiofemError) as e:
            build(m, W)
        assert e.value.code == code
    build(mesh, W)   # the untouched mesh still builds
