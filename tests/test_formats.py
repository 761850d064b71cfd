"""On-disk formats against the reference's own writers (fixtures made by
tests/golden/make_formats_golden.py from io.c's LocationOut, LocationIn,
Output and Write3DShellVTK in the reference build).

Bar: byte-identical files (SHA-256 of the reference's file) for the same
state; LocationIn reads both checkpoint layouts back bit-exactly; the
restated thickness (h0 sqrt(mean C33)) equals UpdateElementThickness's.
"""
import hashlib
import json

import numpy as np
import pytest

from conftest import GOLDEN
from biofem.gpu import BIOFEM_CKPT_VEC, BIOFEM_CKPT_VERTEX_ORDER, BiofemError
from biofem import configs, io

CASES = sorted(GOLDEN.glob("formats_*.npz"))


def load(path):
    d = np.load(path)
    meta = json.loads(str(d["meta"]))
    w = None
    # the generator's workloads, rebuilt here (the generator imports the reference build)
    if meta["case"] == "formats_flat_6x5":
        w = configs.small(6, 5, activation="random", index=90, pressure=1e-3)
    elif meta["case"] == "formats_lv_f2":
        w = configs.LVWorkload("lv_f2", 2, index=91)
    assert w is not None and w.name == meta["workload"], meta
    return w, meta, d


def sha(p):
    return hashlib.sha256(p.read_bytes()).hexdigest()


@pytest.mark.parametrize("path", CASES, ids=lambda p: p.stem)
@pytest.mark.parametrize("layout,tag", [(BIOFEM_CKPT_VERTEX_ORDER, "ckpt_vertex"), (BIOFEM_CKPT_VEC, "ckpt_vec")])
def test_checkpoint_files_equal_the_references(path, layout, tag, tmp_path):
    w, meta, d = load(path)
    io.location_out(tmp_path, meta["ti"], d["x"], d["xn"], d["xd"], d["xdd"], layout=layout)
    for k in ("x", "xn", "xd", "xdd"):
        fn = f"{k}0_{meta['ti']:05d}.dat"
        assert sha(tmp_path / fn) == meta["sha256"][f"{tag}/{fn}"], fn
    back = io.location_in(tmp_path, meta["ti"], d["x"].size)
    for k in ("x", "xn", "xd", "xdd"):
        np.testing.assert_array_equal(back[k], d[k])


@pytest.mark.parametrize("path", CASES, ids=lambda p: p.stem)
def test_surface_vtk_equals_the_references(path, tmp_path):
    w, meta, d = load(path)
    m = w.build_mesh()
    from biofem.gpu import GpuShell
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, host_only=True)
    topo = sh.topology()
    mass = io.init_mass(m, topo["dA0"], meta["rho"], configs.H0)
    g = np.asarray(m.gamma_scale) * 1.0   # gamma_ramp_type 0, gamma 1
    io.write_surface(tmp_path, meta["ti"], m, d["x"], topo["xyz0_full"], g, d["Fint"], d["Fext"], d["Fdyn"],
                     d["xd"], mass, np.asarray(m.fib) if meta["lv"] else None)
    fn = f"surface00_{meta['ti']:05d}.vtk"
    ours = (tmp_path / fn).read_bytes()
    ref = d[f"text/{fn}"].tobytes()
    if ours != ref:   # show the first differing line
        for i, (a, b) in enumerate(zip(ours.decode().splitlines(), ref.decode().splitlines())):
            assert a == b, (i, a, b)
    assert hashlib.sha256(ours).hexdigest() == meta["sha256"][f"vtk/{fn}"]
    sh.close()


@pytest.mark.parametrize("path", CASES, ids=lambda p: p.stem)
def test_shell3d_vtk_equals_the_references(path, tmp_path):
    w, meta, d = load(path)
    m = w.build_mesh()
    io.write_shell3d(tmp_path, meta["ti"], m, d["x"], d["thickness"])
    fn = f"shell3d00_{meta['ti']:05d}.vtk"
    assert (tmp_path / fn).read_bytes() == d[f"text/{fn}"].tobytes()


@pytest.mark.parametrize("path", CASES, ids=lambda p: p.stem)
def test_oracle_thickness_is_update_element_thickness(path, oracle_lib):
    """h0 sqrt(mean_q C33) from the oracle's per-thickness-point C33 equals the
    reference's UpdateElementThickness output stored in the fixture."""
    w, meta, d = load(path)
    m = w.build_mesh()
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0)
    th = np.array([configs.H0 * np.sqrt(np.mean(o.elem_state(d["x"], e, w.n_qp)[1])) for e in range(m.n_elmt)])
    np.testing.assert_allclose(th, d["thickness"], rtol=1e-13, atol=0)
    assert np.ptp(th) > 0


def test_checkpoint_edge_cases(tmp_path):
    x = np.arange(12, dtype=np.float64) * 0.5
    io.location_out(tmp_path, 3, x, x + 1, x + 2, x + 3, ibi=2, layout=BIOFEM_CKPT_VEC)
    raw = (tmp_path / "x2_00003.dat").read_bytes()
    assert raw[:8] == (1211214).to_bytes(4, "big") + (12).to_bytes(4, "big")
    assert np.array_equal(np.frombuffer(raw[8:], ">f8"), x)
    # a VecView record with 64-bit header integers reads too
    (tmp_path / "x2_00004.dat").write_bytes((1211214).to_bytes(8, "big") + (12).to_bytes(8, "big") + raw[8:])
    for k in ("xn", "xd", "xdd"):
        (tmp_path / f"{k}2_00004.dat").write_bytes((tmp_path / f"{k}2_00003.dat").read_bytes())
    back = io.location_in(tmp_path, 4, 12, ibi=2)
    np.testing.assert_array_equal(back["x"], x)
    np.testing.assert_array_equal(back["xdd"], x + 3)
    with pytest.raises(BiofemError) as e:
        io.location_in(tmp_path, 3, 13, ibi=2)       # length differs from the mesh
    assert e.value.code == 92
    with pytest.raises(BiofemError) as e:
        io.location_in(tmp_path, 5, 12, ibi=2)       # no such checkpoint
    assert e.value.code == 91
    with pytest.raises(ValueError):
        io.location_out(tmp_path, 1, x, x, x, x[:-1])
