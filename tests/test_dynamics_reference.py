"""The oracle's dynamic term against the reference's own: FDynamic and xAccVel
(main.c:1157-1412) of the reference's main.c, compiled with its hot-path files
and material.c into oracle/_ref/libbiofem_ref_dyn.so (oracle/build_ref.py).
The committed fixtures tests/golden/dyn_*.npz (tests/golden/make_dyn_golden.py)
hold the reference's outputs, so the pin runs wherever the oracle builds; the
live comparison runs where the reference sources exist."""
import numpy as np
import pytest

from biofem import configs
from conftest import GOLDEN

DYN_CASES = {
    "dyn_flat_6x5": lambda: configs.small(6, 5, index=93, pressure=0.0),
    "dyn_lv_f2": lambda: configs.LVWorkload("lv_f2", 2, index=94),
}


def _oracle_dyn_outputs(o, f, tag):
    """The oracle's FDynamic (through the residual's Fdyn part) and xAccVel at
    the fixture's state, for scheme `tag`."""
    dt, rho, dampf = (float(v) for v in f["consts"])
    ti = 0 if tag == "newmark" else 1
    o.set_dynamics(dt, rho, float(f[f"gamma_{tag}"]), dampf, ti, 1)
    o.set_dynamic_state(xn=f["xn"], xnm1=f["xnm1"], xd=f["xd"], xdd=f["xdd"])
    _, _, _, Fdyn = o.residual_parts(f["x"])
    o.dynamic_update(f["x"])
    s = o.dynamic_state()
    o.set_dynamics(None)
    return Fdyn, s["xd"], s["xdd"]


@pytest.mark.parametrize("case", sorted(DYN_CASES))
@pytest.mark.parametrize("tag", ["newmark", "central"])
def test_oracle_dynamic_term_equals_the_reference_fixture(oracle_lib, case, tag):
    """FDynamic and xAccVel of the oracle equal, bit for bit, the reference's
    own main.c functions on the path an active-strain run takes (DMPlex
    context initialised), as recorded in tests/golden/dyn_*.npz; the serial
    path of the same functions (ghost and bridging triangles included)
    differs on free boundary rows, which the fixtures record too."""
    f = np.load(GOLDEN / f"{case}.npz")
    w = DYN_CASES[case]()
    m = w.build_mesh()
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0, clamp=bool(f["clamp"]))
    Fdyn, xd, xdd = _oracle_dyn_outputs(o, f, tag)
    np.testing.assert_array_equal(Fdyn, f[f"Fdyn_{tag}_dmplex"])
    np.testing.assert_array_equal(xd, f[f"xd_{tag}_dmplex"])
    np.testing.assert_array_equal(xdd, f[f"xdd_{tag}_dmplex"])
    if not bool(f["clamp"]):   # free edges: the serial path's extra ghost-triangle mass shows
        assert np.abs(f[f"Fdyn_{tag}_serial"] - f[f"Fdyn_{tag}_dmplex"])[: 3 * m.n_v].max() > 0


def test_oracle_dynamic_term_equals_the_live_reference(oracle_lib):
    """The same against the reference build itself, at a state of its own."""
    from oracle.pyoracle import RefOracle
    try:
        ref = RefOracle(dyn=True)
    except FileNotFoundError:
        pytest.skip("reference sources not present")
    w = configs.small(7, 5, index=96, pressure=0.0)
    m = w.build_mesh()
    ref.setup(m, w, configs.MU, configs.BULK, configs.H0, clamp=False)
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0, clamp=False)
    x0 = w.initial_x(m, ref.topology().xyz0_full)
    rng = np.random.default_rng(97)
    n = x0.size
    f = dict(x=x0 + 1e-3 * rng.standard_normal(n), xn=x0 + 1e-3 * rng.standard_normal(n),
             xnm1=x0 + 1e-3 * rng.standard_normal(n), xd=rng.standard_normal(n), xdd=rng.standard_normal(n),
             consts=np.array([1e-3, 0.9, 3.0]), gamma_newmark=np.array(0.55), gamma_central=np.array(0.5))
    for tag, ti in (("newmark", 0), ("central", 1)):
        Fdyn, xd, xdd = _oracle_dyn_outputs(o, f, tag)
        ref.set_dynamics(1e-3, 0.9, float(f[f"gamma_{tag}"]), 3.0, ti, 1)
        np.testing.assert_array_equal(Fdyn, ref.fdynamic(f["x"], f["xn"], f["xnm1"], f["xd"], f["xdd"]))
        rxd, rxdd = ref.xaccvel(f["x"], f["xn"], f["xd"], f["xdd"])
        np.testing.assert_array_equal(xd, rxd)
        np.testing.assert_array_equal(xdd, rxdd)
