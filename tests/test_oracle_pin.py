"""Pin the restated oracle (oracle/oracle.cpp) to the reference.

The golden fixtures in tests/golden/ were produced by the reference's own C
files (src/active_strain.c, bending.c, io.c, external.c, math.c compiled by
oracle/build_ref.py; generator: tests/golden/make_golden.py).  The oracle must
reproduce them BITWISE: topology tables (GlobalGhostInit/IrrVer/Patch) and the
FormFunctionFEM residual.  Where the reference sources are present the tests
also re-run the reference build live on fresh inputs.
"""
import json

import numpy as np
import pytest

from conftest import GOLDEN, golden_case
from biofem import configs
from biofem.configs import Workload

FULL = sorted(p for p in GOLDEN.glob("*.npz") if "meta" in np.load(p) and "R" in np.load(p))


def load_case(path):
    return golden_case(path)


@pytest.mark.parametrize("path", FULL, ids=lambda p: p.stem)
def test_oracle_matches_reference_golden(path, oracle_lib):
    w, meta, d = load_case(path)
    m = w.build_mesh()
    o = oracle_lib.setup(m, w, meta["mu"], meta["bulk"], meta["h0"])
    t = o.topology()
    for k in ("patch", "ire", "val", "irv", "gtri", "xyz0_full", "dA0"):
        assert np.array_equal(getattr(t, k), d[k]), k
    x = w.initial_x(m, t.xyz0_full)
    assert np.array_equal(x, d["x"])
    R, Fi, Fe = o.residual(x, want_parts=True)
    assert np.array_equal(R, d["R"])
    assert np.array_equal(Fi, d["Fint"])
    assert np.array_equal(Fe, d["Fext"])
    for k, ec in enumerate(d["sample_elems"]):
        S, C33, g, _ = o.elem_state(x, int(ec), w.n_qp)
        np.testing.assert_array_equal(S, d["sample_S"][k])
        np.testing.assert_array_equal(C33, d["sample_C33"][k])
        np.testing.assert_array_equal(g, d["sample_geom"][k])


def test_golden_fixtures_present():
    names = {p.stem for p in FULL}
    assert "C1_flat_32x24" in names and len(names) >= 4


def test_oracle_matches_live_reference(oracle_lib):
    """Fresh shape/parameters not in the fixtures, against the live reference build."""
    pytest.importorskip("oracle.build_ref")
    from oracle import build_ref
    if not build_ref.available():
        pytest.skip("reference sources not on this host")
    from oracle.pyoracle import RefOracle
    w = configs.small(7, 9, n_qp=4, c33_iters=2, activation="random", index=21, pressure=5e-4)
    m = w.build_mesh()
    ref = RefOracle().setup(m, w, configs.MU, configs.BULK, configs.H0)
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0)
    tr, to = ref.topology(), o.topology()
    for k in ("patch", "ire", "val", "irv", "gtri", "xyz0_full", "dA0"):
        assert np.array_equal(getattr(tr, k), getattr(to, k)), k
    x = w.initial_x(m, tr.xyz0_full)
    assert np.array_equal(ref.residual(x), o.residual(x))


@pytest.mark.parametrize("apex_vertex", [False, True], ids=["fan", "apex"])
def test_oracle_matches_live_reference_capped(apex_vertex, oracle_lib):
    """Apex-cap triangles (n_elmt_base) on a shape not in the fixtures, free
    rings, against the live reference build."""
    from oracle import build_ref
    if not build_ref.available():
        pytest.skip("reference sources not on this host")
    from oracle.pyoracle import RefOracle
    w = configs.capped(9, 4, apex_vertex, n_qp=2, c33_iters=2, index=23)
    m = w.build_mesh()
    ref = RefOracle().setup(m, w, configs.MU, configs.BULK, configs.H0)
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0)
    tr, to = ref.topology(), o.topology()
    for k in ("patch", "ire", "val", "irv", "gtri", "xyz0_full", "dA0"):
        assert np.array_equal(getattr(tr, k), getattr(to, k)), k
    x = w.initial_x(m, tr.xyz0_full)
    R = ref.residual(x)
    assert np.array_equal(R, o.residual(x))
    cap_nodes = np.unique(m.tri[m.n_elmt_base:])
    assert np.abs(R.reshape(-1, 3)[cap_nodes]).max() > 0.0


def test_oracle_matches_live_reference_holed_sphere(oracle_lib):
    """Holes not declared as rings (stencils that repeat a node), against the
    live reference build."""
    from oracle import build_ref
    if not build_ref.available():
        pytest.skip("reference sources not on this host")
    from oracle.pyoracle import RefOracle
    w = configs.SphereWorkload("sphere_f4_holed", 4, index=72, drop=(5, 200))
    m = w.build_mesh()
    ref = RefOracle().setup(m, w, configs.MU, configs.BULK, configs.H0)
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0)
    tr, to = ref.topology(), o.topology()
    for k in ("patch", "ire", "val", "irv", "gtri", "xyz0_full", "dA0"):
        assert np.array_equal(getattr(tr, k), getattr(to, k)), k
    x = w.initial_x(m, tr.xyz0_full)
    assert np.array_equal(ref.residual(x), o.residual(x))


def test_oracle_jvp_matches_central_differences(oracle_lib):
    """The dual-number directional derivative is the tangent checker; it must
    agree with central differences of the (bitwise-pinned) residual."""
    w = configs.small(8, 6, index=22)
    m = w.build_mesh()
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0)
    x = w.initial_x(m, o.topology().xyz0_full)
    v = np.random.default_rng(3).standard_normal(x.size)
    _, Jv = o.jvp(x, v)
    h = 1e-6
    fd = (o.residual(x + h * v) - o.residual(x - h * v)) / (2 * h)
    assert np.linalg.norm(fd - Jv) <= 1e-8 * np.linalg.norm(Jv)


def test_oracle_dense_jacobian_consistent_with_jvp(oracle_lib):
    w = configs.small(5, 4, index=23)
    m = w.build_mesh()
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0)
    x = w.initial_x(m, o.topology().xyz0_full)
    J = o.jacobian_dense(x)
    v = np.random.default_rng(4).standard_normal(x.size)
    _, Jv = o.jvp(x, v)
    np.testing.assert_allclose(J @ v, Jv, rtol=1e-12, atol=1e-14 * np.abs(Jv).max())


@pytest.mark.parametrize("path", FULL, ids=lambda p: p.stem)
def test_oracle_fast_topology_equals_the_reference_tables(path):
    """The oracle's corner-incident scans (O(N)) give the reference's tables
    bit for bit on every golden mesh, and the same residual."""
    from oracle.pyoracle import Oracle
    w, meta, d = load_case(path)
    m = w.build_mesh()
    o = Oracle().set_fast_topology(True)
    try:
        o.setup(m, w, meta["mu"], meta["bulk"], meta["h0"])
        t = o.topology()
        for k in ("patch", "ire", "val", "irv", "gtri", "xyz0_full", "dA0", "ghost_nv3"):
            if k in d:
                assert np.array_equal(getattr(t, k), d[k]), k
        assert np.array_equal(o.residual(d["x"]), d["R"])
    finally:
        o.set_fast_topology(False)


@pytest.mark.parametrize("name", ["C2_flat_256x192", "C4_lv_ellipsoid"])
def test_oracle_fast_topology_matches_reference_checksum(name):
    """C2 (98,304 triangles) and C4 (200,614 triangles, valence 5/7) through
    the oracle's O(N) scans: the SHA-256 of the reference's own
    Patch()/IrrVer() tables (tests/golden/C2_flat_256x192.npz,
    C4_lv_ellipsoid.npz, made by the reference build's O(N^2) searches)."""
    import hashlib
    from oracle.pyoracle import Oracle
    d = np.load(GOLDEN / f"{name}.npz")
    meta = json.loads(str(d["meta"]))
    w = configs.ALL[name]
    m = w.build_mesh()
    o = Oracle().set_fast_topology(True)
    try:
        o.setup(m, w, configs.MU, configs.BULK, configs.H0)
        t = o.topology()
    finally:
        o.set_fast_topology(False)
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a, dtype=np.int32).tobytes()).hexdigest()
    for k in ("patch", "ire", "val", "irv"):
        assert sha(getattr(t, k)) == meta[f"sha_{k}"], k
