"""The O(N) topology builder and the basis tables of the product library,
checked against the oracle (which is bitwise-pinned to the reference) on the
CPU: no GPU is touched (BuildHostMesh makes no CUDA call)."""
import json

import numpy as np
import pytest

from conftest import GOLDEN
from biofem import configs
from biofem.gpu import GpuShell, basis_tables
from biofem.mesh import flat_membrane, set_random_activation

SHAPES = [(6, 5), (9, 7), (12, 8), (10, 6), (32, 24), (17, 3), (3, 11), (40, 2)]


@pytest.mark.parametrize("nx,ny", SHAPES)
def test_host_topology_equals_oracle(nx, ny, oracle_lib):
    w = configs.small(nx, ny, index=30)
    m = w.build_mesh()
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0)
    to = o.topology()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, host_only=True)
    th = sh.topology()
    for k in ("patch", "ire", "val", "irv", "gtri", "xyz0_full", "dA0"):
        assert np.array_equal(th[k], getattr(to, k)), k
    sh.close()


@pytest.mark.parametrize("freq", [3, 5])
def test_host_topology_equals_oracle_ellipsoid(freq, oracle_lib):
    """Truncated ellipsoid caps: isolated interior vertices of valence 5 and 7
    and a jagged cut rim (boundary valences 5, 6, 7)."""
    w = configs.LVWorkload(f"lv_f{freq}", freq, index=50 + freq)
    m = w.build_mesh()
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0)
    to = o.topology()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, host_only=True)
    th = sh.topology()
    assert th["ire"].sum() > 0
    for k in ("patch", "ire", "val", "irv", "gtri", "xyz0_full", "dA0"):
        assert np.array_equal(th[k], getattr(to, k)), k
    sh.close()


def _padded(m, pad):
    """The mesh with `pad` unreferenced nodes put in front, so every node id
    of its triangles is at least `pad`."""
    import copy
    m2 = copy.deepcopy(m)
    m2.xyz0 = np.vstack([np.zeros((pad, 3)), m.xyz0])
    m2.tri = (m.tri + pad).astype(np.int32)
    m2.bnodes = (m.bnodes + pad).astype(np.int32)
    return m2


def test_node_ids_beyond_the_reference_sentinel():
    """The reference's Patch() marks unresolved stencil slots with the node id
    1000000, which collides with real nodes from 10^6 on.  A mesh whose nodes
    all sit at ids 10^6 and above (node 1000000 among them) must get the
    small mesh's tables shifted by the offset."""
    pad = 1_000_000
    w = configs.small(8, 6, index=95)
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, host_only=True)
    t = sh.topology()
    sh.close()
    sh2 = GpuShell(_padded(m, pad), w, configs.MU, configs.BULK, configs.H0, host_only=True)
    t2 = sh2.topology()
    sh2.close()
    nen = np.where(np.asarray(t["ire"]) == 0, 12, np.asarray(t["val"]) + 6)
    pa, pb = np.asarray(t["patch"]).reshape(-1, 16), np.asarray(t2["patch"]).reshape(-1, 16)
    used = np.arange(16)[None, :] < nen[:, None]
    np.testing.assert_array_equal(pb[used], pa[used] + pad)
    np.testing.assert_array_equal(pb[~used], pa[~used])      # the reference's filler in the unused slots
    for k in ("ire", "val", "irv"):
        np.testing.assert_array_equal(t2[k], t[k])


@pytest.mark.parametrize("valence", range(3, 11))
def test_host_topology_equals_oracle_cone(valence, oracle_lib):
    """One interior vertex of valence 3..10 (the one-step subdivision of every
    valence the reference's tables cover, up to the 16-node patch)."""
    w = configs.cone(valence)
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, host_only=True)
    t = sh.topology()
    sh.close()
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0).topology()
    for k in ("patch", "ire", "val", "irv", "gtri"):
        np.testing.assert_array_equal(np.asarray(t[k]).reshape(np.asarray(getattr(o, k)).shape), getattr(o, k),
                                      err_msg=k)
    assert int(np.where(o.ire == 0, 12, o.val + 6).max()) == max(12, valence + 6)


@pytest.mark.parametrize("apex_vertex", [False, True], ids=["fan", "apex"])
@pytest.mark.parametrize("n_phi,n_theta", [(8, 4), (12, 6), (17, 5)])
def test_host_topology_equals_oracle_capped(n_phi, n_theta, apex_vertex, oracle_lib):
    """Apex-cap triangles (n_elmt_base): they count towards no node's
    valence, the apex ring's ghosts reflect through the base strip only, and
    a cap's patch holds only its corners (slots 3, 6, 7)."""
    w = configs.capped(n_phi, n_theta, apex_vertex)
    m = w.build_mesh()
    assert 0 < m.n_elmt_base < m.n_elmt
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, host_only=True)
    t = sh.topology()
    sh.close()
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0).topology()
    for k in ("patch", "ire", "val", "irv", "gtri", "xyz0_full", "dA0"):
        np.testing.assert_array_equal(np.asarray(t[k]).reshape(np.asarray(getattr(o, k)).shape), getattr(o, k),
                                      err_msg=k)
    cap = np.asarray(t["patch"]).reshape(-1, 16)[m.n_elmt_base:]
    np.testing.assert_array_equal(cap[:, [3, 6, 7]], m.tri[m.n_elmt_base:])
    assert (np.delete(cap, [3, 6, 7], axis=1) == 1_000_000).all()
    assert not np.asarray(t["ire"])[m.n_elmt_base:].any()
    # the apex ring's ghosts reflect through ring-1 nodes (the base strip),
    # not through the cap triangles that share the apex ring's edges
    g3 = np.asarray(t["ghost_nv3"])[:n_phi]
    assert ((g3 >= n_phi) & (g3 < 2 * n_phi)).all()


def test_host_topology_equals_oracle_holed_sphere(oracle_lib):
    """Holes whose rims are no boundary ring: the reference's stencil fill-in
    repeats a node in some patches (the row assembly then takes those slots
    one at a time)."""
    w = configs.SphereWorkload("sphere_f4_holed", 4, index=72, drop=(5, 200))
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, host_only=True)
    t = sh.topology()
    sh.close()
    o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0).topology()
    for k in ("patch", "ire", "val", "irv", "gtri", "xyz0_full", "dA0"):
        np.testing.assert_array_equal(np.asarray(t[k]).reshape(np.asarray(getattr(o, k)).shape), getattr(o, k),
                                      err_msg=k)
    P = np.asarray(t["patch"]).reshape(-1, 16)
    nen = np.where(np.asarray(t["ire"]) == 0, 12, np.asarray(t["val"]) + 6)
    assert sum(len(set(P[e, :nen[e]])) < nen[e] for e in range(len(P))) > 0


@pytest.mark.parametrize("name", ["C2_flat_256x192", "C4_lv_ellipsoid"])
def test_host_topology_matches_reference_checksum(name):
    """C2 (98,304 triangles) and C4 (200,614 triangles, valence-5/7 vertices):
    the reference's O(N^2) GlobalGhostInit/IrrVer/Patch() output is stored as
    SHA-256 checksums in tests/golden/{C2_flat_256x192,C4_lv_ellipsoid}.npz."""
    import hashlib
    path = GOLDEN / f"{name}.npz"
    d = np.load(path)
    meta = json.loads(str(d["meta"]))
    w = configs.ALL[name]
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, host_only=True)
    t = sh.topology()
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    assert sha(t["patch"]) == meta["sha_patch"]
    assert sha(t["ire"]) == meta["sha_ire"]
    assert sha(t["val"]) == meta["sha_val"]
    assert sha(t["irv"]) == meta["sha_irv"]
    assert sha(t["gtri"]) == meta["sha_gtri"]
    sh.close()


def test_basis_tables_equal_oracle_subdivision_weights(oracle_lib):
    tab = basis_tables()
    for v in range(3, 11):
        ref = oracle_lib.irregular_weights(v)
        assert np.array_equal(tab[v, :, : v + 6], ref), v
        assert not tab[v, :, v + 6:].any()


def test_pattern_is_symmetric_structure_on_free_rows():
    w = configs.small(10, 8, index=31)
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, host_only=True)
    rowptr, colind = sh.pattern()
    nb = sh.info.n_v + sh.info.n_ghosts
    assert rowptr[-1] == sh.nnzb and np.all(np.diff(rowptr) >= 1)
    for i in range(nb):
        cols = colind[rowptr[i]:rowptr[i + 1]]
        assert np.all(np.diff(cols) > 0) and i in cols
        assert cols.max() < sh.info.n_v or i >= sh.info.n_v  # ghost columns are folded away
    sh.close()


def test_invalid_inputs_raise():
    from biofem.gpu import BiofemError
    w = configs.small(6, 5, index=32)
    m = w.build_mesh()
    bad = configs.Workload("bad", 6, 5, n_qp=7)
    with pytest.raises(BiofemError) as ei:
        GpuShell(m, bad, configs.MU, configs.BULK, configs.H0, host_only=True)
    assert ei.value.code == 63
    m.tri[0, 0] = 10**6
    with pytest.raises(BiofemError):
        GpuShell(m, w, configs.MU, configs.BULK, configs.H0, host_only=True)
