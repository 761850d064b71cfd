"""Centroid basis-derivative tables: the reference's four-decimal values
(active_strain.c:69-88, the default) and the exact rationals they round (an
extension for meshes much finer than the shell thickness).

Known answers: the exact first-derivative rows are k/324 and the
second-derivative rows k/108; rounded to four decimals they give back the
reference's constants; their rows sum to zero, so a flat uniform patch has
zero second derivatives.  The reference tables' second-derivative rows sum
to -1e-4, -1e-4 and 2e-4, which is what folds the thickness points of fine
meshes.
"""
import numpy as np
import pytest

from biofem import configs


def tables(kind):
    import ctypes
    from biofem.gpu import load_library, _check, _ptr
    lib = load_library()
    out = np.zeros(11 * 80)
    _check(lib, lib.GetGpuBasisTablesKind(ctypes.c_int32(kind), _ptr(out)))
    return out.reshape(11, 5, 16)


def test_exact_tables_round_to_the_reference_constants():
    ref, ex = tables(0)[0, :, :12], tables(1)[0, :, :12]
    np.testing.assert_array_equal(np.round(ex, 4), ref)
    np.testing.assert_allclose(ex[:2] * 324, np.round(ex[:2] * 324), rtol=0, atol=1e-12)
    np.testing.assert_allclose(ex[2:] * 108, np.round(ex[2:] * 108), rtol=0, atol=1e-12)
    np.testing.assert_allclose(ex.sum(1), 0.0, atol=1e-15)
    np.testing.assert_allclose(ref.sum(1), [0.0, 0.0, -1e-4, -1e-4, 2e-4], atol=1e-15)


@pytest.mark.parametrize("kind", [0, 1])
def test_normal_derivative_of_a_flat_patch(kind):
    """a3,alpha = (A_a1 x a2 + a1 x A_a2) / |a1 x a2| (active_strain.c:745-762)
    vanishes on a flat sheet with the exact tables; with the four-decimal
    tables it is ~1e-4 |x| / h, independent of the sheet being flat."""
    from biofem.gpu import GpuShell
    w = configs.Workload("flat_12x8", 12, 8, index=60, basis=kind)
    m = w.build_mesh()
    sh = GpuShell(m, w, configs.MU, configs.BULK, configs.H0, host_only=True)
    t = sh.topology()
    T = tables(kind)
    X = t["xyz0_full"]
    worst = 0.0
    for ec in np.where(t["ire"] == 0)[0]:
        P = X[t["patch"][ec, :12]]
        a1, a2 = T[0, 0, :12] @ P, T[0, 1, :12] @ P
        Aaa, Abb, Aab = T[0, 2, :12] @ P, T[0, 3, :12] @ P, T[0, 4, :12] @ P
        s = np.linalg.norm(np.cross(a1, a2))
        a31 = (np.cross(Aaa, a2) + np.cross(a1, Aab)) / s
        a32 = (np.cross(Aab, a2) + np.cross(a1, Abb)) / s
        worst = max(worst, np.abs(a31).max(), np.abs(a32).max())
    if kind == 1:
        assert worst <= 1e-12, worst
    else:
        assert worst > 1e-4, worst
    # the irregular tables follow the chosen regular table
    for v in (5, 7):
        assert np.abs(T[v, 2:, : v + 6].sum(1)).max() <= (1e-13 if kind else 1e-2)
    sh.close()


def test_oracle_follows_the_table_choice(oracle_lib):
    w0 = configs.Workload("flat_10x8", 10, 8, z_sigma=1e-3, activation="random", index=61)
    w1 = configs.Workload("flat_10x8", 10, 8, z_sigma=1e-3, activation="random", index=61, basis=1)
    m = w0.build_mesh()
    x = None
    out = []
    for w in (w0, w1):
        o = oracle_lib.setup(m, w, configs.MU, configs.BULK, configs.H0)
        if x is None:
            from biofem.gpu import GpuShell
            sh = GpuShell(m, w0, configs.MU, configs.BULK, configs.H0, host_only=True)
            x = w0.initial_x(m, sh.topology()["xyz0_full"])
            sh.close()
        out.append(o.residual(x))
    oracle_lib.setup(m, w0, configs.MU, configs.BULK, configs.H0)   # leave the default tables selected
    d = np.linalg.norm(out[1] - out[0]) / np.linalg.norm(out[0])
    assert 1e-9 < d < 1e-1, d
