"""ctypes bindings to the oracle libraries (TEST INFRASTRUCTURE ONLY).

``Oracle``   -> oracle/_build/liboracle.so  (restated oracle, builds anywhere)
``RefOracle`` -> oracle/_ref/libbiofem_ref.so (the reference's own C files;
                 only where the reference sources exist)

Both expose the same calls: setup(mesh, workload), topology(), residual(x).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_c_int, _c_dbl, _vp = ctypes.c_int, ctypes.c_double, ctypes.c_void_p


def _p(a: np.ndarray):
    return a.ctypes.data_as(_vp)


@dataclass
class Topology:
    patch: np.ndarray      # (n_elmt, 16) int32
    ire: np.ndarray
    val: np.ndarray
    irv: np.ndarray
    gtri: np.ndarray       # (n_elmt + 2 n_ghosts, 3)
    xyz0_full: np.ndarray  # (n_v + n_ghosts, 3)
    dA0: np.ndarray
    ghost_nv3: np.ndarray | None = None


class _Base:
    lib: ctypes.CDLL
    prefix: str

    def _fn(self, name):
        return getattr(self.lib, f"{self.prefix}_{name}")

    def _select_basis(self, kind: int, tnormal: int = 0):
        """Basis-derivative tables (0 the reference's four-decimal values, 1 the
        exact rationals) and thickness metric (0 the reference's a3,alpha, 1
        its tangential part): extensions only the restated oracle has."""
        for name, val in (("set_basis", kind), ("set_thickness_normal", tnormal)):
            fn = getattr(self.lib, f"{self.prefix}_{name}", None)
            if fn is None:
                if val:
                    raise RuntimeError(f"the reference build has no {name} extension")
                continue
            fn.argtypes = [_c_int]
            rc = fn(int(val))
            if rc:
                raise RuntimeError(f"{self.prefix}_{name} failed with code {rc}")

    def _select_load(self, w):
        """Pressure kind (follower / dead load) and activation kind (fibre /
        isotropic) of the workload for the next setup."""
        f = self._fn("set_load_options")
        f.argtypes = [_c_int, _c_int]
        f(int(getattr(w, "dead_load", 0)), int(getattr(w, "iso_act", 0)))

    def _select_elmt_base(self, mesh):
        """ibm->n_elmt_base of the next setup: 0, or the count of base
        elements (the rest are apex-cap triangles)."""
        f = self._fn("set_elmt_base")
        f.argtypes = [_c_int]
        f(int(getattr(mesh, "n_elmt_base", 0)))

    def setup(self, mesh, w, mu: float, bulk: float, h0: float, gamma: float = 1.0, clamp: bool = True):
        from_mesh = dict(
            tri=np.ascontiguousarray(mesh.tri, dtype=np.int32),
            xyz=np.ascontiguousarray(mesh.xyz0, dtype=np.float64),
            nb=np.ascontiguousarray(mesh.n_bnodes, dtype=np.int32),
            bn=np.ascontiguousarray(mesh.bnodes, dtype=np.int32),
            fib=np.ascontiguousarray(mesh.fib, dtype=np.float64),
            gs=np.ascontiguousarray(mesh.gamma_scale, dtype=np.float64),
        )
        self._keep = from_mesh
        self._select_basis(getattr(w, "basis", 0), getattr(w, "tnormal", 0))
        self._select_load(w)
        self._select_elmt_base(mesh)
        f = self._fn("setup")
        f.argtypes = [_c_int, _c_int, _vp, _vp, _c_int, _vp, _vp, _vp, _vp,
                      _c_int, _c_int, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_int]
        rc = f(mesh.n_v, mesh.n_elmt, _p(from_mesh["tri"]), _p(from_mesh["xyz"]), mesh.n_edge,
               _p(from_mesh["nb"]), _p(from_mesh["bn"]), _p(from_mesh["fib"]), _p(from_mesh["gs"]),
               w.n_qp, w.c33_iters, mu, bulk, h0, gamma, w.pressure,
               int(clamp and getattr(w, "clamp", True) and mesh.n_edge > 0))
        if rc:
            raise RuntimeError(f"{self.prefix}_setup failed with code {rc}")
        ng, nd = _c_int(), _c_int()
        self._fn("sizes")(ctypes.byref(ng), ctypes.byref(nd))
        self.n_v, self.n_elmt = mesh.n_v, mesh.n_elmt
        self.n_ghosts, self.n_dof = ng.value, nd.value
        return self

    def residual(self, x: np.ndarray, want_parts: bool = False):
        x = np.ascontiguousarray(x, dtype=np.float64)
        R = np.zeros(self.n_dof)
        Fi = np.zeros(self.n_dof)
        Fe = np.zeros(self.n_dof)
        rc = self._fn("residual")(_p(x), _p(R), _p(Fi), _p(Fe))
        if rc:
            raise RuntimeError(f"{self.prefix}_residual failed with code {rc}")
        return (R, Fi, Fe) if want_parts else R


class Oracle(_Base):
    prefix = "oracle"

    def residual_parts(self, x):
        """(R, Fint, Fext, Fdyn), the forces unscaled."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = [np.zeros(self.n_dof) for _ in range(4)]
        f = self.lib.oracle_residual_parts
        f.argtypes = [_vp] * 5
        rc = f(_p(x), *[_p(a) for a in out])
        if rc:
            raise RuntimeError(f"oracle_residual_parts failed with code {rc}")
        return tuple(out)

    # ---- dynamic term (FDynamic / xAccVel) and per-element activation ----
    def set_dynamics(self, dt=None, rho=0.0, newmark_gamma=0.5, dampfactor=0.0, timeinteg=0, damping=0):
        f = self.lib.oracle_set_dynamics
        f.argtypes = [_c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_int, _c_int]
        rc = f(0.0 if dt is None else float(dt), rho, newmark_gamma, dampfactor, int(timeinteg), int(damping))
        if rc:
            raise RuntimeError(f"oracle_set_dynamics failed with code {rc}")

    def set_dynamic_state(self, xn=None, xnm1=None, xd=None, xdd=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (xn, xnm1, xd, xdd)]
        f = self.lib.oracle_set_dynamic_state
        f.argtypes = [_vp] * 4
        rc = f(*[None if a is None else _p(a) for a in arrs])
        if rc:
            raise RuntimeError(f"oracle_set_dynamic_state failed with code {rc}")

    def dynamic_state(self):
        out = [np.zeros(self.n_dof) for _ in range(4)]
        f = self.lib.oracle_get_dynamic_state
        f.argtypes = [_vp] * 4
        rc = f(*[_p(a) for a in out])
        if rc:
            raise RuntimeError(f"oracle_get_dynamic_state failed with code {rc}")
        return dict(zip(("xn", "xnm1", "xd", "xdd"), out))

    def dynamic_update(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        f = self.lib.oracle_dynamic_update
        f.argtypes = [_vp]
        rc = f(_p(x))
        if rc:
            raise RuntimeError(f"oracle_dynamic_update failed with code {rc}")

    def set_element_gamma(self, gamma_e):
        g = np.ascontiguousarray(gamma_e, dtype=np.float64)
        assert g.size == self.n_elmt
        f = self.lib.oracle_set_element_gamma
        f.argtypes = [_vp]
        rc = f(_p(g))
        if rc:
            raise RuntimeError(f"oracle_set_element_gamma failed with code {rc}")

    def __init__(self, build: bool = True):
        from . import build_oracle  # type: ignore
        path = build_oracle.build() if build else build_oracle.LIB
        self.lib = ctypes.CDLL(str(path))

    def setup_given_topology(self, mesh, w, topo: dict, mu: float, bulk: float, h0: float,
                             gamma: float = 1.0, clamp: bool = True):
        """oracle_setup with the subdivision tables supplied (dict with patch,
        ire, val, irv, gtri, xyz0_full as returned by GetGpuTopology)."""
        ng = int(mesh.n_bnodes.sum())
        gtri = np.ascontiguousarray(topo["gtri"], dtype=np.int32)
        # the reflected interior node of ghost g: the ghost's main triangle is
        # (nv1, nv2, ghost); recover nv3 from x_g = x_nv2 + x_nv1 - x_nv3 is not
        # possible from positions alone, so take it from the caller if present
        gnv3 = np.ascontiguousarray(topo["ghost_nv3"], dtype=np.int32)
        keep = dict(gtri=gtri, x=np.ascontiguousarray(topo["xyz0_full"], dtype=np.float64),
                    nb=np.ascontiguousarray(mesh.n_bnodes, dtype=np.int32),
                    bn=np.ascontiguousarray(mesh.bnodes, dtype=np.int32),
                    patch=np.ascontiguousarray(topo["patch"], dtype=np.int32),
                    ire=np.ascontiguousarray(topo["ire"], dtype=np.int32),
                    val=np.ascontiguousarray(topo["val"], dtype=np.int32),
                    irv=np.ascontiguousarray(topo["irv"], dtype=np.int32), gnv3=gnv3,
                    fib=np.ascontiguousarray(mesh.fib, dtype=np.float64),
                    gs=np.ascontiguousarray(mesh.gamma_scale, dtype=np.float64))
        self._keep = keep
        self._select_basis(getattr(w, "basis", 0), getattr(w, "tnormal", 0))
        self._select_load(w)
        self._select_elmt_base(mesh)
        f = self.lib.oracle_setup_given_topology
        f.argtypes = [_c_int, _c_int, _vp, _vp, _c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                      _c_int, _c_int, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_int]
        rc = f(mesh.n_v, mesh.n_elmt, _p(keep["gtri"]), _p(keep["x"]), mesh.n_edge, _p(keep["nb"]), _p(keep["bn"]),
               _p(keep["patch"]), _p(keep["ire"]), _p(keep["val"]), _p(keep["irv"]), _p(keep["gnv3"]),
               _p(keep["fib"]), _p(keep["gs"]), w.n_qp, w.c33_iters, mu, bulk, h0, gamma, w.pressure,
               int(clamp and getattr(w, "clamp", True) and mesh.n_edge > 0))
        if rc:
            raise RuntimeError(f"oracle_setup_given_topology failed with code {rc}")
        ng_, nd = _c_int(), _c_int()
        self.lib.oracle_sizes(ctypes.byref(ng_), ctypes.byref(nd))
        self.n_v, self.n_elmt = mesh.n_v, mesh.n_elmt
        self.n_ghosts, self.n_dof = ng_.value, nd.value
        return self

    def set_threads(self, n: int):
        self.lib.oracle_set_threads(int(n))

    def set_fast_topology(self, on: bool = True):
        """setup() then builds GlobalGhostInit / IrrVer / Patch with
        corner-incident scans (O(N), the same tables as the reference's full
        scans)."""
        self.lib.oracle_set_fast_topology(int(bool(on)))
        return self

    def topology(self) -> Topology:
        ne, ng, nv = self.n_elmt, self.n_ghosts, self.n_v
        t = Topology(np.zeros((ne, 16), np.int32), np.zeros(ne, np.int32), np.zeros(ne, np.int32),
                     np.zeros(ne, np.int32), np.zeros((ne + 2 * ng, 3), np.int32),
                     np.zeros((nv + ng, 3)), np.zeros(ne), np.zeros(ng, np.int32))
        rc = self.lib.oracle_topology(_p(t.patch), _p(t.ire), _p(t.val), _p(t.irv), _p(t.gtri),
                                      _p(t.xyz0_full), _p(t.dA0), _p(t.ghost_nv3))
        if rc:
            raise RuntimeError(rc)
        return t

    def jvp(self, x: np.ndarray, v: np.ndarray):
        x = np.ascontiguousarray(x, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        R = np.zeros(self.n_dof)
        Jv = np.zeros(self.n_dof)
        rc = self.lib.oracle_jvp(_p(x), _p(v), _p(R), _p(Jv))
        if rc:
            raise RuntimeError(rc)
        return R, Jv

    def jacobian_dense(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        J = np.zeros((self.n_dof, self.n_dof))  # filled column major -> transpose
        rc = self.lib.oracle_jacobian_dense(_p(x), _p(J))
        if rc:
            raise RuntimeError(rc)
        return J.T.copy()

    def jmv(self, x: np.ndarray, V: np.ndarray) -> np.ndarray:
        """J V for a block of directions V (k x ndof), exact (dual numbers)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros_like(V, dtype=np.float64)
        for k0 in range(0, V.shape[0], 8):
            blk = np.ascontiguousarray(V[k0:k0 + 8], dtype=np.float64)
            JV = np.zeros_like(blk)
            rc = self.lib.oracle_jmv8(_p(x), _p(blk), blk.shape[0], _p(JV))
            if rc:
                raise RuntimeError(rc)
            out[k0:k0 + 8] = JV
        return out

    def sparse_jacobian(self, x: np.ndarray, topo):
        """Exact sparse Jacobian of the residual: columns grouped by a greedy
        colouring of the nodes whose residual rows are disjoint, one dual
        direction per (colour, component)."""
        import scipy.sparse as sp
        nv, ne, ng = self.n_v, self.n_elmt, self.n_ghosts
        patch, ire, val = topo.patch, topo.ire, topo.val
        gtri = topo.gtri
        gnv3 = topo.ghost_nv3
        # ghost parents (nv1, nv2 from the ghost's main triangle, nv3 stored)
        parents = {}
        for g in range(ng):
            a, b = gtri[ne + 2 * g][:2]
            parents[nv + g] = (int(a), int(b), int(gnv3[g]))
        infl = [set([j]) for j in range(nv)]         # rows influenced by column node j
        for e in range(ne):
            nen = 12 if ire[e] == 0 else val[e] + 6
            nodes = [int(q) for q in patch[e, :nen] if q != 1000000]   # a cap element's unused slots
            rows = {q for q in nodes if q < nv}
            cols = set()
            for q in nodes:
                cols.update(parents[q] if q >= nv else (q,))
            for j in cols:
                infl[j] |= rows
        colors, used = [], []
        for j in range(nv):
            for c, u in enumerate(used):
                if not (u & infl[j]):
                    colors[c].append(j); u |= infl[j]
                    break
            else:
                colors.append([j]); used.append(set(infl[j]))
        n = self.n_dof
        V = np.zeros((3 * len(colors), n))
        for c, js in enumerate(colors):
            for d in range(3):
                V[3 * c + d, [3 * j + d for j in js]] = 1.0
        JV = self.jmv(x, V)
        rows_i, cols_j, vals = [], [], []
        for c, js in enumerate(colors):
            for j in js:
                rset = np.array(sorted(infl[j]))
                ridx = (3 * rset[:, None] + np.arange(3)[None, :]).ravel()
                for d in range(3):
                    v = JV[3 * c + d, ridx]
                    nz = v != 0.0
                    rows_i.append(ridx[nz]); cols_j.append(np.full(nz.sum(), 3 * j + d)); vals.append(v[nz])
        J = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows_i), np.concatenate(cols_j))), shape=(n, n))
        return J, len(colors)

    def newton(self, x0: np.ndarray, topo, rtol: float = 1e-10, max_it: int = 30, verbose: bool = False,
               jacobian_its: int | None = None):
        """Newton load step on the oracle residual with its exact sparse
        Jacobian (ghost rows/columns replaced by identity) and a direct solve;
        backtracking on ||R|| as the GPU solver does.  The converged state
        depends only on R.  ``jacobian_its`` = k rebuilds the Jacobian on the
        first k iterations only and then keeps its factorisation (a chord
        iteration: cheaper, linearly convergent, same root)."""
        import scipy.sparse as sp
        import scipy.sparse.linalg as spla
        x = np.array(x0, dtype=np.float64)
        nreal = 3 * self.n_v
        R = self.residual(x)
        r0 = np.linalg.norm(R)
        hist = [r0]
        for it in range(max_it):
            rn = np.linalg.norm(R)
            if rn <= rtol * r0:
                break
            if jacobian_its is None or it < jacobian_its:
                J, _ = self.sparse_jacobian(x, topo)
                J = J.tolil()
                for i in range(nreal, self.n_dof):
                    J[i, i] = 1.0
                lu = spla.splu(J.tocsc())
            dx = lu.solve(-R)
            dx[nreal:] = 0.0
            alpha = 1.0
            for _ in range(12):
                xt = x + alpha * dx
                Rt = self.residual(xt)
                if np.linalg.norm(Rt) <= (1 - 1e-4 * alpha) * rn:
                    break
                alpha *= 0.5
            x, R = xt, Rt
            hist.append(np.linalg.norm(R))
            if verbose:
                print(f"newton {it}: |R| = {hist[-1]:.3e} alpha {alpha}")
        return x, hist

    def jfnk_newton_step(self, x: np.ndarray, rtol_lin: float = 1e-5, restart: int = 30, max_lin: int = 1000):
        """One Newton step of the reference's own solver, restated on the
        oracle residual: SNES newtonls with a matrix-free Jacobian
        (MatCreateSNESMF, main.c:461-466), J v by the MatMFFD 'wp' difference
        (R(x + h v) - R(x)) / h with h = sqrt(eps) sqrt(1 + |x|) / |v|,
        unpreconditioned GMRES(30) to the default relative tolerance 1e-5 (PETSc
        defaults; PETSc itself is absent here), then backtracking on ||R||
        (halving; PETSc's bt line search fits a cubic).  Returns
        (x_new, R_new, stats) with stats: residual_evaluations, gmres_its,
        lin_converged, seconds."""
        import time
        import scipy.sparse.linalg as spla
        t0 = time.perf_counter()
        x = np.array(x, dtype=np.float64)
        nres = 0
        R = self.residual(x)
        nres += 1
        eps_rel = float(np.sqrt(np.finfo(np.float64).eps))
        unorm = float(np.linalg.norm(x))

        def mv(v):
            nonlocal nres
            vn = float(np.linalg.norm(v))
            if vn == 0.0:
                return np.zeros_like(v)
            h = eps_rel * np.sqrt(1.0 + unorm) / vn
            nres += 1
            return (self.residual(x + h * v) - R) / h

        n = R.size
        A = spla.LinearOperator((n, n), matvec=mv, dtype=np.float64)
        its = [0]

        def cb(_):
            its[0] += 1

        cycles = max(1, (max_lin + restart - 1) // restart)
        try:
            dx, info = spla.gmres(A, -R, rtol=rtol_lin, atol=0.0, restart=restart, maxiter=cycles,
                                  callback=cb, callback_type="pr_norm")
        except TypeError:   # scipy before the rtol keyword
            dx, info = spla.gmres(A, -R, tol=rtol_lin, atol=0.0, restart=restart, maxiter=cycles,
                                  callback=cb, callback_type="pr_norm")
        rn = float(np.linalg.norm(R))
        alpha = 1.0
        for _ in range(12):
            xt = x + alpha * dx
            Rt = self.residual(xt)
            nres += 1
            if np.linalg.norm(Rt) <= (1 - 1e-4 * alpha) * rn:
                break
            alpha *= 0.5
        stats = {"residual_evaluations": nres, "gmres_its": its[0], "lin_converged": info == 0,
                 "step_length": alpha, "seconds": time.perf_counter() - t0}
        return xt, Rt, stats

    def elem_state(self, x: np.ndarray, ec: int, n_qp: int):
        x = np.ascontiguousarray(x, dtype=np.float64)
        S = np.zeros((n_qp, 3, 3))
        C33 = np.zeros(n_qp)
        g = np.zeros((8, 3))
        Fb = np.zeros(48)
        rc = self.lib.oracle_elem_state(_p(x), int(ec), _p(S), _p(C33), _p(g), _p(Fb))
        if rc:
            raise RuntimeError(rc)
        return S, C33, g, Fb

    def irregular_weights(self, v: int) -> np.ndarray:
        out = np.zeros(5 * (v + 6))
        rc = self.lib.oracle_irregular_weights(int(v), _p(out))
        if rc:
            raise RuntimeError(rc)
        return out.reshape(5, v + 6)


class RefOracle(_Base):
    prefix = "ref"

    def __init__(self, dyn: bool = False):
        """dyn: load oracle/_ref/libbiofem_ref_dyn.so, the build that also holds
        the reference's main.c (FDynamic, xAccVel) and material.c."""
        from . import build_ref  # type: ignore
        path = build_ref.build_dyn() if dyn else build_ref.build()
        if path is None:
            raise FileNotFoundError("reference sources are not present on this host")
        self.lib = ctypes.CDLL(str(path))

    # ---- the reference's own dynamic term (main.c FDynamic / xAccVel) ----
    def set_dynamics(self, dt, rho=0.0, newmark_gamma=0.5, dampfactor=0.0, timeinteg=0, damping=0):
        f = self.lib.ref_set_dynamics
        f.argtypes = [_c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_int, _c_int]
        f(float(dt), float(rho), float(newmark_gamma), float(dampfactor), int(timeinteg), int(damping))

    def fdynamic(self, x, xn, xnm1, xd, xdd, dmplex: bool = True):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, xn, xnm1, xd, xdd)]
        out = np.zeros(self.n_dof)
        f = self.lib.ref_fdynamic
        f.argtypes = [_vp] * 6 + [_c_int]
        rc = f(*[_p(a) for a in arrs], _p(out), int(dmplex))
        if rc:
            raise RuntimeError(f"ref_fdynamic failed with code {rc}")
        return out

    def xaccvel(self, x, xn, xd, xdd, dmplex: bool = True):
        x, xn = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, xn))
        xd, xdd = (np.array(a, dtype=np.float64) for a in (xd, xdd))
        f = self.lib.ref_xaccvel
        f.argtypes = [_vp] * 4 + [_c_int]
        rc = f(_p(x), _p(xn), _p(xd), _p(xdd), int(dmplex))
        if rc:
            raise RuntimeError(f"ref_xaccvel failed with code {rc}")
        return xd, xdd

    def topology(self) -> Topology:
        ne, ng, nv = self.n_elmt, self.n_ghosts, self.n_v
        t = Topology(np.zeros((ne, 16), np.int32), np.zeros(ne, np.int32), np.zeros(ne, np.int32),
                     np.zeros(ne, np.int32), np.zeros((ne + 2 * ng, 3), np.int32),
                     np.zeros((nv + ng, 3)), np.zeros(ne))
        rc = self.lib.ref_topology(_p(t.patch), _p(t.ire), _p(t.val), _p(t.irv), _p(t.gtri),
                                   _p(t.xyz0_full), _p(t.dA0))
        if rc:
            raise RuntimeError(rc)
        return t

    def elem_state(self, ec: int, n_qp: int):
        S = np.zeros((n_qp, 3, 3))
        C33 = np.zeros(n_qp)
        g = np.zeros((8, 3))
        rc = self.lib.ref_elem_state(int(ec), _p(S), _p(C33), _p(g))
        if rc:
            raise RuntimeError(rc)
        return S, C33, g

    # ---- the reference's own on-disk writers and readers (io.c) ----
    def location_out(self, out_dir, ti: int, x, xn, xd, xdd, ibi: int = 0, dmplex: bool = True):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, xn, xd, xdd)]
        f = self.lib.ref_location_out
        f.argtypes = [ctypes.c_char_p, _c_int, _c_int, _vp, _vp, _vp, _vp, _c_int]
        rc = f(str(out_dir).encode(), ti, ibi, *[_p(a) for a in arrs], int(dmplex))
        if rc:
            raise RuntimeError(f"ref_location_out failed with code {rc}")

    def location_in(self, out_dir, ti: int, ibi: int = 0, dmplex: bool = True):
        out = [np.zeros(self.n_dof) for _ in range(4)]
        f = self.lib.ref_location_in
        f.argtypes = [ctypes.c_char_p, _c_int, _c_int, _vp, _vp, _vp, _vp, _c_int]
        rc = f(str(out_dir).encode(), ti, ibi, *[_p(a) for a in out], int(dmplex))
        if rc:
            raise RuntimeError(f"ref_location_in failed with code {rc}")
        return dict(zip(("x", "xn", "xd", "xdd"), out))

    def output_vtk(self, out_dir, ti: int, x, Fdyn, xd, rho: float, lv: bool = False, ibi: int = 0):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, Fdyn, xd)]
        f = self.lib.ref_output_vtk
        f.argtypes = [ctypes.c_char_p, _c_int, _c_int, _vp, _vp, _vp, _c_dbl, _c_int]
        rc = f(str(out_dir).encode(), ti, ibi, *[_p(a) for a in arrs], float(rho), int(lv))
        if rc:
            raise RuntimeError(f"ref_output_vtk failed with code {rc}")

    def thickness(self, x, out_dir=None, ti: int = 0, ibi: int = 0):
        x = np.ascontiguousarray(x, dtype=np.float64)
        th = np.zeros(self.n_elmt)
        f = self.lib.ref_thickness
        f.argtypes = [ctypes.c_char_p, _c_int, _c_int, _vp, _vp]
        rc = f(None if out_dir is None else str(out_dir).encode(), ti, ibi, _p(x), _p(th))
        if rc:
            raise RuntimeError(f"ref_thickness failed with code {rc}")
        return th
