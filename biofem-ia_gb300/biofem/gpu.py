"""Host-side mirror of BioFEM-IA's residual / Jacobian interface over the
C-ABI in include/biofem_gpu.h (libbiofem_gpu.so, sm_103a).

The reference evaluates R(x) inside its PETSc SNES callback
``FormFunctionFEM(SNES, Vec x, Vec R, void *ctx)`` (main.c:757-1032) and
never forms a Jacobian (matrix-free, main.c:464-466).  ``GpuShell`` holds one
mesh resident on the GPU and offers the same call shapes on numpy arrays:

    shell = GpuShell(mesh, workload)
    R = shell.form_function(x)                 # FormFunctionFEM
    R, K = shell.form_jacobian(x)              # new: K = dR/dx, 3x3-block CSR

Errors come back as PETSc error numbers (``BiofemError.code``), as the
reference's PetscCheck/SETERRQ would return them.  There is no CPU fallback:
without the compiled library (or a GPU for the compute calls) every call
raises.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parents[1]
LIB_PATH = PKG / "lib" / "libbiofem_gpu.so"

BIOFEM_BASIS_REFERENCE = 0
BIOFEM_BASIS_EXACT = 1
BIOFEM_PC_AMG = 0
BIOFEM_PC_BJACOBI = 1
BIOFEM_FP64 = 0
BIOFEM_FP32_BULK = 1
BIOFEM_BLOCK_ROW_MAJOR = 0
BIOFEM_BLOCK_COL_MAJOR = 1
BIOFEM_CKPT_VERTEX_ORDER = 0
BIOFEM_CKPT_VEC = 1

_i32p = ctypes.POINTER(ctypes.c_int32)
_f64p = ctypes.POINTER(ctypes.c_double)


class BiofemError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"biofem error {code}: {msg}")
        self.code = code


class MeshDesc(ctypes.Structure):
    _fields_ = [("n_v", ctypes.c_int32), ("n_elmt", ctypes.c_int32), ("n_edge", ctypes.c_int32),
                ("tri", _i32p), ("xyz0", _f64p), ("n_bnodes", _i32p), ("bnodes", _i32p),
                ("n_fib", _f64p), ("gamma_scale", _f64p), ("n_elmt_base", ctypes.c_int32)]


class Params(ctypes.Structure):
    _fields_ = [("n_qp", ctypes.c_int32), ("c33_subitr_nums", ctypes.c_int32), ("mu", ctypes.c_double),
                ("bulk_modulus", ctypes.c_double), ("h0", ctypes.c_double), ("gamma", ctypes.c_double),
                ("pressure", ctypes.c_double), ("clamp_edge", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("basis", ctypes.c_int32), ("thickness_normal", ctypes.c_int32), ("block_layout", ctypes.c_int32),
                ("pressure_kind", ctypes.c_int32), ("activation_kind", ctypes.c_int32)]


class MeshInfo(ctypes.Structure):
    _fields_ = [("n_v", ctypes.c_int32), ("n_ghosts", ctypes.c_int32), ("n_elmt", ctypes.c_int32),
                ("n_dof", ctypes.c_int32), ("n_irregular", ctypes.c_int32), ("nnzb", ctypes.c_int64),
                ("n_contrib", ctypes.c_int64), ("device_bytes", ctypes.c_int64), ("precision", ctypes.c_int32)]


class NewtonOptions(ctypes.Structure):
    _fields_ = [("rtol", ctypes.c_double), ("atol", ctypes.c_double), ("max_newton", ctypes.c_int32),
                ("gmres_restart", ctypes.c_int32), ("gmres_max_it", ctypes.c_int32), ("gmres_rtol", ctypes.c_double),
                ("line_search", ctypes.c_int32), ("preconditioner", ctypes.c_int32), ("forcing", ctypes.c_int32)]


class DynParams(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_double), ("rho", ctypes.c_double), ("newmark_gamma", ctypes.c_double),
                ("dampfactor", ctypes.c_double), ("timeinteg", ctypes.c_int32), ("damping", ctypes.c_int32)]


class SurfaceFields(ctypes.Structure):
    _fields_ = [("n_v", ctypes.c_int32), ("n_elmt", ctypes.c_int32), ("tri", ctypes.c_void_p),
                ("x", ctypes.c_void_p), ("X", ctypes.c_void_p), ("mass", ctypes.c_void_p),
                ("Fint", ctypes.c_void_p), ("Fext", ctypes.c_void_p), ("Fdyn", ctypes.c_void_p),
                ("xd", ctypes.c_void_p), ("dA0", ctypes.c_void_p), ("gamma_e", ctypes.c_void_p),
                ("fib", ctypes.c_void_p)]


class NewtonStats(ctypes.Structure):
    _fields_ = [("newton_its", ctypes.c_int32), ("gmres_its_total", ctypes.c_int32), ("gmres_its_last", ctypes.c_int32),
                ("residual_evals", ctypes.c_int32), ("jacobian_evals", ctypes.c_int32), ("converged", ctypes.c_int32),
                ("r0", ctypes.c_double), ("rfinal", ctypes.c_double), ("gmres_relres_last", ctypes.c_double),
                ("rhist", ctypes.c_double * 64)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "rhist"}
        d["rhist"] = list(self.rhist[: self.newton_its + 1])
        return d


_LIB = None

# every entry point the header declares (checked by tests/test_cabi.py)
EXPORTS = ["InitGpuWorkspace", "DestroyGpuWorkspace", "PrepareGpuMesh", "DestroyGpuMesh", "GetGpuMeshInfo",
           "GetGpuTopology", "GetGpuCsrPattern", "RunGpuResidual", "RunGpuResidualJacobian",
           "RunGpuResidualDevice", "RunGpuResidualJacobianDevice", "BiofemGpuSync", "FormFunctionFEMGpu",
           "FormJacobianFEMGpu", "GetGpuLaunchCounts", "BuildHostMesh", "DestroyHostMesh",
           "GetGpuBasisTables", "BiofemGpuLastError", "EnableGpuKernelTiming", "GetGpuKernelTimes",
           "GetGpuGhostMap", "RunGpuResidualNoAlloc", "BiofemNewtonDefaults", "RunGpuNewtonSolve",
           "RunGpuNewtonSolveDevice", "PrepareGpuMeshOnStream", "ServeCreate", "ServeSubmit", "ServeWait",
           "ServeStatsGet", "ServeDestroy", "BiofemServeEstimateBytes", "GetGpuBasisTablesKind",
           "SetGpuDynamics", "SetGpuDynamicState", "GetGpuDynamicState", "RunGpuDynamicUpdate",
           "SetGpuElementGamma", "RunGpuResidualParts", "RunGpuElementThickness", "BiofemLocationOut",
           "BiofemLocationIn", "BiofemWriteSurfaceVTK", "BiofemWriteShell3dVTK"]


def load_library(path: Path | str | None = None) -> ctypes.CDLL:
    """Load libbiofem_gpu.so (built by __graft_entry__.build() /
    biofem-ia_gb300/csrc/build.py).  Raises if it is missing."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(f"{p} is not built; run biofem-ia_gb300/csrc/build.py")
    lib = ctypes.CDLL(str(p))
    vp = ctypes.c_void_p
    lib.BiofemGpuLastError.restype = ctypes.c_char_p
    lib.PrepareGpuMesh.argtypes = [ctypes.POINTER(MeshDesc), ctypes.POINTER(Params), ctypes.POINTER(vp)]
    lib.BuildHostMesh.argtypes = [ctypes.POINTER(MeshDesc), ctypes.POINTER(Params), ctypes.POINTER(vp)]
    lib.PrepareGpuMeshOnStream.argtypes = [ctypes.POINTER(MeshDesc), ctypes.POINTER(Params), vp, ctypes.POINTER(vp)]
    for name in ("DestroyGpuMesh", "DestroyHostMesh"):
        getattr(lib, name).argtypes = [vp]
    lib.GetGpuMeshInfo.argtypes = [vp, ctypes.POINTER(MeshInfo)]
    lib.GetGpuTopology.argtypes = [vp] + [vp] * 7
    lib.GetGpuCsrPattern.argtypes = [vp, vp, vp]
    lib.GetGpuGhostMap.argtypes = [vp, vp]
    lib.RunGpuResidual.argtypes = [vp, vp, vp]
    lib.RunGpuResidualJacobian.argtypes = [vp, vp, vp, vp]
    lib.RunGpuResidualDevice.argtypes = [vp, vp, vp, vp]
    lib.RunGpuResidualJacobianDevice.argtypes = [vp, vp, vp, vp, vp]
    lib.RunGpuResidualNoAlloc.argtypes = [vp, vp, vp, vp]
    lib.BiofemNewtonDefaults.argtypes = [ctypes.POINTER(NewtonOptions)]
    lib.BiofemNewtonDefaults.restype = None
    lib.RunGpuNewtonSolve.argtypes = [vp, vp, ctypes.POINTER(NewtonOptions), ctypes.POINTER(NewtonStats)]
    lib.RunGpuNewtonSolveDevice.argtypes = [vp, vp, ctypes.POINTER(NewtonOptions), ctypes.POINTER(NewtonStats), vp]
    lib.BiofemGpuSync.argtypes = [vp, vp]
    lib.GetGpuLaunchCounts.argtypes = [vp, vp, vp]
    lib.GetGpuBasisTables.argtypes = [vp]
    lib.EnableGpuKernelTiming.argtypes = [vp, ctypes.c_int]
    lib.GetGpuKernelTimes.argtypes = [vp, vp, ctypes.c_int32, vp]
    lib.GetGpuBasisTablesKind.argtypes = [ctypes.c_int32, vp]
    lib.SetGpuDynamics.argtypes = [vp, ctypes.POINTER(DynParams)]
    lib.SetGpuDynamicState.argtypes = [vp, vp, vp, vp, vp]
    lib.GetGpuDynamicState.argtypes = [vp, vp, vp, vp, vp]
    lib.RunGpuDynamicUpdate.argtypes = [vp, vp]
    lib.SetGpuElementGamma.argtypes = [vp, vp]
    lib.RunGpuResidualParts.argtypes = [vp, vp, vp, vp, vp, vp]
    lib.RunGpuElementThickness.argtypes = [vp, vp, vp]
    i32, i64, cp = ctypes.c_int32, ctypes.c_int64, ctypes.c_char_p
    lib.BiofemLocationOut.argtypes = [cp, i32, i32, i64, vp, vp, vp, vp, i32]
    lib.BiofemLocationIn.argtypes = [cp, i32, i32, i64, vp, vp, vp, vp]
    lib.BiofemWriteSurfaceVTK.argtypes = [cp, i32, i32, ctypes.POINTER(SurfaceFields)]
    lib.BiofemWriteShell3dVTK.argtypes = [cp, i32, i32, i32, i32, vp, vp, vp]
    lib.ServeCreate.argtypes = [ctypes.c_int64, ctypes.c_int32, ctypes.POINTER(vp)]
    lib.ServeSubmit.argtypes = [vp, ctypes.POINTER(MeshDesc), ctypes.POINTER(Params), ctypes.POINTER(NewtonOptions),
                                vp, ctypes.POINTER(ctypes.c_int64)]
    lib.ServeWait.argtypes = [vp, ctypes.c_int64, vp, ctypes.POINTER(NewtonStats), vp]
    lib.ServeStatsGet.argtypes = [vp, vp]
    lib.ServeDestroy.argtypes = [vp]
    lib.BiofemServeEstimateBytes.argtypes = [ctypes.c_int32] * 5 + [ctypes.POINTER(ctypes.c_int64)]
    if path is None:
        _LIB = lib
    return lib


def _check(lib, rc: int):
    if rc:
        raise BiofemError(rc, lib.BiofemGpuLastError().decode())


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def basis_tables() -> np.ndarray:
    """(11, 5, 16) centroid basis-derivative tables the kernels use."""
    lib = load_library()
    out = np.zeros(11 * 80)
    _check(lib, lib.GetGpuBasisTables(_ptr(out)))
    return out.reshape(11, 5, 16)


class GpuShell:
    """One mesh resident on the GPU (or, with host_only=True, only its host tables)."""

    def __init__(self, mesh, workload, mu: float, bulk: float, h0: float, gamma: float = 1.0,
                 clamp_edge: int | None = None, precision: int = BIOFEM_FP64, host_only: bool = False,
                 block_layout: int = BIOFEM_BLOCK_ROW_MAJOR):
        """clamp_edge: the boundary ring clamped in x, y, z; by default ring 0,
        or none (-1) when the mesh has no boundary ring (a closed surface) or
        the workload asks for none (``workload.clamp`` False)."""
        if clamp_edge is None:
            clamp_edge = 0 if mesh.n_edge > 0 and getattr(workload, "clamp", True) else -1
        self.lib = load_library()
        self._arrays = dict(
            tri=np.ascontiguousarray(mesh.tri, dtype=np.int32),
            xyz0=np.ascontiguousarray(mesh.xyz0, dtype=np.float64),
            nb=np.ascontiguousarray(mesh.n_bnodes, dtype=np.int32),
            bn=np.ascontiguousarray(mesh.bnodes, dtype=np.int32),
            fib=np.ascontiguousarray(mesh.fib, dtype=np.float64),
            gs=np.ascontiguousarray(mesh.gamma_scale, dtype=np.float64))
        a = self._arrays
        self.desc = MeshDesc(mesh.n_v, mesh.n_elmt, mesh.n_edge,
                             a["tri"].ctypes.data_as(_i32p), a["xyz0"].ctypes.data_as(_f64p),
                             a["nb"].ctypes.data_as(_i32p), a["bn"].ctypes.data_as(_i32p),
                             a["fib"].ctypes.data_as(_f64p), a["gs"].ctypes.data_as(_f64p),
                             int(getattr(mesh, "n_elmt_base", 0)))
        self.params = Params(workload.n_qp, workload.c33_iters, mu, bulk, h0, gamma, workload.pressure,
                             clamp_edge, precision, getattr(workload, "basis", BIOFEM_BASIS_REFERENCE),
                             getattr(workload, "tnormal", 0), block_layout, getattr(workload, "dead_load", 0),
                             getattr(workload, "iso_act", 0))
        self.host_only = host_only
        h = ctypes.c_void_p()
        fn = self.lib.BuildHostMesh if host_only else self.lib.PrepareGpuMesh
        _check(self.lib, fn(ctypes.byref(self.desc), ctypes.byref(self.params), ctypes.byref(h)))
        self.handle = h
        info = MeshInfo()
        _check(self.lib, self.lib.GetGpuMeshInfo(self.handle, ctypes.byref(info)))
        self.info = info
        self.n_dof = info.n_dof
        self.nnzb = info.nnzb
        self.precision = precision
        self.k_dtype = np.float64 if precision == BIOFEM_FP64 else np.float32

    def close(self):
        if self.handle:
            (self.lib.DestroyHostMesh if self.host_only else self.lib.DestroyGpuMesh)(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- tables ----
    def topology(self) -> dict:
        i = self.info
        ne, ng, nv = i.n_elmt, i.n_ghosts, i.n_v
        t = dict(patch=np.zeros((ne, 16), np.int32), ire=np.zeros(ne, np.int32), val=np.zeros(ne, np.int32),
                 irv=np.zeros(ne, np.int32), gtri=np.zeros((ne + 2 * ng, 3), np.int32),
                 xyz0_full=np.zeros((nv + ng, 3)), dA0=np.zeros(ne))
        _check(self.lib, self.lib.GetGpuTopology(self.handle, *(_ptr(t[k]) for k in
                                                                ("patch", "ire", "val", "irv", "gtri", "xyz0_full", "dA0"))))
        g3 = np.zeros((ng, 3), np.int32)
        _check(self.lib, self.lib.GetGpuGhostMap(self.handle, _ptr(g3)))
        t["ghost3"] = g3
        t["ghost_nv3"] = g3[:, 2].copy()
        return t

    def pattern(self):
        rowptr = np.zeros(self.info.n_v + self.info.n_ghosts + 1, np.int32)
        colind = np.zeros(self.nnzb, np.int32)
        _check(self.lib, self.lib.GetGpuCsrPattern(self.handle, _ptr(rowptr), _ptr(colind)))
        return rowptr, colind

    def launch_counts(self):
        r, j = ctypes.c_int32(), ctypes.c_int32()
        _check(self.lib, self.lib.GetGpuLaunchCounts(self.handle, ctypes.byref(r), ctypes.byref(j)))
        return r.value, j.value

    # ---- FormFunctionFEM / Jacobian on host arrays ----
    def form_function(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        if x.size != self.n_dof:
            raise BiofemError(63, f"x has {x.size} entries, expected {self.n_dof}")
        R = np.empty(self.n_dof)
        _check(self.lib, self.lib.RunGpuResidual(self.handle, _ptr(x), _ptr(R)))
        return R

    def form_jacobian(self, x: np.ndarray):
        x = np.ascontiguousarray(x, dtype=np.float64)
        if x.size != self.n_dof:
            raise BiofemError(63, f"x has {x.size} entries, expected {self.n_dof}")
        R = np.empty(self.n_dof)
        K = np.empty((self.nnzb, 3, 3), dtype=self.k_dtype)
        _check(self.lib, self.lib.RunGpuResidualJacobian(self.handle, _ptr(x), _ptr(R), _ptr(K)))
        return R, K

    # ---- one load step ----
    def newton_options(self, **kw) -> NewtonOptions:
        o = NewtonOptions()
        self.lib.BiofemNewtonDefaults(ctypes.byref(o))
        names = {f[0] for f in NewtonOptions._fields_}
        for k, v in kw.items():
            if k not in names:
                raise TypeError(f"unknown Newton option {k!r} (fields: {sorted(names)})")
            setattr(o, k, v)
        return o

    def newton(self, x: np.ndarray, **kw):
        """RunGpuNewtonSolve: Newton + preconditioned GMRES load step from x.
        Returns (x_converged, stats dict); a failure raises BiofemError with
        the statistics gathered so far in its ``stats`` attribute."""
        x = np.array(x, dtype=np.float64, copy=True)
        o = self.newton_options(**kw)
        st = NewtonStats()
        rc = self.lib.RunGpuNewtonSolve(self.handle, _ptr(x), ctypes.byref(o), ctypes.byref(st))
        if rc:
            err = BiofemError(rc, self.lib.BiofemGpuLastError().decode())
            err.stats = st.as_dict()
            raise err
        return x, st.as_dict()

    def newton_device(self, d_x: int, stream: int = 0, **kw):
        o = self.newton_options(**kw)
        st = NewtonStats()
        _check(self.lib, self.lib.RunGpuNewtonSolveDevice(self.handle, ctypes.c_void_p(d_x), ctypes.byref(o),
                                                          ctypes.byref(st), ctypes.c_void_p(stream or None)))
        return st.as_dict()

    # ---- dynamics (FDynamic / xAccVel) and time-dependent activation ----
    def set_dynamics(self, dt=None, rho=0.0, newmark_gamma=0.5, dampfactor=0.0, timeinteg=0, damping=0):
        """SetGpuDynamics; dt=None switches the dynamic term off."""
        if dt is None:
            _check(self.lib, self.lib.SetGpuDynamics(self.handle, None))
            return
        d = DynParams(dt, rho, newmark_gamma, dampfactor, timeinteg, damping)
        _check(self.lib, self.lib.SetGpuDynamics(self.handle, ctypes.byref(d)))

    def set_dynamic_state(self, xn=None, xnm1=None, xd=None, xdd=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (xn, xnm1, xd, xdd)]
        _check(self.lib, self.lib.SetGpuDynamicState(self.handle, *[None if a is None else _ptr(a) for a in arrs]))

    def dynamic_state(self):
        out = [np.empty(self.n_dof) for _ in range(4)]
        _check(self.lib, self.lib.GetGpuDynamicState(self.handle, *[_ptr(a) for a in out]))
        return dict(zip(("xn", "xnm1", "xd", "xdd"), out))

    def dynamic_update(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        _check(self.lib, self.lib.RunGpuDynamicUpdate(self.handle, _ptr(x)))

    def set_element_gamma(self, gamma_e):
        g = np.ascontiguousarray(gamma_e, dtype=np.float64)
        assert g.size == self.info.n_elmt
        _check(self.lib, self.lib.SetGpuElementGamma(self.handle, _ptr(g)))

    # ---- output quantities ----
    def residual_parts(self, x):
        """RunGpuResidualParts: (R, Fint, Fext, Fdyn), the forces unscaled."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = [np.empty(self.n_dof) for _ in range(4)]
        _check(self.lib, self.lib.RunGpuResidualParts(self.handle, _ptr(x), *[_ptr(a) for a in out]))
        return tuple(out)

    def element_thickness(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        th = np.empty(self.info.n_elmt)
        _check(self.lib, self.lib.RunGpuElementThickness(self.handle, _ptr(x), _ptr(th)))
        return th

    # ---- device-resident calls (raw CUDA pointers as ints) ----
    def residual_device(self, d_x: int, d_R: int, stream: int = 0):
        """stream: a cudaStream_t handle as int (0 = the CUDA default stream)."""
        _check(self.lib, self.lib.RunGpuResidualDevice(self.handle, ctypes.c_void_p(d_x), ctypes.c_void_p(d_R),
                                                       ctypes.c_void_p(stream or None)))

    def jacobian_device(self, d_x: int, d_R: int, d_K: int, stream: int = 0):
        _check(self.lib, self.lib.RunGpuResidualJacobianDevice(self.handle, ctypes.c_void_p(d_x), ctypes.c_void_p(d_R),
                                                               ctypes.c_void_p(d_K), ctypes.c_void_p(stream or None)))

    def residual_device_noalloc(self, d_x: int, d_R: int, stream: int = 0):
        """RunGpuResidualNoAlloc: same residual, work arrays in the library's
        fixed device array (no allocation; meshes up to ~19k triangles)."""
        _check(self.lib, self.lib.RunGpuResidualNoAlloc(self.handle, ctypes.c_void_p(d_x), ctypes.c_void_p(d_R),
                                                        ctypes.c_void_p(stream or None)))

    def sync(self, stream: int = 0):
        _check(self.lib, self.lib.BiofemGpuSync(self.handle, ctypes.c_void_p(stream or None)))

    def kernel_timing(self, on: bool):
        _check(self.lib, self.lib.EnableGpuKernelTiming(self.handle, int(on)))

    def kernel_times(self, nslots: int = 5):
        ms = np.zeros(nslots)
        calls = ctypes.c_int32()
        _check(self.lib, self.lib.GetGpuKernelTimes(self.handle, _ptr(ms), nslots, ctypes.byref(calls)))
        return ms, calls.value

    def residual_jacobian_host_ptrs(self, x_ptr: int, R_ptr: int, K_ptr: int):
        """RunGpuResidualJacobian on caller-owned (e.g. pinned) host buffers."""
        _check(self.lib, self.lib.RunGpuResidualJacobian(self.handle, ctypes.c_void_p(x_ptr), ctypes.c_void_p(R_ptr),
                                                         ctypes.c_void_p(K_ptr)))

    def residual_host_ptrs(self, x_ptr: int, R_ptr: int):
        _check(self.lib, self.lib.RunGpuResidual(self.handle, ctypes.c_void_p(x_ptr), ctypes.c_void_p(R_ptr)))

    # ---- helpers ----
    def to_scipy(self, K: np.ndarray):
        import scipy.sparse as sp
        rowptr, colind = self.pattern()
        nb = self.info.n_v + self.info.n_ghosts
        return sp.bsr_matrix((K.reshape(-1, 3, 3).astype(np.float64), colind, rowptr), shape=(3 * nb, 3 * nb))


def FormFunctionFEM(snes, x: np.ndarray, R: np.ndarray, ctx: GpuShell) -> int:
    """SNES residual callback shape (main.c:120,757): fills R in place, returns 0."""
    R[:] = ctx.form_function(x)
    return 0


def FormJacobianFEM(snes, x: np.ndarray, J: np.ndarray, P, ctx: GpuShell) -> int:
    """SNES Jacobian callback shape (SNESSetJacobian slot, main.c:462-466):
    fills the (nnzb, 3, 3) block values J in place, returns 0."""
    _, K = ctx.form_jacobian(x)
    J[...] = K
    return 0


def mesh_desc(mesh):
    """(MeshDesc, arrays to keep alive) for a biofem.mesh.Mesh."""
    a = dict(tri=np.ascontiguousarray(mesh.tri, dtype=np.int32), xyz0=np.ascontiguousarray(mesh.xyz0, dtype=np.float64),
             nb=np.ascontiguousarray(mesh.n_bnodes, dtype=np.int32), bn=np.ascontiguousarray(mesh.bnodes, dtype=np.int32),
             fib=np.ascontiguousarray(mesh.fib, dtype=np.float64),
             gs=np.ascontiguousarray(mesh.gamma_scale, dtype=np.float64))
    d = MeshDesc(mesh.n_v, mesh.n_elmt, mesh.n_edge, a["tri"].ctypes.data_as(_i32p), a["xyz0"].ctypes.data_as(_f64p),
                 a["nb"].ctypes.data_as(_i32p), a["bn"].ctypes.data_as(_i32p), a["fib"].ctypes.data_as(_f64p),
                 a["gs"].ctypes.data_as(_f64p), int(getattr(mesh, "n_elmt_base", 0)))
    return d, a


class Serve:
    """ServeCreate / ServeSubmit / ServeWait: the continuous-batching load-step service."""

    def __init__(self, hbm_budget_bytes: int, max_slots: int):
        self.lib = load_library()
        h = ctypes.c_void_p()
        _check(self.lib, self.lib.ServeCreate(int(hbm_budget_bytes), int(max_slots), ctypes.byref(h)))
        self.handle = h
        self._ndof = {}

    def submit(self, mesh, workload, mu, bulk, h0, x0, gamma=1.0, clamp_edge=0, precision=BIOFEM_FP64, **newton):
        d, keep = mesh_desc(mesh)
        prm = Params(workload.n_qp, workload.c33_iters, mu, bulk, h0, gamma, workload.pressure, clamp_edge, precision,
                     getattr(workload, "basis", BIOFEM_BASIS_REFERENCE), getattr(workload, "tnormal", 0), 0,
                     getattr(workload, "dead_load", 0), getattr(workload, "iso_act", 0))
        o = NewtonOptions()
        self.lib.BiofemNewtonDefaults(ctypes.byref(o))
        for k, v in newton.items():
            setattr(o, k, v)
        x0 = np.ascontiguousarray(x0, dtype=np.float64)
        t = ctypes.c_int64()
        _check(self.lib, self.lib.ServeSubmit(self.handle, ctypes.byref(d), ctypes.byref(prm), ctypes.byref(o),
                                              _ptr(x0), ctypes.byref(t)))
        self._ndof[t.value] = x0.size
        return t.value

    def wait(self, ticket: int):
        x = np.empty(self._ndof.pop(ticket))
        st = NewtonStats()
        times = np.zeros(3)
        _check(self.lib, self.lib.ServeWait(self.handle, ctypes.c_int64(ticket), _ptr(x), ctypes.byref(st), _ptr(times)))
        return x, st.as_dict(), times

    def stats(self):
        out = np.zeros(6, np.int64)
        _check(self.lib, self.lib.ServeStatsGet(self.handle, _ptr(out)))
        return dict(zip(["in_use", "peak_in_use", "active", "peak_active", "queued", "completed"], out.tolist()))

    def close(self):
        if self.handle:
            self.lib.ServeDestroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def estimate_bytes(n_v, n_elmt, n_ghosts, precision=BIOFEM_FP64, gmres_restart=0) -> int:
    lib = load_library()
    b = ctypes.c_int64()
    _check(lib, lib.BiofemServeEstimateBytes(n_v, n_elmt, n_ghosts, precision, gmres_restart, ctypes.byref(b)))
    return b.value
