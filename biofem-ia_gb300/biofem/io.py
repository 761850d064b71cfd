"""Checkpoints and VTK output of a time-stepped shell (formats.cpp through the C-ABI).

* ``location_out`` / ``location_in``: the LocationOut / LocationIn checkpoint
  files (io.c:1272-1376, 1513-1640): x, xn, xd, xdd, big-endian PETSc binary,
  original-vertex order.
* ``checkpoint`` / ``restart``: the same from and into a GpuShell's dynamic
  state.  A restart leaves xnm1 at the reference coordinates, as the
  reference does (Init sets it, LocationIn does not store it).
* ``StepWriter``: Output (io.c:540-964) every ``tiout`` steps, file ti + 1 for
  step ti (main.c:601-608), optionally with the 3-D shell file of
  Write3DShellVTK (io.c:983-1064); its hooks plug into dynamics.time_loop.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .gpu import BIOFEM_CKPT_VERTEX_ORDER, SurfaceFields, _check, _ptr, load_library

TAGS = ("x", "xn", "xd", "xdd")


def _lib(lib=None):
    return lib if lib is not None else load_library()


def location_out(out_dir, ti: int, x, xn, xd, xdd, ibi: int = 0, layout: int = BIOFEM_CKPT_VERTEX_ORDER, lib=None):
    lib = _lib(lib)
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, xn, xd, xdd)]
    n = arrs[0].size
    if any(a.size != n for a in arrs):
        raise ValueError("checkpoint vectors differ in length")
    _check(lib, lib.BiofemLocationOut(os.fsencode(str(out_dir)), ti, ibi, n, *[_ptr(a) for a in arrs], layout))


def location_in(out_dir, ti: int, n_dof: int, ibi: int = 0, lib=None) -> dict:
    lib = _lib(lib)
    out = [np.empty(n_dof) for _ in TAGS]
    _check(lib, lib.BiofemLocationIn(os.fsencode(str(out_dir)), ti, ibi, n_dof, *[_ptr(a) for a in out]))
    return dict(zip(TAGS, out))


def checkpoint(shell, out_dir, ti: int, x, ibi: int = 0, layout: int = BIOFEM_CKPT_VERTEX_ORDER):
    s = shell.dynamic_state()
    location_out(out_dir, ti, x, s["xn"], s["xd"], s["xdd"], ibi, layout, shell.lib)


def restart(shell, out_dir, ti: int, ibi: int = 0):
    """Load checkpoint ti into the shell's dynamic state (the dynamic term must
    be on); returns x."""
    c = location_in(out_dir, ti, shell.n_dof, ibi, shell.lib)
    shell.set_dynamic_state(xn=c["xn"], xd=c["xd"], xdd=c["xdd"])
    return c["x"]


def init_mass(mesh, dA0, rho: float, h0: float) -> np.ndarray:
    """Lumped nodal mass of Init (main.c:1465-1470): each real triangle adds
    rho dA0 h0 / 3 to its corners, in triangle order."""
    m = np.zeros(mesh.n_v)
    me = 1. / 3. * rho * np.asarray(dA0, dtype=np.float64) * h0
    np.add.at(m, np.asarray(mesh.tri).ravel(), np.repeat(me, 3))
    return m


def write_surface(out_dir, ti: int, mesh, x, X, gamma_e, Fint=None, Fext=None, Fdyn=None, xd=None, mass=None,
                  fib=None, ibi: int = 0, lib=None):
    """BiofemWriteSurfaceVTK; node arrays may be full-length (ghost entries are
    ignored), x and X as well."""
    lib = _lib(lib)
    nv, ne = mesh.n_v, mesh.n_elmt

    def node3(a):
        return None if a is None else np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel()[: 3 * nv])

    keep = dict(tri=np.ascontiguousarray(mesh.tri, dtype=np.int32), x=node3(x), X=node3(X), Fint=node3(Fint),
                Fext=node3(Fext), Fdyn=node3(Fdyn), xd=node3(xd),
                mass=None if mass is None else np.ascontiguousarray(mass, dtype=np.float64),
                gamma_e=np.ascontiguousarray(gamma_e, dtype=np.float64),
                fib=None if fib is None else np.ascontiguousarray(fib, dtype=np.float64))
    if keep["gamma_e"].size != ne:
        raise ValueError("gamma_e needs one value per element")
    f = SurfaceFields(nv, ne, *[None if keep[k] is None else _ptr(keep[k]) for k in
                                ("tri", "x", "X", "mass", "Fint", "Fext", "Fdyn", "xd")],
                      None, _ptr(keep["gamma_e"]), None if keep["fib"] is None else _ptr(keep["fib"]))
    _check(lib, lib.BiofemWriteSurfaceVTK(os.fsencode(str(out_dir)), ti, ibi, ctypes.byref(f)))


def write_shell3d(out_dir, ti: int, mesh, x, thickness_e, ibi: int = 0, lib=None):
    lib = _lib(lib)
    tri = np.ascontiguousarray(mesh.tri, dtype=np.int32)
    xr = np.ascontiguousarray(np.asarray(x, dtype=np.float64).ravel()[: 3 * mesh.n_v])
    th = np.ascontiguousarray(thickness_e, dtype=np.float64)
    _check(lib, lib.BiofemWriteShell3dVTK(os.fsencode(str(out_dir)), ti, ibi, mesh.n_v, mesh.n_elmt, _ptr(tri),
                                          _ptr(xr), _ptr(th)))


class StepWriter:
    """Output of a time loop: pass ``pre_update=w.pre_update, on_step=w.on_step``
    to dynamics.time_loop.  The forces are those of the converged state with the
    step's dynamic state (before xAccVel), the velocity the updated one, as in
    the reference's loop order (main.c:501-608)."""

    def __init__(self, shell, mesh, out_dir, act, dt: float, tisteps: int, rho: float, h0: float, delay=None,
                 tiout: int = 1, shell3d: bool = False, fib: bool = False, ibi: int = 0):
        self.sh, self.mesh, self.dir = shell, mesh, out_dir
        self.act, self.dt, self.tisteps, self.delay = act, dt, tisteps, delay
        self.tiout, self.shell3d, self.ibi = tiout, shell3d, ibi
        topo = shell.topology()
        self.X = topo["xyz0_full"].ravel()
        self.mass = init_mass(mesh, topo["dA0"], rho, h0)
        self.fib = np.asarray(mesh.fib) if fib else None
        self._parts = None
        self.written = []

    def _due(self, ti):
        return ti == (ti // self.tiout) * self.tiout

    def pre_update(self, ti, x):
        self._parts = self.sh.residual_parts(x) if self._due(ti) else None

    def on_step(self, ti, x, rec):
        if not self._due(ti):
            return
        _, Fint, Fext, Fdyn = self._parts
        xd = self.sh.dynamic_state()["xd"]
        g = self.act.element_gamma(ti, self.dt, self.tisteps, self.mesh.gamma_scale, self.delay)
        write_surface(self.dir, ti + 1, self.mesh, x, self.X, g, Fint, Fext, Fdyn, xd, self.mass, self.fib,
                      self.ibi, self.sh.lib)
        if self.shell3d:
            write_shell3d(self.dir, ti + 1, self.mesh, x, self.sh.element_thickness(x), self.ibi, self.sh.lib)
        self.written.append(ti + 1)
