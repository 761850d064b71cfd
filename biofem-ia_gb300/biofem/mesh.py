"""Synthetic membrane meshes in BioFEM-IA's IBMNodes layout.

A mesh here is the set of arrays the reference's ``Input()`` fills from the
``nlist/elist/blist`` files (io.c:373-479), 0-based:

* ``xyz0``   (n_v, 3) float64 reference coordinates of the real nodes;
* ``tri``    (n_elmt, 3) int32 triangle corners (nv1, nv2, nv3);
* ``n_bnodes`` / ``bnodes``: boundary rings.  Every ring is a CLOSED loop, one
  ghost node per ring node (``GlobalGhostInit``, bending.c:1670-1757);
* ``fib`` (n_elmt, 3) fibre directions (``ibm->n_fib``) and ``gamma_scale``
  (n_elmt,) so that gamma * gamma_scale = 1 - lambda_a (active_strain.c:1212).

The flat rectangle uses row-alternating cell diagonals: row j of cells uses
the "/" diagonal when j is even and the "\\" diagonal when j is odd.  Interior
nodes then all have valence 6; nodes on the left and right sides have 2 or 4
triangles (boundary valence 5 or 7 after IrrVer's +3 rule, bending.c:1229-1248)
and the four corners 1 or 2 (valence 4 or 5), so those patches take the
reference's irregular (one-step subdivision) branch.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

SEED_BASE = 20261203


@dataclass
class Mesh:
    xyz0: np.ndarray
    tri: np.ndarray
    n_bnodes: np.ndarray
    bnodes: np.ndarray
    fib: np.ndarray
    gamma_scale: np.ndarray
    meta: dict = field(default_factory=dict)

    @property
    def n_v(self) -> int:
        return int(self.xyz0.shape[0])

    @property
    def n_elmt(self) -> int:
        return int(self.tri.shape[0])

    @property
    def n_edge(self) -> int:
        return int(self.n_bnodes.shape[0])

    @property
    def n_ghosts(self) -> int:
        return int(self.n_bnodes.sum())

    @property
    def n_dof(self) -> int:
        return 3 * (self.n_v + self.n_ghosts)


def flat_membrane(nx: int, ny: int, lx: float = 1.0, ly: float = 0.75,
                  z_sigma: float = 0.0, seed: int | None = None, z_smooth: bool = False) -> Mesh:
    """Structured nx-by-ny-cell rectangle, 2 triangles per cell, CCW triangles.

    Node (i, j) has index j*(nx+1)+i.  Cells are ordered row-major and each
    cell emits its two triangles in order.  The single boundary ring runs
    counter-clockwise from node 0.  ``z_sigma`` > 0 adds seeded N(0, z_sigma)
    to the z coordinate of every real node; with ``z_smooth`` the
    perturbation is instead a seeded combination of the 9 lowest sine modes
    sin(k pi x/lx) sin(l pi y/ly), k, l = 1..3, scaled to peak z_sigma.  A
    mesh-independent imperfection keeps the reference surface's curvature
    bounded: per-node noise of fixed size gives curvatures ~ z_sigma / h^2,
    which for h below ~5e-3 exceed 2/h0 and fold the shell's outer
    thickness points.
    """
    if nx < 2 or ny < 2:
        raise ValueError("flat_membrane needs at least 2x2 cells")
    xs = np.linspace(0.0, lx, nx + 1)
    ys = np.linspace(0.0, ly, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    xyz0 = np.zeros(((nx + 1) * (ny + 1), 3))
    xyz0[:, 0] = X.ravel()
    xyz0[:, 1] = Y.ravel()
    if z_sigma > 0.0:
        rng = np.random.Generator(np.random.PCG64(SEED_BASE if seed is None else seed))
        if z_smooth:
            coef = rng.standard_normal((3, 3))
            z = np.zeros(xyz0.shape[0])
            for k in range(3):
                for l in range(3):
                    z += coef[k, l] * np.sin((k + 1) * np.pi * xyz0[:, 0] / lx) * np.sin((l + 1) * np.pi * xyz0[:, 1] / ly)
            xyz0[:, 2] = z_sigma * z / max(np.abs(z).max(), 1e-300)
        else:
            xyz0[:, 2] = rng.normal(0.0, z_sigma, size=xyz0.shape[0])

    i = np.arange(nx)
    j = np.arange(ny)
    I, J = np.meshgrid(i, j, indexing="xy")
    n00 = (J * (nx + 1) + I).ravel()
    n10 = n00 + 1
    n01 = n00 + (nx + 1)
    n11 = n01 + 1
    slash = ((J % 2) == 0).ravel()
    t1 = np.where(slash[:, None], np.stack([n00, n10, n11], 1), np.stack([n00, n10, n01], 1))
    t2 = np.where(slash[:, None], np.stack([n00, n11, n01], 1), np.stack([n10, n11, n01], 1))
    tri = np.empty((2 * nx * ny, 3), dtype=np.int32)
    tri[0::2] = t1
    tri[1::2] = t2

    bottom = [jj * 0 + ii for ii in range(0, nx + 1) for jj in (0,)]
    right = [jj * (nx + 1) + nx for jj in range(1, ny + 1)]
    top = [ny * (nx + 1) + ii for ii in range(nx - 1, -1, -1)]
    left = [jj * (nx + 1) for jj in range(ny - 1, 0, -1)]
    ring = np.array(bottom + right + top + left, dtype=np.int32)

    n_e = tri.shape[0]
    fib = np.zeros((n_e, 3))
    fib[:, 0] = 1.0
    return Mesh(xyz0=xyz0, tri=tri, n_bnodes=np.array([ring.size], dtype=np.int32),
                bnodes=ring, fib=fib, gamma_scale=np.zeros(n_e),
                meta=dict(kind="flat", nx=nx, ny=ny, lx=lx, ly=ly, z_sigma=z_sigma, seed=seed, z_smooth=z_smooth))


def element_centroids(mesh: Mesh) -> np.ndarray:
    return mesh.xyz0[mesh.tri].mean(axis=1)


def set_uniform_activation(mesh: Mesh, lambda_a: float, fiber=(1.0, 0.0, 0.0)) -> Mesh:
    mesh.fib[:] = np.asarray(fiber, dtype=float)
    mesh.gamma_scale[:] = 1.0 - lambda_a
    return mesh


def set_smooth_activation(mesh: Mesh) -> Mesh:
    """lambda_a = 0.85 + 0.1 sin(2 pi x_c) cos(2 pi y_c) at the reference centroid, fibre e_x."""
    c = element_centroids(mesh)
    lam = 0.85 + 0.1 * np.sin(2 * np.pi * c[:, 0]) * np.cos(2 * np.pi * c[:, 1])
    mesh.fib[:] = (1.0, 0.0, 0.0)
    mesh.gamma_scale[:] = 1.0 - lam
    return mesh


def set_random_activation(mesh: Mesh, seed: int, lam_lo=0.85, lam_hi=1.0) -> Mesh:
    """Per-element fibre angle U[0, pi) in the xy plane, lambda_a U[lam_lo, lam_hi]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    th = rng.uniform(0.0, np.pi, size=mesh.n_elmt)
    lam = rng.uniform(lam_lo, lam_hi, size=mesh.n_elmt)
    mesh.fib[:, 0] = np.cos(th)
    mesh.fib[:, 1] = np.sin(th)
    mesh.fib[:, 2] = 0.0
    mesh.gamma_scale[:] = 1.0 - lam
    return mesh


def initial_state(mesh: Mesh, xyz0_full: np.ndarray, disp_amp: float = 0.0,
                  seed: int | None = None) -> np.ndarray:
    """SNES iterate x (3*(n_v+n_ghosts)): reference positions, plus a seeded
    U(-disp_amp, disp_amp)^3 displacement of every real node.  Ghost entries
    are carried along unchanged (the residual recomputes them)."""
    x = np.array(xyz0_full, dtype=float).reshape(-1).copy()
    if disp_amp > 0.0:
        rng = np.random.Generator(np.random.PCG64(SEED_BASE + 7 if seed is None else seed))
        d = rng.uniform(-disp_amp, disp_amp, size=(mesh.n_v, 3))
        x[: 3 * mesh.n_v] += d.reshape(-1)
    return x


# ---- reference file formats (bin/biofem:551-575, read by io.c:33-79,373-479) ----
def write_input_files(mesh: Mesh, in_dir: str | Path, ibi: int = 0) -> None:
    """nlist/elist/blist in the layout Input() reads (1-based ids)."""
    d = Path(in_dir)
    d.mkdir(parents=True, exist_ok=True)
    with open(d / f"nlist{ibi:02d}", "w") as f:
        f.write(f"{mesh.n_v}\n")
        for k, (x, y, z) in enumerate(mesh.xyz0, start=1):
            f.write(f"{k}\t0\t0\t{x:.17e} {y:.17e} {z:.17e}\n")
    with open(d / f"elist{ibi:02d}", "w") as f:
        f.write(f"{mesh.n_elmt}\n")
        for e, (a, b, c) in enumerate(mesh.tri, start=1):
            f.write(f"1\t1\t0\t0\t0\t0\t0\t0\t4\t0\t{e}\t{a+1}\t{b+1}\t{c+1}\t{c+1}\n")
    with open(d / f"blist{ibi:02d}", "w") as f:
        f.write(f"{mesh.n_edge}\n{mesh.n_ghosts}\n")
        for n in mesh.n_bnodes:
            f.write(f"{int(n)}\n")
        f.write(" ".join(str(int(b) + 1) for b in mesh.bnodes) + "\n")


def read_input_files(in_dir: str | Path, ibi: int = 0) -> Mesh:
    """Inverse of write_input_files (also reads files written by bin/biofem)."""
    d = Path(in_dir)
    with open(d / f"nlist{ibi:02d}") as f:
        n_v = int(f.readline())
        xyz0 = np.array([[float(t) for t in f.readline().split()[3:6]] for _ in range(n_v)])
    with open(d / f"elist{ibi:02d}") as f:
        n_e = int(f.readline())
        tri = np.array([[int(t) - 1 for t in f.readline().split()[11:14]] for _ in range(n_e)], dtype=np.int32)
    with open(d / f"blist{ibi:02d}") as f:
        toks = f.read().split()
    n_edge = int(toks[0])
    n_bnodes = np.array([int(t) for t in toks[2:2 + n_edge]], dtype=np.int32)
    bnodes = np.array([int(t) - 1 for t in toks[2 + n_edge:2 + n_edge + int(n_bnodes.sum())]], dtype=np.int32)
    fib = np.zeros((n_e, 3))
    fib[:, 0] = 1.0
    return Mesh(xyz0=xyz0, tri=tri, n_bnodes=n_bnodes, bnodes=bnodes, fib=fib,
                gamma_scale=np.zeros(n_e), meta=dict(kind="file", path=str(d)))
