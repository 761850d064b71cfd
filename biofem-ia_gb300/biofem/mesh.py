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
    n_elmt_base: int = 0   # ibm->n_elmt_base: > 0 makes the elements from it on flat apex-cap triangles

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


def cone_disc(valence: int, rings: int, radius: float = 1.0, z_sigma: float = 0.0,
              seed: int | None = None) -> Mesh:
    """A flat disc whose centre vertex has `valence` triangles and every
    other interior vertex six: `valence` sectors of a triangular lattice,
    ring r (1..rings) holding valence * r vertices at radius r / rings, the
    sector k spanning the angles [2 pi k / valence, 2 pi (k + 1) / valence).
    Ring r and r + 1 are joined sector by sector with 2 r + 1 triangles
    (valence * rings^2 triangles in all), counter-clockwise.  The single
    boundary ring is the outer ring, counter-clockwise.  With valence 3..10
    the centre's triangles take the one-step subdivision of that valence,
    up to the 16-node patch of valence 10.  ``z_sigma`` > 0 adds a seeded
    smooth bump a (1 - rho^2) cos(theta - phi) of peak z_sigma."""
    if not 3 <= valence <= 10 or rings < 3:
        raise ValueError("cone_disc needs valence 3..10 and at least 3 rings")
    start = [0]
    for r in range(1, rings + 1):
        start.append(start[-1] + (1 if r == 1 else valence * (r - 1)))
    n_v = 1 + valence * rings * (rings + 1) // 2
    xyz0 = np.zeros((n_v, 3))

    def vid(r: int, m: int) -> int:
        return 0 if r == 0 else start[r] + (m % (valence * r))

    for r in range(1, rings + 1):
        for m in range(valence * r):
            th = 2.0 * np.pi * m / (valence * r)
            xyz0[vid(r, m)] = (radius * r / rings * np.cos(th), radius * r / rings * np.sin(th), 0.0)
    if z_sigma > 0.0:
        rng = np.random.Generator(np.random.PCG64(SEED_BASE if seed is None else seed))
        phi = rng.uniform(0.0, 2.0 * np.pi)
        rho2 = (xyz0[:, 0] ** 2 + xyz0[:, 1] ** 2) / radius ** 2
        th = np.arctan2(xyz0[:, 1], xyz0[:, 0])
        z = (1.0 - rho2) * (0.5 + 0.5 * np.cos(th - phi))
        xyz0[:, 2] = z_sigma * z / max(np.abs(z).max(), 1e-300)
    tri = []
    for r in range(rings):
        for k in range(valence):
            inner = [vid(r, k * r + m) for m in range(r + 1)]
            outer = [vid(r + 1, k * (r + 1) + m) for m in range(r + 2)]
            for m in range(r + 1):
                tri.append((inner[m], outer[m], outer[m + 1]))
            for m in range(r):
                tri.append((inner[m], outer[m + 1], inner[m + 1]))
    tri = np.array(tri, dtype=np.int32)
    e1 = xyz0[tri[:, 1]] - xyz0[tri[:, 0]]
    e2 = xyz0[tri[:, 2]] - xyz0[tri[:, 0]]
    flip = (e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]) < 0
    tri[flip] = tri[flip][:, [0, 2, 1]]
    ring = np.array([vid(rings, m) for m in range(valence * rings)], dtype=np.int32)
    n_e = tri.shape[0]
    fib = np.zeros((n_e, 3))
    fib[:, 0] = 1.0
    return Mesh(xyz0=xyz0, tri=tri, n_bnodes=np.array([ring.size], dtype=np.int32), bnodes=ring, fib=fib,
                gamma_scale=np.zeros(n_e),
                meta=dict(kind="cone", valence=valence, rings=rings, radius=radius, z_sigma=z_sigma, seed=seed,
                          hmean=radius / rings))


def closed_sphere(freq: int, seed: int, radius: float = 1.0, jitter: float = 0.1, lambda_a: float = 0.9) -> Mesh:
    """A closed surface: the icosahedron's frequency-`freq` geodesic sphere
    (12 vertices of valence 5, the rest 6; 20 freq^2 triangles), outward
    triangles, no boundary ring (so no ghost nodes and nothing to clamp);
    every node moved tangentially by a seeded `jitter` x its shortest edge and
    pulled back to the sphere; fibres along the local east direction,
    activation lambda_a on every element."""
    rng = np.random.Generator(np.random.PCG64(seed))
    V, F = _icosahedron()
    F = _orient_outward(V, F)
    V, F = _geodesic(V, F, freq)
    F = _orient_outward(V, F)
    e = np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1)
    elen = np.linalg.norm(V[e[:, 0]] - V[e[:, 1]], axis=1)
    hmin = np.full(len(V), np.inf)
    np.minimum.at(hmin, e[:, 0], elen)
    np.minimum.at(hmin, e[:, 1], elen)
    nrm = V / np.linalg.norm(V, axis=1)[:, None]
    d = rng.uniform(-1.0, 1.0, size=V.shape) * (jitter * hmin)[:, None]
    d -= (d * nrm).sum(1)[:, None] * nrm
    W = V + d
    V = radius * W / np.linalg.norm(W, axis=1)[:, None]
    c = V[F].mean(1)
    east = np.cross(np.array([0.0, 0.0, 1.0])[None, :], c)
    small = np.linalg.norm(east, axis=1) <= 1e-10
    east[small] = np.array([1.0, 0.0, 0.0])
    east -= ((east * c).sum(1) / (c * c).sum(1))[:, None] * c
    east /= np.linalg.norm(east, axis=1)[:, None]
    return Mesh(xyz0=V, tri=F.astype(np.int32), n_bnodes=np.zeros(0, dtype=np.int32), bnodes=np.zeros(0, dtype=np.int32),
                fib=east, gamma_scale=np.full(len(F), 1.0 - lambda_a),
                meta=dict(kind="sphere", freq=freq, seed=seed, radius=radius, jitter=jitter, hmean=float(elen.mean())))


def capped_lv(n_phi: int, n_theta: int, a: float = 2.0, b: float = 1.0, f_cut: float = 0.375,
              apex_vertex: bool = False, seed: int = SEED_BASE, jitter: float = 0.1,
              alpha_apex: float = 60.0, alpha_base: float = -60.0, lambda_a: float = 0.88) -> Mesh:
    """Truncated prolate spheroid x^2/b^2 + y^2/b^2 + z^2/a^2 = 1 as structured
    quad strips, closed at the apex by flat cap triangles (ibm->n_elmt_base,
    the LV options -lv_a, -lv_b, -lv_f_cut).

    Ring k (0..n_theta-1) holds n_phi nodes at polar angle (k + 1) t_cut /
    n_theta, t_cut = acos(1 - 2 f_cut), node j at azimuth 2 pi j / n_phi.  Ring
    k and k + 1 are joined by n_phi quads, each cut along the same diagonal, so
    that every node counts six base triangles (ring nodes three, which IrrVer's
    boundary rule makes six).  The base triangles come first (n_elmt_base of
    them); then the cap: a fan from an apex node at z = a (n_phi triangles)
    when ``apex_vertex``, else a fan from ring-0 node 0 over the apex ring
    (n_phi - 2 triangles, no apex node).  Boundary rings: ring 0 (the apex
    ring, edge 0, whose ghosts reflect through the base strip) and the base
    ring, both following the base triangles' boundary edges.  Interior ring
    nodes get a seeded tangential jitter of `jitter` x the azimuthal step.
    Triangles face outward.  Fibres: the mid-wall helix with the latitude
    sweep, as lv_ellipsoid; cap triangles carry no activation (gamma_scale
    0), the rest 1 - lambda_a.
    """
    if n_phi < 4 or n_theta < 3:
        raise ValueError("capped_lv needs n_phi >= 4 and n_theta >= 3")
    rng = np.random.Generator(np.random.PCG64(seed))
    t_cut = np.arccos(1.0 - 2.0 * f_cut)
    th = (np.arange(n_theta) + 1.0) * t_cut / n_theta
    ph = 2.0 * np.pi * np.arange(n_phi) / n_phi
    if jitter > 0.0:
        dph = rng.uniform(-1.0, 1.0, size=(n_theta, n_phi)) * jitter * (2.0 * np.pi / n_phi)
        dph[0] = 0.0
        dph[-1] = 0.0
    else:
        dph = np.zeros((n_theta, n_phi))
    PH = ph[None, :] + dph
    TH = np.repeat(th[:, None], n_phi, axis=1)
    V = np.stack([b * np.sin(TH) * np.cos(PH), b * np.sin(TH) * np.sin(PH), a * np.cos(TH)], axis=-1).reshape(-1, 3)

    def nid(k, j):
        return k * n_phi + (j % n_phi)

    F = []
    for k in range(n_theta - 1):
        for j in range(n_phi):
            A, B, C, D = nid(k, j), nid(k, j + 1), nid(k + 1, j + 1), nid(k + 1, j)
            F.append((A, B, C))
            F.append((A, C, D))
    n_base = len(F)
    if apex_vertex:
        apex = len(V)
        V = np.vstack([V, [[0.0, 0.0, a]]])
        for j in range(n_phi):
            F.append((apex, nid(0, j), nid(0, j + 1)))
    else:
        for j in range(1, n_phi - 1):
            F.append((nid(0, 0), nid(0, j), nid(0, j + 1)))
    F = np.array(F, dtype=np.int64)
    # outward: the normal points away from the spheroid's centre
    c = V[F].mean(1)
    nrm = np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]])
    flip = (nrm * c).sum(1) < 0.0
    F[flip] = F[flip][:, [0, 2, 1]]
    # boundary rings from the base triangles' boundary half-edges
    base = F[:n_base]
    he = np.concatenate([base[:, [0, 1]], base[:, [1, 2]], base[:, [2, 0]]])
    hs = set(map(tuple, he))
    nxt = {h[0]: h[1] for h in map(tuple, he) if (h[1], h[0]) not in hs}
    rings = []
    for first in (nid(0, 0), nid(n_theta - 1, 0)):
        ring = [first]
        while nxt[ring[-1]] != first:
            ring.append(nxt[ring[-1]])
        if len(ring) != n_phi:
            raise RuntimeError("a boundary ring is not a closed loop of n_phi nodes")
        rings.append(ring)
    bnodes = np.array(rings[0] + rings[1], dtype=np.int32)
    # fibres and activation
    z_base = a * np.cos(t_cut)
    c = V[F].mean(1)
    en = c / np.array([b * b, b * b, a * a])
    en /= np.linalg.norm(en, axis=1)[:, None]
    down = np.array([0.0, 0.0, -1.0])
    el = down[None, :] - (en @ down)[:, None] * en
    small = np.linalg.norm(el, axis=1) <= 1e-10
    ex = np.array([1.0, 0.0, 0.0])
    el[small] = ex - (en[small] @ ex)[:, None] * en[small]
    el /= np.linalg.norm(el, axis=1)[:, None]
    ec_ = np.cross(en, el)
    zs = np.clip((a - c[:, 2]) / (a - z_base), 0.0, 1.0)
    alpha = np.deg2rad((1.0 - zs) * alpha_apex + zs * alpha_base)
    fib = np.cos(alpha)[:, None] * ec_ + np.sin(alpha)[:, None] * el
    gs = np.full(len(F), 1.0 - lambda_a)
    gs[n_base:] = 0.0
    e = np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1)
    hmean = float(np.linalg.norm(V[e[:, 0]] - V[e[:, 1]], axis=1).mean())
    return Mesh(xyz0=V, tri=F.astype(np.int32), n_bnodes=np.array([n_phi, n_phi], dtype=np.int32), bnodes=bnodes,
                fib=fib, gamma_scale=gs, n_elmt_base=n_base,
                meta=dict(kind="capped_lv", n_phi=n_phi, n_theta=n_theta, a=a, b=b, f_cut=f_cut,
                          apex_vertex=apex_vertex, seed=seed, jitter=jitter, hmean=hmean))


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


# ---- truncated ellipsoid shell (C4; the LV loader's geometry, lv_geometry_unstructured.c) ----
def _icosahedron():
    t = (1.0 + 5.0 ** 0.5) / 2.0
    V = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
                  (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], dtype=float)
    F = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
                  (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
                  (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)], dtype=np.int64)
    return V / np.linalg.norm(V, axis=1)[:, None], F


def _orient_outward(V, F):
    c = V[F].mean(1)
    n = np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]])
    flip = (n * c).sum(1) < 0
    F = F.copy()
    F[flip] = F[flip][:, [0, 2, 1]]
    return F


def _midpoint_refine(V, F):
    key = {}
    Vl = list(V)
    def mid(a, b):
        k = (min(a, b), max(a, b))
        if k not in key:
            p = V[a] + V[b]
            key[k] = len(Vl)
            Vl.append(p / np.linalg.norm(p))
        return key[k]
    out = []
    for a, b, c in F:
        ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
        out += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
    return np.array(Vl), np.array(out, dtype=np.int64)


def _flip_edges(V, F, nflip, rng, zmin):
    """Flip nflip edges of the base sphere whose two ends and two opposite
    corners all have valence 6 (ends become 5, opposite corners 7), each
    vertex used once, all four corners above zmin."""
    F = [list(f) for f in F]
    used = set()
    done = 0
    for _ in range(2000):
        if done == nflip:
            break
        val = np.bincount(np.array(F).ravel(), minlength=len(V))
        fi = int(rng.integers(len(F)))
        k = int(rng.integers(3))
        a, b = F[fi][k], F[fi][(k + 1) % 3]
        c = F[fi][(k + 2) % 3]
        fj = [j for j, f in enumerate(F) if j != fi and a in f and b in f]
        if len(fj) != 1:
            continue
        fj = fj[0]
        d = [v for v in F[fj] if v not in (a, b)][0]
        quad = (a, b, c, d)
        if any(v in used for v in quad) or any(val[v] != 6 for v in quad) or any(V[v, 2] < zmin for v in quad):
            continue
        F[fi] = [c, a, d]
        F[fj] = [d, b, c]
        used.update(quad)
        done += 1
    return np.array(F, dtype=np.int64)


def _geodesic(V, F, n):
    """Frequency-n subdivision of every base face, points pushed to the unit
    sphere; base vertices keep their valence, all new vertices get 6."""
    key, pts, tris = {}, [], []
    def vid(f, i, j):
        a, b, c = F[f]
        if i == 0 and j == 0:
            k = ("v", a)
        elif i == n and j == 0:
            k = ("v", b)
        elif i == 0 and j == n:
            k = ("v", c)
        elif j == 0:
            k = ("e", a, b, i) if a < b else ("e", b, a, n - i)
        elif i == 0:
            k = ("e", a, c, j) if a < c else ("e", c, a, n - j)
        elif i + j == n:
            k = ("e", b, c, j) if b < c else ("e", c, b, i)
        else:
            k = ("f", f, i, j)
        if k not in key:
            p = V[a] + (V[b] - V[a]) * (i / n) + (V[c] - V[a]) * (j / n)
            key[k] = len(pts)
            pts.append(p / np.linalg.norm(p))
        return key[k]
    for f in range(len(F)):
        for j in range(n):
            for i in range(n - j):
                tris.append((vid(f, i, j), vid(f, i + 1, j), vid(f, i, j + 1)))
                if i + j < n - 1:
                    tris.append((vid(f, i + 1, j), vid(f, i + 1, j + 1), vid(f, i, j + 1)))
    return np.array(pts), np.array(tris, dtype=np.int64)


def _clean_cap(F):
    """Drop triangles until the cut boundary is one simple ring: no pinched
    boundary vertex and no triangle with two boundary edges."""
    while True:
        e = np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1)
        u, inv, cnt = np.unique(e, axis=0, return_inverse=True, return_counts=True)
        bmask = (cnt == 1)[inv.ravel()].reshape(3, -1).T          # (nf, 3) edge is on the boundary
        nbe = np.bincount(u[cnt == 1].ravel(), minlength=F.max() + 1)
        pinch = np.where(nbe > 2)[0]
        drop = bmask.sum(1) >= 2
        if len(pinch):
            drop |= np.isin(F, pinch).any(1)
        if not drop.any():
            return F
        F = F[~drop]


def lv_ellipsoid(freq: int, seed: int, a: float = 2.0, b: float = 1.0, f_cut: float = 0.375, nflip: int = 4,
                 jitter: float = 0.1, alpha_apex: float = 60.0, alpha_base: float = -60.0,
                 lambda_a: float = 0.88) -> Mesh:
    """Truncated prolate spheroid shell x^2/b^2 + y^2/b^2 + z^2/a^2 = 1 kept
    for z >= a (1 - 2 f_cut) (the LV options -lv_a, -lv_b, -lv_f_cut), apex at
    z = +a, outward-oriented triangles, the cut rim as the one boundary ring.

    Mesh: the icosahedron refined twice by edge midpoints, nflip seeded edge
    flips above the cut (valence 5/7 pairs), then a frequency-`freq` geodesic
    subdivision, so the extraordinary vertices stay isolated; interior nodes get a seeded
    tangential jitter of `jitter` x the node's shortest edge, pulled back to the
    surface.  Fibres: the mid-wall helix of lv_geometry_unstructured.c:296-366
    with the latitude sweep: e_n = unit grad F at the element centroid, e_l =
    the projection of -e_z, e_c = e_n x e_l, alpha = (1 - z*) alpha_apex +
    z* alpha_base with z* = (a - c_z) / (a - z_base); activation lambda_a on
    every element (tapers off).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    V, F = _icosahedron()
    V, F = _midpoint_refine(V, _orient_outward(V, F))
    V, F = _midpoint_refine(V, _orient_outward(V, F))
    z_base = a * (1.0 - 2.0 * f_cut)
    F = _orient_outward(V, _flip_edges(V, _orient_outward(V, F), nflip, rng, z_base / a + 0.15))
    V, F = _geodesic(V, F, freq)
    F = _orient_outward(V, F)
    V = V * np.array([b, b, a])
    keep = V[:, 2] >= z_base
    F = F[keep[F].all(1)]
    F = _clean_cap(F)
    used = np.unique(F)
    remap = -np.ones(len(V), dtype=np.int64)
    remap[used] = np.arange(len(used))
    V, F = V[used], remap[F]
    # boundary ring, following the triangles' edge directions
    he = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
    s = set(map(tuple, he))
    bhe = [h for h in map(tuple, he) if (h[1], h[0]) not in s]
    nxt = dict(bhe)
    start = min(nxt)
    ring = [start]
    while nxt[ring[-1]] != start:
        ring.append(nxt[ring[-1]])
    if len(ring) != len(bhe):
        raise RuntimeError("the cut boundary is not a single ring")
    ring = np.array(ring, dtype=np.int32)
    # tangential jitter of interior nodes, scaled by each node's shortest edge
    e = np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1)
    elen = np.linalg.norm(V[e[:, 0]] - V[e[:, 1]], axis=1)
    hmean = elen.mean()
    hmin = np.full(len(V), np.inf)
    np.minimum.at(hmin, e[:, 0], elen)
    np.minimum.at(hmin, e[:, 1], elen)
    interior = np.ones(len(V), bool)
    interior[ring] = False
    grad = V / np.array([b * b, b * b, a * a])
    nrm = grad / np.linalg.norm(grad, axis=1)[:, None]
    d = rng.uniform(-1.0, 1.0, size=V.shape) * (jitter * hmin)[:, None]
    d -= (d * nrm).sum(1)[:, None] * nrm
    W = V + np.where(interior[:, None], d, 0.0)
    s_ = np.sqrt((W[:, 0] / b) ** 2 + (W[:, 1] / b) ** 2 + (W[:, 2] / a) ** 2)
    V = np.where(interior[:, None], W / s_[:, None], V)
    # fibres (mid-wall helix, latitude sweep) and activation
    c = V[F].mean(1)
    en = c / np.array([b * b, b * b, a * a])
    en /= np.linalg.norm(en, axis=1)[:, None]
    down = np.array([0.0, 0.0, -1.0])
    el = down[None, :] - (en @ down)[:, None] * en
    small = np.linalg.norm(el, axis=1) <= 1e-10
    ex = np.array([1.0, 0.0, 0.0])
    el[small] = ex - (en[small] @ ex)[:, None] * en[small]
    el /= np.linalg.norm(el, axis=1)[:, None]
    ec_ = np.cross(en, el)
    zs = np.clip((a - c[:, 2]) / (a - z_base), 0.0, 1.0)
    alpha = np.deg2rad((1.0 - zs) * alpha_apex + zs * alpha_base)
    fib = np.cos(alpha)[:, None] * ec_ + np.sin(alpha)[:, None] * el
    return Mesh(xyz0=V, tri=F.astype(np.int32), n_bnodes=np.array([ring.size], dtype=np.int32), bnodes=ring,
                fib=fib, gamma_scale=np.full(len(F), 1.0 - lambda_a),
                meta=dict(kind="lv", freq=freq, seed=seed, a=a, b=b, f_cut=f_cut, nflip=nflip, jitter=jitter,
                          hmean=hmean))
