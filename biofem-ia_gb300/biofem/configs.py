"""The workloads the path is measured and checked on.

Each entry names the mesh, the activation field, the material (stated
convention mu = E/(2(1+nu)), K = E/(3(1-2nu)) with E = 1, nu = 0.3), the
quadrature (``-num_gaussian_quad_points``), the C33 sub-iteration count
(``-C33_subitr_nums``), the follower pressure and the initial state.
Seeds are SEED_BASE + config index.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import mesh as meshmod

E_MOD = 1.0
NU = 0.3
MU = E_MOD / (2.0 * (1.0 + NU))
BULK = E_MOD / (3.0 * (1.0 - 2.0 * NU))
H0 = 0.01


@dataclass(frozen=True)
class Workload:
    name: str
    nx: int
    ny: int
    n_qp: int = 3
    c33_iters: int = 3
    pressure: float = 1e-4
    z_sigma: float = 0.0
    activation: str = "uniform"      # uniform | smooth | random
    lambda_a: float = 0.9
    disp_rel: float = 0.0            # displacement amplitude / edge length h
    index: int = 0
    theta: float = 0.0               # fibre angle from e_x (uniform activation)
    z_smooth: bool = False           # smooth imperfection instead of per-node noise
    basis: int = 0                   # 0 reference four-decimal basis tables, 1 exact (extension)
    tnormal: int = 0                 # 1: thickness metric from n,alpha only (extension)
    dead_load: int = 0               # 1: dead-load pressure (SurfaceConstNormalPressure) instead of follower
    iso_act: int = 0                 # 1: isotropic active gradient (-cart_fib_act 0) instead of along the fibre

    @property
    def seed(self) -> int:
        return meshmod.SEED_BASE + self.index

    @property
    def n_elmt(self) -> int:
        return 2 * self.nx * self.ny

    def build_mesh(self) -> meshmod.Mesh:
        m = meshmod.flat_membrane(self.nx, self.ny, z_sigma=self.z_sigma, seed=self.seed, z_smooth=self.z_smooth)
        if self.activation == "uniform":
            meshmod.set_uniform_activation(m, self.lambda_a, (np.cos(self.theta), np.sin(self.theta), 0.0))
        elif self.activation == "smooth":
            meshmod.set_smooth_activation(m)
        elif self.activation == "random":
            meshmod.set_random_activation(m, self.seed + 1)
        else:
            raise ValueError(self.activation)
        m.meta["workload"] = self.name
        return m

    def initial_x(self, m: meshmod.Mesh, xyz0_full: np.ndarray) -> np.ndarray:
        h = m.meta["lx"] / self.nx
        return meshmod.initial_state(m, xyz0_full, disp_amp=self.disp_rel * h, seed=self.seed + 2)


# C1: 32x24 cells (825 nodes, 1536 triangles), z perturbed N(0,1e-3), lambda_a 0.9 along e_x.
C1 = Workload("C1_flat_32x24", 32, 24, z_sigma=1e-3, activation="uniform", lambda_a=0.9, index=0)
# C2: 256x192 cells (49,601 nodes, 98,304 triangles), smooth lambda_a field, displacement 1e-2 h.
C2 = Workload("C2_flat_256x192", 256, 192, activation="smooth", disp_rel=1e-2, index=1)
# C3: 1024x768 cells (788,225 nodes, 1,572,864 triangles), random fibre angle and lambda_a,
# 6 thickness points (an extension: the reference's rule stops at 5).  With h ~ h0/10 the
# reference's four-decimal basis tables fold the outer thickness points of every element
# (their second-derivative rows do not sum to zero), and the normal part of a3,alpha folds
# them on the ghost-reflected side patches, so C3 uses the exact tables and n,alpha.
C3 = Workload("C3_flat_1024x768", 1024, 768, n_qp=6, activation="random", index=2, basis=1, tnormal=1)

@dataclass(frozen=True)
class LVWorkload:
    """Truncated prolate spheroid shell (the LV loader's geometry), see
    mesh.lv_ellipsoid: semi-axes (1, 1, 2), cut at z = 0.5, helix -60 deg at
    the base to +60 deg at the apex, lambda_a uniform, internal follower
    pressure, base ring clamped, starting from the reference state."""
    name: str
    freq: int
    index: int = 0
    n_qp: int = 3
    c33_iters: int = 3
    pressure: float = 1e-3
    lambda_a: float = 0.88
    nflip: int = 4
    jitter: float = 0.1
    basis: int = 0
    tnormal: int = 0
    dead_load: int = 0
    iso_act: int = 0

    @property
    def seed(self) -> int:
        return meshmod.SEED_BASE + self.index

    def build_mesh(self) -> meshmod.Mesh:
        m = meshmod.lv_ellipsoid(self.freq, self.seed, nflip=self.nflip, jitter=self.jitter, lambda_a=self.lambda_a)
        m.meta["workload"] = self.name
        return m

    def initial_x(self, m: meshmod.Mesh, xyz0_full: np.ndarray) -> np.ndarray:
        return meshmod.initial_state(m, xyz0_full)


# C4: ~200k triangles (frequency-41 geodesic cap: 200,614 triangles, 100,761 nodes, 20
# extraordinary interior vertices of valence 5/7, a jagged cut rim of boundary valence 5/6/7).
C4 = LVWorkload("C4_lv_ellipsoid", 41, index=3)

ALL = {w.name: w for w in (C1, C2, C3, C4)}


@dataclass(frozen=True)
class ConeWorkload:
    """A flat disc with one interior vertex of the given valence (3..10; see
    mesh.cone_disc): the one-step subdivision of every valence the
    reference's tables cover, up to the 16-node patch.  Random fibre angle
    and lambda_a, follower pressure, boundary ring clamped, a seeded smooth
    bump and a seeded displacement of 1e-2 of the ring spacing."""
    name: str
    valence: int
    rings: int = 5
    index: int = 0
    n_qp: int = 3
    c33_iters: int = 3
    pressure: float = 1e-3
    z_sigma: float = 2e-3
    disp_rel: float = 1e-2
    basis: int = 0
    tnormal: int = 0
    dead_load: int = 0
    iso_act: int = 0

    @property
    def seed(self) -> int:
        return meshmod.SEED_BASE + self.index

    def build_mesh(self) -> meshmod.Mesh:
        m = meshmod.cone_disc(self.valence, self.rings, z_sigma=self.z_sigma, seed=self.seed)
        meshmod.set_random_activation(m, self.seed + 1)
        m.meta["workload"] = self.name
        return m

    def initial_x(self, m: meshmod.Mesh, xyz0_full: np.ndarray) -> np.ndarray:
        return meshmod.initial_state(m, xyz0_full, disp_amp=self.disp_rel * m.meta["hmean"], seed=self.seed + 2)


@dataclass(frozen=True)
class SphereWorkload:
    """A closed surface (mesh.closed_sphere): no boundary ring, so no ghost
    nodes and no clamp; internal follower pressure, fibres along the local
    east direction, a seeded displacement of 1e-2 of the mean edge.  With
    ``drop`` the listed triangles are removed: holes whose rims are not
    declared as rings, so the patches there repeat a node (the reference's
    stencil fill-in, bending.c:1637-1650)."""
    name: str
    freq: int
    index: int = 0
    n_qp: int = 3
    c33_iters: int = 3
    pressure: float = 1e-3
    lambda_a: float = 0.9
    jitter: float = 0.1
    disp_rel: float = 1e-2
    basis: int = 0
    tnormal: int = 0
    dead_load: int = 0
    iso_act: int = 0
    drop: tuple = ()       # triangles removed: holes whose rims are no boundary ring

    @property
    def seed(self) -> int:
        return meshmod.SEED_BASE + self.index

    def build_mesh(self) -> meshmod.Mesh:
        m = meshmod.closed_sphere(self.freq, self.seed, jitter=self.jitter, lambda_a=self.lambda_a)
        if self.drop:
            keep = np.ones(m.n_elmt, bool)
            keep[list(self.drop)] = False
            m.tri, m.fib, m.gamma_scale = m.tri[keep], m.fib[keep], m.gamma_scale[keep]
            m.meta["drop"] = list(self.drop)
        m.meta["workload"] = self.name
        return m

    def initial_x(self, m: meshmod.Mesh, xyz0_full: np.ndarray) -> np.ndarray:
        return meshmod.initial_state(m, xyz0_full, disp_amp=self.disp_rel * m.meta["hmean"], seed=self.seed + 2)


@dataclass(frozen=True)
class CappedLVWorkload:
    """A truncated prolate spheroid of structured quad strips closed at the
    apex by flat cap triangles (mesh.capped_lv, ibm->n_elmt_base): a fan from
    an apex node, or from the apex ring's first node.  Follower pressure,
    mid-wall helix fibres, no activation on the cap, a seeded displacement of
    1e-2 of the mean edge.  No ring is clamped unless ``clamp`` (ring 0, the
    apex ring: in the fan from the apex ring every cap row would be a
    clamped row)."""
    name: str
    n_phi: int
    n_theta: int
    apex_vertex: bool = False
    clamp: bool = False
    index: int = 0
    n_qp: int = 3
    c33_iters: int = 3
    pressure: float = 1e-3
    jitter: float = 0.1
    disp_rel: float = 1e-2
    basis: int = 0
    tnormal: int = 0
    dead_load: int = 0
    iso_act: int = 0

    @property
    def seed(self) -> int:
        return meshmod.SEED_BASE + self.index

    def build_mesh(self) -> meshmod.Mesh:
        m = meshmod.capped_lv(self.n_phi, self.n_theta, apex_vertex=self.apex_vertex, seed=self.seed,
                              jitter=self.jitter)
        m.meta["workload"] = self.name
        return m

    def initial_x(self, m: meshmod.Mesh, xyz0_full: np.ndarray) -> np.ndarray:
        return meshmod.initial_state(m, xyz0_full, disp_amp=self.disp_rel * m.meta["hmean"], seed=self.seed + 2)


def capped(n_phi: int, n_theta: int, apex_vertex: bool = False, **kw) -> CappedLVWorkload:
    args = dict(index=80 + n_phi + (1 if apex_vertex else 0))
    args.update(kw)
    tag = "apex" if apex_vertex else "fan"
    return CappedLVWorkload(f"capped_{tag}_{n_phi}x{n_theta}", n_phi, n_theta, apex_vertex, **args)


def cone(valence: int, **kw) -> ConeWorkload:
    args = dict(index=60 + valence)
    args.update(kw)
    return ConeWorkload(f"cone_v{valence}", valence, **args)


def small(nx: int, ny: int, **kw) -> Workload:
    """A small flat case for parity tests (z perturbed, smooth activation, displaced)."""
    args = dict(z_sigma=1e-3, activation="smooth", disp_rel=1e-2, index=10)
    args.update(kw)
    return Workload(f"flat_{nx}x{ny}", nx, ny, **args)


SERVE_SEED = meshmod.SEED_BASE + 500


def serve_request(i: int, nx_lo: int = 16, nx_hi: int = 256) -> Workload:
    """Request i of the load-step serving stream (the `biofem sweep` case mix):
    nx = round(exp U[ln nx_lo, ln nx_hi]), ny = round(0.75 nx), a seeded
    smooth z imperfection of peak 1e-3 (per-node noise of that size folds the
    shell at the finer meshes of the range), lambda_a ~ U[0.85, 1] and fibre
    angle ~ U[0, pi) uniform over the sheet, follower pressure
    ~ U[1e-5, 1e-3], starting from the reference state."""
    rng = np.random.default_rng(SERVE_SEED + i)
    nx = int(round(np.exp(rng.uniform(np.log(nx_lo), np.log(nx_hi)))))
    ny = max(2, int(round(0.75 * nx)))
    lam = float(rng.uniform(0.85, 1.0))
    theta = float(rng.uniform(0.0, np.pi))
    p = float(rng.uniform(1e-5, 1e-3))
    return Workload(f"serve_{i}_{nx}x{ny}", nx, ny, pressure=p, z_sigma=1e-3, activation="uniform",
                    lambda_a=lam, index=1000 + i, theta=theta, z_smooth=True)
