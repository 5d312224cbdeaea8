"""Seeded synthetic Magritte models for the formal-solve workloads.

No public dataset is involved: every model is generated from a seed with the
shapes, sizes and value distributions of the workload it stands for.  A model is
a ``RawModel``: exactly the fields a Magritte user sets through the Python API
before calling ``compute_spectral_discretisation`` (positions, velocities as
v/c, neighbour lists, boundary, rays, abundances, temperature, turbulence, line
data, quadrature).  ``magritte_gb300.core.Model.from_raw`` loads one into the
host model.

Workloads:
  * ``grid_cube``       -- 20^3 Cartesian grid, 26-neighbour lists, 12 HEALPix
                           rays, 2-level CO-like line, nquads 11 (8000 points).
  * ``grid_sphere``     -- 64^3 grid with a spherical cutout of radius half the
                           box (rays of uneven length), 48 rays, 5-level linear
                           rotor (4 lines), nquads 31.
  * ``single_ray_1d``   -- the reference's 1D single-ray known-answer models
                           (tests/benchmarks/analytic/all_constant_single_ray.py,
                           all_zero_single_ray.py).
The molecular mass of the CO-like species is not fixed by the workload
descriptions; 28 amu is used throughout.
"""
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import healpix

# Physical constants, identical to src/tools/constants.hpp:15-40 of the reference.
CC = 2.99792458e8
HH = 6.62607004e-34
KB = 1.38064852e-23
AMU = 1.66053904e-27
T_CMB = 2.7254800

BC_ZERO, BC_THERMAL, BC_CMB = 0, 1, 2


@dataclass
class CollisionPartner:
    num_col_partner: int
    orth_or_para_H2: str
    icol: np.ndarray
    jcol: np.ndarray
    tmp: np.ndarray
    Cd: np.ndarray  # [ntmp][ncol] de-excitation rates [m^3/s]
    Ce: np.ndarray  # [ntmp][ncol] excitation rates

    @property
    def ncol(self):
        return len(self.icol)

    @property
    def ntmp(self):
        return len(self.tmp)


@dataclass
class Linedata:
    """Line data of one line-producing species (src/model/lines/lineProducingSpecies/
    linedata/linedata.hpp:10-39)."""
    num: int
    sym: str
    inverse_mass: float
    energy: np.ndarray
    weight: np.ndarray
    irad: np.ndarray
    jrad: np.ndarray
    A: np.ndarray
    colpar: List[CollisionPartner] = field(default_factory=list)
    # line frequencies and Einstein B coefficients as given (a model read from files
    # carries its own); None derives them from the levels as the reference's setup does
    frequency_given: Optional[np.ndarray] = None
    Bs_given: Optional[np.ndarray] = None
    Ba_given: Optional[np.ndarray] = None

    @property
    def nlev(self):
        return len(self.energy)

    @property
    def nrad(self):
        return len(self.irad)

    @property
    def frequency(self):
        if self.frequency_given is not None:
            return self.frequency_given
        return (self.energy[self.irad] - self.energy[self.jrad]) / HH

    @property
    def Bs(self):
        if self.Bs_given is not None:
            return self.Bs_given
        f = self.frequency
        return self.A * CC**2 / (2.0 * HH * f**3)

    @property
    def Ba(self):
        if self.Ba_given is not None:
            return self.Ba_given
        return self.weight[self.irad] / self.weight[self.jrad] * self.Bs


@dataclass
class RawModel:
    name: str
    dimension: int
    position: np.ndarray           # [P,3] m
    velocity: np.ndarray           # [P,3] v/c
    neighbors: np.ndarray          # flat CSR column indices
    n_neighbors: np.ndarray        # [P]
    boundary2point: np.ndarray     # [B]
    boundary_condition: np.ndarray  # [B] 0 Zero, 1 Thermal, 2 CMB
    boundary_temperature: np.ndarray  # [B]
    ray_direction: np.ndarray      # [nrays,3]
    ray_weight: np.ndarray         # [nrays]
    abundance: np.ndarray          # [P, nspecs] number densities
    temperature: np.ndarray        # [P]
    vturb2: np.ndarray             # [P] (v_turb/c)^2
    linedata: List[Linedata]
    quad_roots: List[np.ndarray]
    quad_weights: List[np.ndarray]
    nquads: int
    spherical_symmetry: bool = False
    # adaptive ray directions (Rays::use_adaptive_directions): per-point directions
    # [P][nrays][3] and weights [P][nrays]; ray_direction / ray_weight then hold point
    # 0's, which is what the reference's imagers read (Rays::get_direction<false>)
    adaptive_direction: Optional[np.ndarray] = None
    adaptive_weight: Optional[np.ndarray] = None

    @property
    def npoints(self):
        return self.position.shape[0]

    @property
    def nrays(self):
        return self.ray_direction.shape[0]


def quadrature(nquads: int):
    """Gauss-Hermite roots and normalised weights (magritte/setup.py:480-503)."""
    roots, weights = np.polynomial.hermite.hermgauss(nquads)
    return roots, weights / np.sum(weights)


def linear_rotor(nlev: int, B_hz: float, A10: float, mass_amu: float, num: int = 0,
                 collider: int = 1, seed: int = 0, ntmp: int = 8) -> Linedata:
    """Synthetic linear rotor: E_J = h B J(J+1), g_J = 2J+1, transitions J -> J-1
    with A_ul scaling as nu^3 from ``A10``.  One collision partner with
    de-excitation rates C0 (T/100)^alpha (seeded) and excitation rates from
    detailed balance (magritte/setup.py:731-735)."""
    J = np.arange(nlev, dtype=np.float64)
    energy = HH * B_hz * J * (J + 1.0)
    weight = 2.0 * J + 1.0
    irad = np.arange(1, nlev, dtype=np.uint32)
    jrad = irad - 1
    nu = (energy[irad] - energy[jrad]) / HH
    A = A10 * (nu / nu[0]) ** 3
    rng = np.random.default_rng(seed)
    pairs = [(i, j) for i in range(1, nlev) for j in range(i)]
    icol = np.array([p[0] for p in pairs], dtype=np.uint32)
    jcol = np.array([p[1] for p in pairs], dtype=np.uint32)
    tmp = np.geomspace(10.0, 1000.0, ntmp)
    C0 = 10.0 ** rng.uniform(-17.0, -16.0, size=len(pairs))  # m^3/s
    alpha = rng.uniform(0.0, 0.5, size=len(pairs))
    Cd = np.array([C0 * (t / 100.0) ** alpha for t in tmp])
    Ce = np.array([[Cd[t][k] * weight[icol[k]] / weight[jcol[k]]
                    * np.exp(-(energy[icol[k]] - energy[jcol[k]]) / (KB * tmp[t]))
                    for k in range(len(pairs))] for t in range(len(tmp))])
    cp = CollisionPartner(collider, "n", icol, jcol, tmp, Cd, Ce)
    return Linedata(num=num, sym="rotor", inverse_mass=1.0 / mass_amu, energy=energy, weight=weight,
                    irad=irad, jrad=jrad, A=A, colpar=[cp])


def two_level(nu_hz: float, A: float, g_ratio: float, mass_amu: float, num: int = 0,
              collider: int = 1) -> Linedata:
    """Two-level species with E_u = h nu, g_u/g_l = g_ratio."""
    energy = np.array([0.0, HH * nu_hz])
    weight = np.array([1.0, g_ratio])
    irad = np.array([1], dtype=np.uint32)
    jrad = np.array([0], dtype=np.uint32)
    tmp = np.array([20.0])
    Cd = np.array([[2.0e-16]])
    Ce = np.array([[Cd[0][0] * weight[1] / weight[0] * np.exp(-energy[1] / (KB * tmp[0]))]])
    cp = CollisionPartner(collider, "n", np.array([1], dtype=np.uint32), np.array([0], dtype=np.uint32),
                          tmp, Cd, Ce)
    return Linedata(num=num, sym="2lev", inverse_mass=1.0 / mass_amu, energy=energy, weight=weight,
                    irad=irad, jrad=jrad, A=np.array([A]), colpar=[cp])


def lamda_test_species() -> Linedata:
    """The reference's fictitious 'test' species (tests/data/test.txt): 2 levels,
    E = 0 and 6 cm^-1, g = 1 and 3, A = 1e-4 /s, molecular weight 1, one H2
    collision rate 2e-10 cm^3/s at 20 K.  Energies are converted from cm^-1 to J
    as the LAMDA reader does (magritte/setup.py:650-660: E[J] = E[cm^-1] * 100 h c)."""
    energy = np.array([0.0, 6.0]) * 1.0e2 * HH * CC
    weight = np.array([1.0, 3.0])
    irad = np.array([1], dtype=np.uint32)
    jrad = np.array([0], dtype=np.uint32)
    tmp = np.array([20.0])
    Cd = np.array([[2.0e-10 * 1.0e-6]])
    Ce = np.array([[Cd[0][0] * weight[1] / weight[0] * np.exp(-(energy[1] - energy[0]) / (KB * tmp[0]))]])
    cp = CollisionPartner(1, "n", np.array([1], dtype=np.uint32), np.array([0], dtype=np.uint32), tmp, Cd, Ce)
    return Linedata(num=0, sym="test", inverse_mass=1.0, energy=energy, weight=weight, irad=irad,
                    jrad=jrad, A=np.array([1.0e-4]), colpar=[cp])


# --------------------------------------------------------------------------
# Geometry builders
# --------------------------------------------------------------------------
_OFFSETS26 = [(dx, dy, dz) for dx in (-1, 0, 1) for dy in (-1, 0, 1) for dz in (-1, 0, 1)
              if (dx, dy, dz) != (0, 0, 0)]


def grid_neighbors(keep: np.ndarray):
    """26-neighbour CSR lists on an n^3 grid restricted to ``keep`` (bool [n,n,n]).
    Point order: x fastest, then y, then z.  Neighbour order: offsets (dx, dy, dz)
    in lexicographic order over {-1,0,1}^3.  Returns (index map, neighbors,
    n_neighbors, full_mask) where full_mask marks points with all 26 neighbours."""
    n = keep.shape[0]
    idx = -np.ones(keep.shape, dtype=np.int64)
    kz, ky, kx = np.nonzero(keep.transpose(2, 1, 0))  # order: x fastest
    pts = np.stack([kx, ky, kz], axis=1)
    idx[pts[:, 0], pts[:, 1], pts[:, 2]] = np.arange(len(pts))
    nbs = []
    counts = np.zeros(len(pts), dtype=np.uint32)
    for off in _OFFSETS26:
        q = pts + np.array(off)
        ok = np.all((q >= 0) & (q < n), axis=1)
        nb = np.full(len(pts), -1, dtype=np.int64)
        nb[ok] = idx[q[ok, 0], q[ok, 1], q[ok, 2]]
        nbs.append(nb)
    nbs = np.stack(nbs, axis=1)  # [P, 26]
    valid = nbs >= 0
    counts = valid.sum(axis=1).astype(np.uint32)
    flat = nbs[valid].astype(np.uint32)  # row-major keeps offset order per point
    full = counts == 26
    return pts, flat, counts, full


def grid_cube(n: int = 20, box: float = 1.0e13, nside: int = 1, nquads: int = 11, seed: int = 0,
              n_h2: float = 1.0e12, abundance: float = 1.0e-4, t_range=(20.0, 100.0),
              v_turb: float = 150.0, sigma_v: float = 1.0e3) -> RawModel:
    """Cartesian n^3 grid in a cube of side ``box``; surface points are CMB
    boundaries; T ~ U(t_range); velocity i.i.d. Gaussian per component."""
    rng = np.random.default_rng(seed)
    keep = np.ones((n, n, n), dtype=bool)
    pts, nbs, counts, full = grid_neighbors(keep)
    dx = box / (n - 1)
    position = pts.astype(np.float64) * dx
    P = len(pts)
    on_surface = np.any((pts == 0) | (pts == n - 1), axis=1)
    b2p = np.nonzero(on_surface)[0].astype(np.uint32)
    temperature = rng.uniform(t_range[0], t_range[1], size=P)
    velocity = rng.normal(0.0, sigma_v, size=(P, 3)) / CC
    direction, weight = healpix.uniform_rays(12 * nside * nside)
    ld = two_level(1.1527e11, 7.2e-8, 3.0, 28.0)
    roots, wts = quadrature(nquads)
    abund = np.stack([np.full(P, n_h2 * abundance), np.full(P, n_h2)], axis=1)
    return RawModel(
        name=f"grid_cube_{n}", dimension=3, position=position, velocity=velocity, neighbors=nbs,
        n_neighbors=counts, boundary2point=b2p, boundary_condition=np.full(len(b2p), BC_CMB, np.int32),
        boundary_temperature=np.full(len(b2p), T_CMB), ray_direction=direction, ray_weight=weight,
        abundance=abund, temperature=temperature, vturb2=np.full(P, (v_turb / CC) ** 2),
        linedata=[ld], quad_roots=[roots], quad_weights=[wts], nquads=nquads)


def grid_sphere(n: int = 64, box: float = 1.0e13, nside: int = 2, nquads: int = 31, nlev: int = 5,
                seed: int = 0, n_h2: float = 1.0e12, abundance: float = 1.0e-4, t0: float = 300.0,
                v_in: float = 5.0e3, v_out: float = 15.0e3, sigma_v: float = 0.5e3,
                v_turb: float = 150.0) -> RawModel:
    """n^3 grid cut to the sphere of radius box/2 about the box centre; points
    missing any of their 26 neighbours are CMB boundaries.  T = t0 (r/dx)^-0.5
    (t0 inside one cell), radial velocity rising linearly from v_in at the centre
    to v_out at the edge plus Gaussian noise, a 5-level linear rotor with
    B = 57.6 GHz."""
    rng = np.random.default_rng(seed)
    dx = box / (n - 1)
    g = np.arange(n, dtype=np.float64)
    c = 0.5 * (n - 1)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    r_cells = np.sqrt((X - c) ** 2 + (Y - c) ** 2 + (Z - c) ** 2)
    keep = r_cells <= 0.5 * (n - 1)
    pts, nbs, counts, full = grid_neighbors(keep)
    position = pts.astype(np.float64) * dx
    P = len(pts)
    b2p = np.nonzero(~full)[0].astype(np.uint32)
    rel = (pts - c) * dx
    r = np.sqrt(np.sum(rel * rel, axis=1))
    rmax = 0.5 * (n - 1) * dx
    temperature = t0 * np.maximum(r / dx, 1.0) ** -0.5
    rhat = np.zeros_like(rel)
    nz = r > 0
    rhat[nz] = rel[nz] / r[nz, None]
    vr = v_in + (v_out - v_in) * (r / rmax)
    velocity = (vr[:, None] * rhat + rng.normal(0.0, sigma_v, size=(P, 3))) / CC
    direction, weight = healpix.uniform_rays(12 * nside * nside)
    ld = linear_rotor(nlev, 57.6e9, 7.2e-8, 28.0, seed=seed)
    roots, wts = quadrature(nquads)
    abund = np.stack([np.full(P, n_h2 * abundance), np.full(P, n_h2)], axis=1)
    return RawModel(
        name=f"grid_sphere_{n}", dimension=3, position=position, velocity=velocity, neighbors=nbs,
        n_neighbors=counts, boundary2point=b2p, boundary_condition=np.full(len(b2p), BC_CMB, np.int32),
        boundary_temperature=np.full(len(b2p), T_CMB), ray_direction=direction, ray_weight=weight,
        abundance=abund, temperature=temperature, vturb2=np.full(P, (v_turb / CC) ** 2),
        linedata=[ld], quad_roots=[roots], quad_weights=[wts], nquads=nquads)


_CUTOUT_CACHE = {}


def _sphere_cutout(n: int):
    """Grid points of the n^3 sphere cutout (radius (n-1)/2 cells about the box
    centre), their CSR neighbours and the boundary mask, cached per n."""
    if n not in _CUTOUT_CACHE:
        g = np.arange(n, dtype=np.float64)
        c = 0.5 * (n - 1)
        X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
        keep = np.sqrt((X - c) ** 2 + (Y - c) ** 2 + (Z - c) ** 2) <= 0.5 * (n - 1)
        _CUTOUT_CACHE[n] = grid_neighbors(keep)
    return _CUTOUT_CACHE[n]


def batch_model(npoints: int, nside: int = 1, nlev: int = 2, nquads: int = 11, seed: int = 0,
                box: float = 1.0e13, n_h2: float = 1.0e12, abundance: float = 1.0e-4,
                t_range=(20.0, 100.0), v_turb: float = 150.0, sigma_v: float = 1.0e3) -> RawModel:
    """One model of the many-model batch: the sphere cutout of an n^3 grid with n
    chosen so that the cutout has about ``npoints`` points (pi/6 n^3), boundary
    points those missing a neighbour (CMB), T ~ U(t_range), velocity i.i.d.
    Gaussian per component, an ``nlev``-level linear rotor (B = 57.6 GHz)."""
    rng = np.random.default_rng(seed)
    n = max(4, int(round((6.0 * npoints / np.pi) ** (1.0 / 3.0))))
    pts, nbs, counts, full = _sphere_cutout(n)
    dx = box / (n - 1)
    position = pts.astype(np.float64) * dx
    P = len(pts)
    b2p = np.nonzero(~full)[0].astype(np.uint32)
    temperature = rng.uniform(t_range[0], t_range[1], size=P)
    velocity = rng.normal(0.0, sigma_v, size=(P, 3)) / CC
    direction, weight = healpix.uniform_rays(12 * nside * nside)
    ld = linear_rotor(nlev, 57.6e9, 7.2e-8, 28.0, seed=seed)
    roots, wts = quadrature(nquads)
    abund = np.stack([np.full(P, n_h2 * abundance), np.full(P, n_h2)], axis=1)
    return RawModel(
        name=f"batch_{n}_{seed}", dimension=3, position=position, velocity=velocity, neighbors=nbs,
        n_neighbors=counts, boundary2point=b2p, boundary_condition=np.full(len(b2p), BC_CMB, np.int32),
        boundary_temperature=np.full(len(b2p), T_CMB), ray_direction=direction, ray_weight=weight,
        abundance=abund, temperature=temperature, vturb2=np.full(P, (v_turb / CC) ** 2),
        linedata=[ld], quad_roots=[roots], quad_weights=[wts], nquads=nquads)


def many_models(n_models: int = 512, p_range=(2000, 60000), seed: int = 0):
    """Specifications of the many-model batch: point counts log-uniform in p_range,
    nside in {1, 2} (12 or 48 rays), 2-5 levels, nquads in {11, 21, 31}.  Returns
    a list of keyword dicts for batch_model."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_models):
        out.append(dict(npoints=int(np.exp(rng.uniform(np.log(p_range[0]), np.log(p_range[1])))),
                        nside=int(rng.integers(1, 3)), nlev=int(rng.integers(2, 6)),
                        nquads=int(rng.choice([11, 21, 31])), seed=seed * 100003 + i))
    return out


def single_ray_1d(npoints: int = 50, dx: float = 1.0e12, nTT: float = 1.0e3, nH2: float = 1.0e12,
                  temp: float = 4.5, turb: float = 0.0, dv: float = 0.0, nquads: int = 1,
                  bc: int = BC_CMB) -> RawModel:
    """The 1D single-ray models of the reference's analytic benchmarks
    (tests/benchmarks/analytic/all_constant_single_ray.py:17-67): points on the x
    axis, Delaunay neighbours in 1D (previous/next point, magritte/setup.py:60-70),
    the two end points as boundary, rays [-1,0,0] and [1,0,0]."""
    position = np.array([[i * dx, 0.0, 0.0] for i in range(npoints)])
    velocity = np.array([[i * dv, 0.0, 0.0] for i in range(npoints)])
    nbs = [1]
    n_nbs = [1]
    for p in range(1, npoints - 1):
        nbs.extend([p - 1, p + 1])
        n_nbs.append(2)
    nbs.append(npoints - 2)
    n_nbs.append(1)
    b2p = np.array([0, npoints - 1], dtype=np.uint32)
    direction = np.array([[-1.0, 0.0, 0.0], [1.0, 0.0, 0.0]])
    weight = np.array([0.5, 0.5])
    roots, wts = quadrature(nquads)
    abund = np.array([[nTT, nH2, 0.0] for _ in range(npoints)])
    return RawModel(
        name="single_ray_1d", dimension=1, position=position, velocity=velocity,
        neighbors=np.array(nbs, dtype=np.uint32), n_neighbors=np.array(n_nbs, dtype=np.uint32),
        boundary2point=b2p, boundary_condition=np.full(2, bc, np.int32),
        boundary_temperature=np.full(2, T_CMB), ray_direction=direction, ray_weight=weight,
        abundance=abund, temperature=np.full(npoints, temp), vturb2=np.full(npoints, (turb / CC) ** 2),
        linedata=[lamda_test_species()], quad_roots=[roots], quad_weights=[wts], nquads=nquads)


def rays_spherical_symmetry(nrays: int):
    """Ray directions and weights of a 1D spherically symmetric model, uniform variant of
    setup.set_rays_spherical_symmetry (magritte/setup.py:226-330): nrays/2 directions in
    the upper x-y half plane from +x to +y at equal angles, each weighted by the cosine
    difference of the half-way directions to its neighbours (the integral of sin theta
    over its sector), then their antipodes with the same weights; weights normalised."""
    h = nrays // 2
    nextra = h - 1
    Rx, Ry = [1.0], [0.0]
    step = 0.5 * np.pi / nextra
    for k in range(1, nextra):
        Rx.append(np.cos(k * step))
        Ry.append(np.sin(k * step))
    Rx.append(0.0)
    Ry.append(1.0)
    Wt = []
    for n in range(h):
        if n == 0:
            ux, uy = 0.5 * (Rx[n] + Rx[n + 1]), 0.5 * (Ry[n] + Ry[n + 1])
            lx, ly = Rx[0], Ry[0]
        elif n == h - 1:
            ux, uy = Rx[-1], Ry[-1]
            lx, ly = 0.5 * (Rx[n] + Rx[n - 1]), 0.5 * (Ry[n] + Ry[n - 1])
        else:
            ux, uy = 0.5 * (Rx[n] + Rx[n + 1]), 0.5 * (Ry[n] + Ry[n + 1])
            lx, ly = 0.5 * (Rx[n] + Rx[n - 1]), 0.5 * (Ry[n] + Ry[n - 1])
        Wt.append(lx / np.sqrt(lx ** 2 + ly ** 2) - ux / np.sqrt(ux ** 2 + uy ** 2))
    direction = np.array([[x, y, 0.0] for x, y in zip(Rx, Ry)] + [[-x, -y, -0.0] for x, y in zip(Rx, Ry)])
    weight = np.array(Wt + Wt)
    return direction, weight / weight.sum()


def spherical_1d(name: str, radius: np.ndarray, v_radial: np.ndarray, abundance: np.ndarray,
                 temperature: np.ndarray, vturb2: np.ndarray, nrays: int, nquads: int,
                 linedata: List[Linedata]) -> RawModel:
    """A 1D spherically symmetric model as the reference's 1D benchmarks build it: shells
    at ``radius`` (ascending) on the x axis with radial velocities, 1D Delaunay
    neighbours (magritte/setup.py:59-70), the innermost and outermost shells as CMB
    boundaries (setup.py:392-396) and the uniform spherical-symmetry rays."""
    P = len(radius)
    position = np.stack([radius, np.zeros(P), np.zeros(P)], axis=1)
    velocity = np.stack([v_radial, np.zeros(P), np.zeros(P)], axis=1)
    nbs = [1]
    n_nbs = [1]
    for p in range(1, P - 1):
        nbs.extend([p - 1, p + 1])
        n_nbs.append(2)
    nbs.append(P - 2)
    n_nbs.append(1)
    b2p = np.array([0, P - 1], dtype=np.uint32)
    direction, weight = rays_spherical_symmetry(nrays)
    roots, wts = quadrature(nquads)
    return RawModel(
        name=name, dimension=1, position=position, velocity=velocity,
        neighbors=np.array(nbs, dtype=np.uint32), n_neighbors=np.array(n_nbs, dtype=np.uint32),
        boundary2point=b2p, boundary_condition=np.full(2, BC_CMB, np.int32), boundary_temperature=np.full(2, T_CMB),
        ray_direction=direction, ray_weight=weight, abundance=abundance, temperature=temperature, vturb2=vturb2,
        linedata=linedata, quad_roots=[roots], quad_weights=[wts], nquads=nquads, spherical_symmetry=True)


def density_distribution_1d(kind: str = "a", npoints: int = 200, nrays: int = 50, nquads: int = 50) -> RawModel:
    """The reference's 1D density-distribution benchmark
    (tests/benchmarks/analytic/density_distribution_1D.py:17-87): shells log-spaced over
    1e13..7.8e16 m, n_H2 = 2e13 (r_in/r)^2 m^-3, X_mol 1e-8 (a) or 1e-6 (b), T = 20 K,
    v_turb = 150 m/s, no velocity, the 2-level 'test' species."""
    r_in, r_out, nH2_in = 1.0e13, 7.8e16, 2.0e13
    X_mol = {"a": 1.0e-8, "b": 1.0e-6}[kind]
    rs = np.logspace(np.log10(r_in), np.log10(r_out), npoints, endpoint=True)
    nH2 = nH2_in * (r_in / rs) ** 2
    abund = np.stack([X_mol * nH2, nH2, np.zeros(npoints)], axis=1)
    return spherical_1d(f"density_distribution_VZ{kind}_1D", rs, np.zeros(npoints), abund,
                        np.full(npoints, 20.0), np.full(npoints, (150.0 / CC) ** 2), nrays, nquads,
                        [lamda_test_species()])


def velocity_gradient_1d(npoints: int = 100, nrays: int = 100, nquads: int = 100) -> RawModel:
    """The reference's 1D constant-velocity-gradient benchmark
    (tests/benchmarks/analytic/constant_velocity_gradient_1D.py:14-73): shells at
    (i+1) 1e4 m moving outward at (i+1) 250 m/s, n_TT = 1e8, n_H2 = 1e12 m^-3, T = 45 K,
    no turbulence, the 2-level 'test' species."""
    dx, dv = 1.0e4, 2.5e2 / CC
    i = np.arange(npoints, dtype=np.float64)
    abund = np.tile(np.array([1.0e8, 1.0e12, 0.0]), (npoints, 1))
    return spherical_1d("constant_velocity_gradient_1D", (i + 1.0) * dx, (i + 1.0) * dv, abund,
                        np.full(npoints, 45.0), np.zeros(npoints), nrays, nquads, [lamda_test_species()])


def with_adaptive_rays(raw: RawModel, seed: int = 0, jitter: float = 0.5, identical: bool = False) -> RawModel:
    """A copy of ``raw`` with adaptive (per-point) ray directions, the layout
    Rays::use_adaptive_directions reads (rays.cpp:33-45): each point's rays are its own
    random rotation of the model's directions (antipodes stay paired), with weights
    jittered per point by up to ``jitter`` (the same for a ray and its antipode) and
    normalised per point.  ``identical``: every point gets the
    model's own rays and weights (the adaptive layout holding the shared rays)."""
    from dataclasses import replace
    from scipy.spatial.transform import Rotation

    P, R = raw.npoints, raw.nrays
    if identical:
        dirs = np.broadcast_to(raw.ray_direction, (P, R, 3)).copy()
        wts = np.broadcast_to(raw.ray_weight, (P, R)).copy()
    else:
        from .healpix import antipodes

        rng = np.random.default_rng(seed)
        rot = Rotation.random(P, random_state=rng)
        dirs = np.einsum("pij,rj->pri", rot.as_matrix(), raw.ray_direction)
        f = 1.0 + jitter * rng.uniform(-1.0, 1.0, size=(P, R))
        f = 0.5 * (f + f[:, antipodes(raw.ray_direction)])
        wts = raw.ray_weight[None, :] * f
        wts /= wts.sum(axis=1, keepdims=True)
    return replace(raw, name=raw.name + "_adaptive", ray_direction=np.ascontiguousarray(dirs[0]),
                   ray_weight=np.ascontiguousarray(wts[0]), adaptive_direction=dirs, adaptive_weight=wts)


def delaunay_neighbors(position: np.ndarray):
    """Neighbour CSR lists from a Delaunay triangulation of the points, as
    ``set_Delaunay_neighbor_lists`` builds them in 3D (magritte/setup.py:82-93)."""
    from scipy.spatial import Delaunay

    indptr, indices = Delaunay(position).vertex_neighbor_vertices
    n_nbs = np.diff(indptr).astype(np.uint32)
    return np.ascontiguousarray(indices, dtype=np.uint32), n_nbs


def van_zadelhoff_1(kind: str = "a", nshells: int = 20, nrays: int = 48, nquads: int = 11,
                    seed: int = 0) -> RawModel:
    """Problem 1 of the van Zadelhoff et al. (2002) non-LTE benchmark in the 3D form
    of the reference's tests/benchmarks/numeric/vanZadelhoff_1_3D_healpix.py:
    HEALPix shells (nside = 2 + s) at log-spaced radii 1e13..7.8e16 m, each shell
    randomly rotated (seeded), Delaunay neighbours, the inner and outer shells as CMB
    boundaries, n_H2 = 2e13 (r_in/r)^2 m^-3, X_mol = 1e-8 (a) or 1e-6 (b), T = 20 K,
    v_turb = 150 m/s, no velocity, the 2-level 'test' species, ``nrays`` HEALPix rays."""
    from scipy.spatial.transform import Rotation

    r_in, r_out, nH2_in = 1.0e13, 7.8e16, 2.0e13
    X_mol = {"a": 1.0e-8, "b": 1.0e-6}[kind]
    rng = np.random.default_rng(seed)
    r_shell = np.logspace(np.log10(r_in), np.log10(r_out), nshells, endpoint=True)
    n_in_shell = [healpix.nside2npix(2 + s) for s in range(nshells)]
    parts = []
    for s, (r, n) in enumerate(zip(r_shell, n_in_shell)):
        pos = r * healpix.pix2vec_ring(2 + s)
        pos = Rotation.random(random_state=rng).apply(pos)
        parts.append(pos)
    position = np.concatenate(parts)
    P = position.shape[0]
    rs = np.linalg.norm(position, axis=1)
    nH2 = nH2_in * (r_in / rs) ** 2
    nbs, n_nbs = delaunay_neighbors(position)
    b2p = np.concatenate([np.arange(n_in_shell[0]), np.arange(P - n_in_shell[-1], P)]).astype(np.uint32)
    direction, weight = healpix.uniform_rays(nrays)
    roots, wts = quadrature(nquads)
    abund = np.stack([X_mol * nH2, nH2, np.zeros(P)], axis=1)
    return RawModel(
        name=f"vanZadelhoff_1{kind}_3D", dimension=3, position=position, velocity=np.zeros((P, 3)),
        neighbors=nbs, n_neighbors=n_nbs, boundary2point=b2p, boundary_condition=np.full(len(b2p), BC_CMB, np.int32),
        boundary_temperature=np.full(len(b2p), T_CMB), ray_direction=direction, ray_weight=weight,
        abundance=abund, temperature=np.full(P, 20.0), vturb2=np.full(P, (150.0 / CC) ** 2),
        linedata=[lamda_test_species()], quad_roots=[roots], quad_weights=[wts], nquads=nquads)


def nlte_sphere(npoints: int = 500_000, nside: int = 4, nlev: int = 10, nquads: int = 21, seed: int = 0,
                r_in: float = 1.0e12, r_out: float = 1.0e14, nH2_in: float = 1.0e14, X_mol: float = 1.0e-6,
                v_out: float = 15.0e3, v_turb: float = 150.0, nside_in: int = 4, nside_out: int = 16) -> RawModel:
    """The non-LTE ALI workload: ``npoints`` interior points with number density
    ~ r^-2 (uniform in r) between r_in and r_out, HEALPix boundary shells (CMB) at
    r_in (nside_in) and r_out (nside_out), interior points on the convex hull also
    boundary points, Delaunay neighbours, 12 nside^2 rays, a 10-level linear rotor (B = 57.6 GHz, A_10 = 7.2e-8 /s, 28 amu) with one seeded
    collision partner (H2), n_H2 = nH2_in (r_in/r)^2, X_mol = 1e-6, outward wind
    ``v_out``, v_turb 150 m/s.  The workload does not fix the temperature; it is
    T = 100 K (r/r_in)^-0.4, at least 10 K."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(r_in, r_out, size=npoints)
    d = rng.normal(size=(npoints, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    inner = r_in * healpix.pix2vec_ring(nside_in)
    outer = r_out * healpix.pix2vec_ring(nside_out)
    position = np.concatenate([inner, r[:, None] * d, outer])
    P = position.shape[0]
    b2p = np.concatenate([np.arange(len(inner)), np.arange(P - len(outer), P)]).astype(np.uint32)
    # interior points just below r_out can stick out of the outer shell's flat faces and
    # so lie on the convex hull, where a ray leaves the Delaunay mesh: they are boundary
    # points too (appended after the shells)
    from scipy.spatial import ConvexHull

    hull = np.setdiff1d(ConvexHull(position).vertices, b2p)
    b2p = np.concatenate([b2p, np.sort(hull)]).astype(np.uint32)
    rs = np.linalg.norm(position, axis=1)
    nH2 = nH2_in * (r_in / rs) ** 2
    velocity = (v_out / CC) * position / rs[:, None]
    temperature = np.maximum(100.0 * (rs / r_in) ** -0.4, 10.0)
    nbs, n_nbs = delaunay_neighbors(position)
    direction, weight = healpix.uniform_rays(12 * nside * nside)
    ld = linear_rotor(nlev, 57.6e9, 7.2e-8, 28.0, num=0, collider=1, seed=seed)
    roots, wts = quadrature(nquads)
    abund = np.stack([X_mol * nH2, nH2], axis=1)
    return RawModel(
        name=f"nlte_sphere_{npoints}", dimension=3, position=position, velocity=velocity, neighbors=nbs,
        n_neighbors=n_nbs, boundary2point=b2p, boundary_condition=np.full(len(b2p), BC_CMB, np.int32),
        boundary_temperature=np.full(len(b2p), T_CMB), ray_direction=direction, ray_weight=weight,
        abundance=abund, temperature=temperature, vturb2=np.full(P, (v_turb / CC) ** 2),
        linedata=[ld], quad_roots=[roots], quad_weights=[wts], nquads=nquads)


def velocity_gradient_shells(nshells: int = 10, dx: float = 1.0e4, dv: float = 2.5e2, nTT: float = 1.0e8,
                             nH2: float = 1.0e12, temp: float = 45.0, turb: float = 0.0, nside: int = 1,
                             nquads: int = 10, seed: int = 0) -> RawModel:
    """The constant-velocity-gradient imaging benchmark in 3D (the reference's
    tests/benchmarks/analytic/constant_velocity_gradient_3D_new_imager.py): HEALPix
    shells (nside 2 + s) at radii dx, 2 dx, .., nshells dx, each randomly rotated
    (seeded), radial velocity s dv at shell s, Delaunay neighbours, inner and outer
    shells as CMB boundaries, the 2-level 'test' species in LTE at ``temp``."""
    from scipy.spatial.transform import Rotation

    rng = np.random.default_rng(seed)
    r_shell = np.linspace(dx, nshells * dx, nshells, endpoint=True)
    n_in_shell = [healpix.nside2npix(2 + s) for s in range(nshells)]
    pos_parts, vel_parts = [], []
    for s, (r, n) in enumerate(zip(r_shell, n_in_shell)):
        pos = r * healpix.pix2vec_ring(2 + s)
        pos = Rotation.random(random_state=rng).apply(pos)
        pos_parts.append(pos)
        vel_parts.append((r / dx) * (dv / CC) * pos / r)
    position = np.concatenate(pos_parts)
    velocity = np.concatenate(vel_parts)
    P = position.shape[0]
    nbs, n_nbs = delaunay_neighbors(position)
    b2p = np.concatenate([np.arange(n_in_shell[0]), np.arange(P - n_in_shell[-1], P)]).astype(np.uint32)
    direction, weight = healpix.uniform_rays(12 * nside * nside)
    roots, wts = quadrature(nquads)
    abund = np.array([[nTT, nH2, 0.0] for _ in range(P)])
    return RawModel(
        name="constant_velocity_gradient_3D", dimension=3, position=position, velocity=velocity, neighbors=nbs,
        n_neighbors=n_nbs, boundary2point=b2p, boundary_condition=np.full(len(b2p), BC_CMB, np.int32),
        boundary_temperature=np.full(len(b2p), T_CMB), ray_direction=direction, ray_weight=weight,
        abundance=abund, temperature=np.full(P, temp), vturb2=np.full(P, (turb / CC) ** 2),
        linedata=[lamda_test_species()], quad_roots=[roots], quad_weights=[wts], nquads=nquads)
