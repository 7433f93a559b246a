"""Seeded synthetic systems with the shapes of the KoMD benchmark workloads.

Reduced units map onto KoMD's units as sigma = 1 Angstrom, m = 1 u,
epsilon = 1 internal energy unit (u*A^2/ps^2) and time unit = 1 ps, so a
reduced configuration can be written straight into a KoMD checkpoint (the
checkpoint's eps column is already in internal units, see
IO/CheckpointIO.cpp:56 of the reference).

Every generator takes an explicit seed and returns plain numpy arrays; no
file or network access.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# Joule -> internal energy (u*A^2/ps^2), util/constants.h:20 of the reference
CONV_J_EI = 6.022140754e22
# reduced temperature -> Kelvin for sigma=1 A, m=1 u, eps=1 internal unit
T_STAR_TO_K = 1.66053906892e-27 * 1e4 / 1.380649e-23


@dataclass
class System:
    """Sites in molecule order (molecules are contiguous runs of sites)."""

    r: np.ndarray            # (n, 3) float64 positions
    v: np.ndarray            # (n, 3) float64 velocities
    m: np.ndarray            # (n,) masses
    eps: np.ndarray          # (n,) epsilon (internal units)
    sig: np.ndarray          # (n,) sigma
    mol_id: np.ndarray       # (n,) uint64 molecule ID per site
    low: np.ndarray          # (3,) domain low
    high: np.ndarray         # (3,) domain high
    bonds: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int64))
    angles: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int64))

    @property
    def n(self) -> int:
        return int(self.r.shape[0])

    @property
    def mol_off(self) -> np.ndarray:
        """CSR molecule offsets: consecutive sites with equal IDs form one molecule."""
        ids = self.mol_id
        starts = np.flatnonzero(np.concatenate(([True], ids[1:] != ids[:-1])))
        return np.concatenate((starts, [self.n])).astype(np.int64)

    @property
    def box(self) -> np.ndarray:
        return self.high - self.low


def fcc_positions(ncell: int | tuple, rho: float, offset: float = 0.25):
    """FCC lattice of ncell^3 unit cells at number density rho.

    Returns (r, L) with 4*ncell^3 sites; the lattice is shifted by
    offset*a so that no site sits on a cell boundary."""
    nc = np.array((ncell,) * 3 if np.isscalar(ncell) else ncell, dtype=np.int64)
    a = (4.0 / rho) ** (1.0 / 3.0)
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(np.arange(nc[0]), np.arange(nc[1]), np.arange(nc[2]), indexing="ij"), -1).reshape(-1, 3)
    # z slowest, x fastest, matching a nested z/y/x loop
    g = g[np.lexsort((g[:, 0], g[:, 1], g[:, 2]))]
    r = ((g[:, None, :] + basis[None, :, :]).reshape(-1, 3) + offset) * a
    return r, nc * a


def maxwell_boltzmann(n: int, t_star: float, m: np.ndarray, rng: np.random.Generator,
                      exact: bool = True) -> np.ndarray:
    """Seeded Maxwell-Boltzmann velocities with zero total momentum,
    optionally rescaled to exactly t_star."""
    v = rng.standard_normal((n, 3)) * np.sqrt(t_star / m)[:, None]
    v -= (m[:, None] * v).sum(0) / m.sum()
    if exact and n > 1:
        t_now = (m[:, None] * v * v).sum() / (3.0 * n)
        v *= np.sqrt(t_star / t_now)
    return v


def argon_fcc(ncell: int | tuple, rho: float = 0.8442, t_star: float = 0.722, seed: int = 1,
              jitter: float = 0.0) -> System:
    """Single-site LJ argon on an FCC lattice (the 4k plain-LJ, 32k LJ+ATM and 256k LJ+ATM workloads)."""
    rng = np.random.default_rng(seed)
    r, L = fcc_positions(ncell, rho)
    if jitter > 0:
        r = r + rng.normal(0.0, jitter, r.shape)
        r = np.mod(r, L)
    n = r.shape[0]
    m = np.ones(n)
    v = maxwell_boltzmann(n, t_star, m, rng)
    return System(r=r, v=v, m=m, eps=np.ones(n), sig=np.ones(n),
                  mol_id=np.arange(1, n + 1, dtype=np.uint64),
                  low=np.zeros(3), high=L.astype(np.float64))


def trimmed_fcc(n_target: int, rho: float, t_star: float, seed: int) -> System:
    """FCC box filled to >= n_target sites and then trimmed at random by seed
    (the batched-replica workload); the box keeps the filled volume scaled so
    that the trimmed system has density rho."""
    rng = np.random.default_rng(seed)
    k = int(np.ceil((n_target / 4.0) ** (1.0 / 3.0)))
    r, L = fcc_positions(k, rho * (4 * k ** 3) / n_target)
    keep = np.sort(rng.choice(r.shape[0], n_target, replace=False))
    r = r[keep]
    m = np.ones(n_target)
    v = maxwell_boltzmann(n_target, t_star, m, rng)
    return System(r=r, v=v, m=m, eps=np.ones(n_target), sig=np.ones(n_target),
                  mol_id=np.arange(1, n_target + 1, dtype=np.uint64), low=np.zeros(3), high=L)


def replica_specs(count: int, seed: int, n_min: int = 2000, n_max: int = 20000, rho=(0.70, 0.90),
                  t_star=(0.6, 1.5)) -> list:
    """(lattice seed, atoms, rho*, T*) of each replica of the batched-replica
    workload: atom counts uniform in [n_min, n_max], rho* and T* uniform in
    their ranges, all drawn from one seeded generator (build each with
    trimmed_fcc)."""
    rng = np.random.default_rng(seed)
    return [(int(rng.integers(1 << 30)), int(rng.integers(n_min, n_max + 1)), float(rng.uniform(*rho)),
             float(rng.uniform(*t_star))) for _ in range(count)]


def _rotation(rng: np.random.Generator) -> np.ndarray:
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def triatomic_sc(n_mol_side: int, rho_site: float = 0.8, t_star: float = 1.0, seed: int = 3,
                 r0: float = 1.0, theta0_deg: float = 109.47) -> System:
    """Flexible 3-site molecules (bond r0, angle theta0) centred on the sites
    of a simple-cubic lattice with a random orientation each (the 300k-site multi-site workload).
    Topology: bonds (0,1), (1,2); angle (0,1,2) with site 1 the vertex."""
    rng = np.random.default_rng(seed)
    n_mol = n_mol_side ** 3
    L = (3 * n_mol / rho_site) ** (1.0 / 3.0)
    a = L / n_mol_side
    g = np.stack(np.meshgrid(*(np.arange(n_mol_side),) * 3, indexing="ij"), -1).reshape(-1, 3)
    g = g[np.lexsort((g[:, 0], g[:, 1], g[:, 2]))]
    centres = (g + 0.5) * a
    th = np.deg2rad(theta0_deg)
    body = np.array([[r0 * np.sin(th / 2), r0 * np.cos(th / 2), 0.0], [0, 0, 0],
                     [-r0 * np.sin(th / 2), r0 * np.cos(th / 2), 0.0]])
    body -= body.mean(0)
    r = np.empty((3 * n_mol, 3))
    for k in range(n_mol):
        r[3 * k:3 * k + 3] = centres[k] + body @ _rotation(rng).T
    n = 3 * n_mol
    m = np.ones(n)
    v = maxwell_boltzmann(n, t_star, m, rng)
    mol_id = np.repeat(np.arange(1, n_mol + 1, dtype=np.uint64), 3)
    base = 3 * np.arange(n_mol)
    bonds = np.concatenate([np.stack([base, base + 1], 1), np.stack([base + 1, base + 2], 1)]).astype(np.int64)
    angles = np.stack([base, base + 1, base + 2], 1).astype(np.int64)
    return System(r=r, v=v, m=m, eps=np.ones(n), sig=np.ones(n), mol_id=mol_id,
                  low=np.zeros(3), high=np.full(3, L), bonds=bonds, angles=angles)


def triatomic_count(n_mol: int, rho_site: float = 0.8, t_star: float = 1.0, seed: int = 3, r0: float = 1.0,
                    theta0_deg: float = 109.47, aligned: bool = False) -> System:
    """Exactly n_mol flexible 3-site molecules at site density rho_site, centred
    on a seeded random n_mol of the points of the smallest simple-cubic lattice
    with at least n_mol points.  Orientations: random per molecule, or
    (aligned) one orientation for all, the seeded candidate (of 4000) that keeps
    sites of different molecules farthest apart -- at rho_site 0.8 random
    orientations put sites of neighbouring molecules within a fraction of sigma."""
    rng = np.random.default_rng(seed)
    side = int(np.ceil(n_mol ** (1.0 / 3.0) - 1e-9))
    while side ** 3 < n_mol:
        side += 1
    L = (3 * n_mol / rho_site) ** (1.0 / 3.0)
    a = L / side
    g = np.stack(np.meshgrid(*(np.arange(side),) * 3, indexing="ij"), -1).reshape(-1, 3)
    g = g[np.lexsort((g[:, 0], g[:, 1], g[:, 2]))]
    keep = np.sort(rng.choice(side ** 3, n_mol, replace=False))
    centres = (g[keep] + 0.5) * a
    th = np.deg2rad(theta0_deg)
    body = np.array([[r0 * np.sin(th / 2), r0 * np.cos(th / 2), 0.0], [0, 0, 0],
                     [-r0 * np.sin(th / 2), r0 * np.cos(th / 2), 0.0]])
    body -= body.mean(0)
    if aligned:
        shifts = np.array([[i, j, k] for i in range(-2, 3) for j in range(-2, 3) for k in range(-2, 3)
                           if (i, j, k) != (0, 0, 0)], float) * a
        best, rot = -1.0, None
        for _ in range(4000):
            R = _rotation(rng)
            b = body @ R.T
            d = (shifts[:, None, None, :] + b[None, None, :, :] - b[None, :, None, :]).reshape(-1, 3)
            dmin = float(np.sqrt((d * d).sum(1)).min())
            if dmin > best:
                best, rot = dmin, R
        r = (centres[:, None, :] + (body @ rot.T)[None, :, :]).reshape(-1, 3)
    else:
        r = np.empty((3 * n_mol, 3))
        for k in range(n_mol):
            r[3 * k:3 * k + 3] = centres[k] + body @ _rotation(rng).T
    n = 3 * n_mol
    m = np.ones(n)
    v = maxwell_boltzmann(n, t_star, m, rng)
    v -= (v * m[:, None]).sum(0) / m.sum()   # no net momentum
    base = 3 * np.arange(n_mol)
    bonds = np.concatenate([np.stack([base, base + 1], 1), np.stack([base + 1, base + 2], 1)]).astype(np.int64)
    angles = np.stack([base, base + 1, base + 2], 1).astype(np.int64)
    return System(r=r, v=v, m=m, eps=np.ones(n), sig=np.ones(n),
                  mol_id=np.repeat(np.arange(1, n_mol + 1, dtype=np.uint64), 3), low=np.zeros(3),
                  high=np.full(3, L), bonds=bonds, angles=angles)


def nu_star_to_energy_3b(nu_star: float) -> float:
    """Reduced ATM coefficient -> the input file's energy_3b (J*nm^9), the
    inverse of ATM::ATM's conversion (potentials/ATM.cpp:11-14)."""
    return nu_star / (1e9 * CONV_J_EI)


def energy_3b_to_nu(energy_3b: float) -> float:
    """Input energy_3b -> internal nu, as ATM::ATM does."""
    return energy_3b * 1e9 * (6.022140754 * 10.0 ** 22)
