"""The multi-site workload's starting configuration, on the CPU (oracle only).

The workload places flexible 3-site molecules (bond 1.0, angle 109.47 deg) on
a simple-cubic lattice at site density 0.8 with "a randomly rotated" lattice.
With an independent random orientation per molecule, sites of neighbouring
molecules overlap at this density (the lattice spacing is 1.55 sigma, the
molecule spans 1.6 sigma): most force components start above the
reference's Limit cap (20 eps/sigma, the functor main.cpp:57-66 always adds),
and under that cap the molecules tear apart, because Limit caps the bond and
angle forces as well.  One seeded orientation for all molecules (the
candidate that keeps sites of different molecules farthest apart) starts
without overlaps and, with no cap, keeps the molecules intact.  The GPU runs
of this workload use that orientation; these tests record why, at the same
density on a smaller box, with the oracle's reference-semantics forces.
"""
import os

import numpy as np
import pytest

N_MOL = 4096
RHO_SITE = 0.8
STEPS = 100
DT = 0.002


@pytest.fixture(autouse=True)
def _all_cores(oracle_lib):
    """The oracle on every core (another test may have left it on one)."""
    keep = oracle_lib.num_threads()
    oracle_lib.set_threads(os.cpu_count() or 1)
    yield
    oracle_lib.set_threads(keep)


def _setup(oracle_lib, aligned, limit):
    from komd_gb300 import lattice
    s = lattice.triatomic_count(N_MOL, rho_site=RHO_SITE, t_star=1.0, seed=31, aligned=aligned)
    L = float((s.high - s.low)[0])
    cell = L / np.floor(L / 4.2)   # cutoff + the molecule's diameter: every site pair inside the cutoff
    bonded = dict(bonds=s.bonds, angles=s.angles, kb=1000.0, r0=1.0, ka=100.0, theta0=np.deg2rad(109.47))
    sim = oracle_lib.OracleSim(s, cell, 2.5, dt=DT, limit=limit, bonded=bonded)
    sim.update_container()
    sim.forces(listless=True)
    return s, sim


def _min_intermolecular(s):
    from scipy.spatial import cKDTree
    L = (s.high - s.low).astype(np.float64)
    x = np.mod(s.r - s.low, L)
    pairs = cKDTree(x, boxsize=L).query_pairs(1.0, output_type="ndarray")
    pairs = pairs[s.mol_id[pairs[:, 0]] != s.mol_id[pairs[:, 1]]]
    d = x[pairs[:, 0]] - x[pairs[:, 1]]
    d -= L * np.round(d / L)
    return float(np.sqrt((d * d).sum(1)).min()) if len(d) else 1.0


def _bond_range(s, r):
    b = np.linalg.norm(r[s.bonds[:, 0]] - r[s.bonds[:, 1]], axis=1)
    return float(b.min()), float(b.max())


def test_random_orientations_overlap_and_tear(oracle_lib):
    s, sim = _setup(oracle_lib, aligned=False, limit=20.0)
    assert _min_intermolecular(s) < 0.3
    assert (np.abs(sim.f) == 20.0).mean() > 0.5       # most components start at the cap
    _, raw = _setup(oracle_lib, aligned=False, limit=1e30)
    assert np.abs(raw.f).max() > 1e8                  # uncapped: one step of dt 0.002 moves a site by > 1e2 sigma
    for k in range(STEPS):
        sim.step(listless=True)
    lo, hi = _bond_range(s, sim.r)
    assert hi > 1.5 or lo < 0.5, (lo, hi)             # the capped bond forces do not hold the molecules


def test_aligned_orientation_starts_clear_and_holds(oracle_lib):
    """The orientation the GPU runs use, with no cap (as they run)."""
    s, sim = _setup(oracle_lib, aligned=True, limit=1e30)
    assert _min_intermolecular(s) > 0.8
    assert np.abs(sim.f).max() < 1e3
    for k in range(STEPS):
        sim.step(listless=True)
    lo, hi = _bond_range(s, sim.r)
    assert 0.8 < lo and hi < 1.2, (lo, hi)
