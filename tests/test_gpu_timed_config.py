"""The benchmark's timed configuration itself against the FP64 oracle.

The benchmark times LJ + ATM argon at 256,000 atoms on the Verlet path with
the skin and cell edge its autotuner picks (skin 0.4 on cells of 67.184 / 23
= 2.921, or 0.6 on cells of 67.184 / 21 = 3.199, in recorded runs), FULL triplets
with F = -grad V, FP32 pair and triplet arithmetic and FP64 integration,
after 400 equilibration steps in which the FCC lattice melts.  Here the same
system and configuration run through komd_gpu_step (the step graph, with its
on-demand list rebuilds), and at the reached state the forces, the triplet
count and the pair count are compared with the oracle evaluated at the
engine's positions.  Counts are decided by FP32 cutoff tests on the GPU and by
FP64 ones in the oracle: they may differ by the pairs and triplets with a
side within 2e-5 of the cutoff in squared length, and by no more.

A second case runs the two-home form of the Verlet list build (chosen where
the cells hold more than 26 sites on average) on the 32,000-atom workload.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP32_FORCE_RMSE = 1e-5


def rel_rmse(a, b):
    return float(np.sqrt(((a - b) ** 2).sum(1).mean()) / np.sqrt((b ** 2).sum(1).mean()))


def _cfg(s, cell, skin):
    from komd_gb300 import gpu
    return gpu.make_config(s.low, s.high, cell, cutoff=2.5, cutoff_3b=2.0, nu=0.073, dt=0.005,
                           terms=gpu.TERM_LJ | gpu.TERM_ATM, precision=gpu.FP32, atm_sign=gpu.ATM_SIGN_PHYSICAL,
                           atm_enum=gpu.ATM_ENUM_FULL, virial_mode=gpu.VIRIAL_CORRECT, skin=skin)


def _oracle_at(oracle_lib, s, r, v, cell):
    from komd_gb300 import lattice
    at = lattice.System(r=r, v=v, m=s.m, eps=s.eps, sig=s.sig, mol_id=s.mol_id, low=s.low, high=s.high)
    sim = oracle_lib.OracleSim(at, cell, 2.5, nu=0.073, cutoff_atm=2.0, atm=True, atm_mode="full",
                               atm_sign=oracle_lib.ATM_SIGN_PHYSICAL, virial_mode=oracle_lib.VIRIAL_CORRECT)
    sim.update_container()
    sim.forces()
    return sim


def _pair_counts(r, box, rc, band):
    """Unique pairs with |r_ij| <= rc (minimum image, FP64), and the pairs whose
    squared distance lies within `band` of rc^2: an FP32 cutoff test may
    decide those either way."""
    from scipy.spatial import cKDTree
    x = np.mod(r, box)
    t = cKDTree(x, boxsize=box)
    n = len(x)
    inside = (t.count_neighbors(t, rc) - n) // 2
    hi = (t.count_neighbors(t, np.sqrt(rc * rc + band)) - n) // 2
    lo = (t.count_neighbors(t, np.sqrt(rc * rc - band)) - n) // 2
    return int(inside), int(hi - lo)


def _ambiguous_triplets(r, box, rc, band):
    """An upper bound on the triplets (all sides <= rc) that an FP32 cutoff
    test may count differently from FP64: those with a side whose squared
    length lies within `band` of rc^2."""
    from scipy.spatial import cKDTree
    x = np.mod(r, box)
    t = cKDTree(x, boxsize=box)
    r_hi = np.sqrt(rc * rc + band)
    pairs = t.query_pairs(r_hi, output_type="ndarray")
    d = x[pairs[:, 0]] - x[pairs[:, 1]]
    d -= box * np.round(d / box)
    q = (d * d).sum(1)
    near = pairs[np.abs(q - rc * rc) <= band]
    count = 0
    for i, j in near:
        common = set(t.query_ball_point(x[i], r_hi)) & set(t.query_ball_point(x[j], r_hi))
        count += len(common - {int(i), int(j)})
    return count


@pytest.mark.parametrize("skin,ncells", [(0.4, 23), (0.6, 21)])
def test_timed_256k_state_matches_oracle(oracle_lib, skin, ncells):
    """The autotuner's leading shapes: skin 0.4 on cells of 2.921 (one home
    site per lane in the list build) and skin 0.6 on cells of 3.199 (27.6
    sites per cell: the two-home build)."""
    from komd_gb300 import gpu, lattice
    s = lattice.argon_fcc(40, rho=0.8442, t_star=0.722, seed=1)   # the benchmark's system (rank 0)
    L = float((s.high - s.low)[0])
    cell = L / ncells                                               # >= cutoff 2.5 + skin
    assert cell >= 2.5 + skin
    g = gpu.GpuSystem(s, _cfg(s, cell, skin))
    g.update_container()
    g.forces()
    g.step(400)                                                     # the benchmark's equilibration
    r, v, f = g.download()
    obs = g.measure(gpu.MEASURE_ENERGY | gpu.MEASURE_PRESSURE)
    g.close()
    sim = _oracle_at(oracle_lib, s, r, v, cell)
    err = rel_rmse(f, sim.f)
    assert err < FP32_FORCE_RMSE, f"force rel RMSE {err:.3e}"
    # the melted state the benchmark times, not the lattice (5.12M triplets)
    assert obs["triplets"] > 9.0e6
    box = (s.high - s.low).astype(np.float64)
    amb3 = _ambiguous_triplets(r - s.low, box, 2.0, 2e-5)
    assert abs(obs["triplets"] - sim.atm_out.triplets) <= amb3, (obs["triplets"], sim.atm_out.triplets, amb3)
    pairs, ambiguous = _pair_counts(r - s.low, box, 2.5, 2e-5)
    assert abs(obs["pairs_in_cutoff"] - pairs) <= ambiguous, (obs["pairs_in_cutoff"], pairs, ambiguous)
    assert obs["u_lj"] == pytest.approx(sim.lj_out.u_total, rel=1e-5)
    assert obs["u_atm"] == pytest.approx(sim.atm_out.energy, rel=1e-5)
    # Newton's third law of the once-per-pair / once-per-triplet sums
    assert np.abs(f.sum(0)).max() < 1e-3 * np.sqrt(s.n) * np.abs(f).mean()


def test_two_home_list_build_32k(oracle_lib):
    """Cells of 3.36 sigma hold about 32 sites at rho* 0.8442: the Verlet list
    build serves two home sites per lane.  After 100 steps with on-demand
    rebuilds the forces match the oracle and the per-step-cell path."""
    from komd_gb300 import gpu, lattice
    s = lattice.argon_fcc(20, rho=0.8442, t_star=0.722, seed=61, jitter=0.03)
    L = float((s.high - s.low)[0])
    cell = L / 10
    assert 0.8442 * cell ** 3 > 26.0
    g = gpu.GpuSystem(s, _cfg(s, cell, 0.5))
    g.update_container()
    g.forces()
    g.step(100)
    r, v, f = g.download()
    obs = g.measure(gpu.MEASURE_ENERGY)
    g.close()
    sim = _oracle_at(oracle_lib, s, r, v, cell)
    assert rel_rmse(f, sim.f) < FP32_FORCE_RMSE
    amb3 = _ambiguous_triplets(r - s.low, (s.high - s.low).astype(np.float64), 2.0, 2e-5)
    assert abs(obs["triplets"] - sim.atm_out.triplets) <= amb3, (obs["triplets"], sim.atm_out.triplets, amb3)
    at = lattice.System(r=r, v=v, m=s.m, eps=s.eps, sig=s.sig, mol_id=s.mol_id, low=s.low, high=s.high)
    b = gpu.GpuSystem(at, _cfg(at, cell, 0.0))
    b.update_container()
    b.forces()
    _, _, fb = b.download()
    b.close()
    assert rel_rmse(f, fb) < 2e-6
