"""Edge cases of the engine through the C ABI: empty and tiny systems,
crowded cells (more than 32 and more than 64 sites per cell, which take the
Verlet build's two-home form and several staging rounds of the per-step pair
kernel), and list capacities that grow when the density is far from uniform.
Bars as in test_gpu_parity: FP64 forces to 1e-12, FP32 forces to a relative
RMSE of 1e-5 against the FP64 oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP32_FORCE_RMSE = 1e-5


def rel_rmse(a, b):
    return float(np.sqrt(((a - b) ** 2).sum(1).mean()) / np.sqrt((b ** 2).sum(1).mean()))


def _sites(r, v, L):
    from komd_gb300 import lattice
    r = np.asarray(r, np.float64).reshape(-1, 3)
    n = r.shape[0]
    return lattice.System(r=r, v=np.asarray(v, np.float64).reshape(-1, 3), m=np.ones(n), eps=np.ones(n),
                          sig=np.ones(n), mol_id=np.arange(1, n + 1, dtype=np.uint64), low=np.zeros(3),
                          high=np.asarray(L, np.float64))


def _physics(s, cell, skin, precision=None):
    from komd_gb300 import gpu
    return gpu.make_config(s.low, s.high, cell, cutoff=2.5, cutoff_3b=2.0, nu=0.073, dt=0.005,
                           terms=gpu.TERM_LJ | gpu.TERM_ATM, atm_sign=gpu.ATM_SIGN_PHYSICAL,
                           atm_enum=gpu.ATM_ENUM_FULL, virial_mode=gpu.VIRIAL_CORRECT, skin=skin,
                           precision=gpu.FP32 if precision is None else precision)


def _oracle_forces(oracle_lib, s, cell):
    sim = oracle_lib.OracleSim(s, cell, 2.5, nu=0.073, cutoff_atm=2.0, atm=True, atm_mode="full",
                               atm_sign=oracle_lib.ATM_SIGN_PHYSICAL, virial_mode=oracle_lib.VIRIAL_CORRECT)
    sim.update_container()
    sim.forces()
    return np.array(sim.f)


def test_empty_system_is_rejected():
    """No sites: the upload fails with an argument error (no launch runs)."""
    from komd_gb300 import gpu
    s = _sites(np.zeros((0, 3)), np.zeros((0, 3)), [9.0, 9.0, 9.0])
    with pytest.raises(gpu.KomdError) as err:
        gpu.GpuSystem(s, _physics(s, 3.0, 0.0))
    assert gpu.STATUS[err.value.code] == "ERR_ARG"


def test_one_site_moves_freely():
    """A lone site has no partners: zero force, and a step is the free drift
    r + v dt (FP64, exact) on both the per-step and the Verlet path."""
    from komd_gb300 import gpu
    for skin in (0.0, 0.3):
        s = _sites([[4.0, 4.5, 5.0]], [[0.5, -0.25, 0.125]], [9.0, 9.0, 9.0])
        g = gpu.GpuSystem(s, _physics(s, 3.0, skin))
        g.update_container()
        g.forces()
        _, _, f = g.download()
        assert np.array_equal(f, np.zeros((1, 3)))
        g.step(4)
        r, v, f = g.download()
        assert np.array_equal(v, s.v)
        expect = s.r.copy()
        for _ in range(4):
            expect = expect + s.v * 0.005
        assert np.array_equal(r, expect)
        g.close()


@pytest.mark.parametrize("image", [False, True])
def test_two_sites_follow_the_lj_formula(image):
    """Two sites 1.1 sigma apart (directly, or across the periodic boundary):
    F = 24 eps (2 (s/r)^12 - (s/r)^6) / r along the separation, equal and
    opposite (FP64 mode, one pair, no triplet)."""
    from komd_gb300 import gpu
    L = 9.0
    x0, x1 = (0.3, L - 0.8) if image else (4.0, 5.1)
    s = _sites([[x0, 4.0, 4.0], [x1, 4.0, 4.0]], np.zeros((2, 3)), [L, L, L])
    g = gpu.GpuSystem(s, _physics(s, 3.0, 0.0, precision=gpu.FP64))
    g.update_container()
    g.forces()
    _, _, f = g.download()
    r = 1.1
    mag = 24.0 * (2.0 * r ** -12 - r ** -6) / r
    sign = -1.0 if image else 1.0   # force on site 0 along +x is repulsive away from site 1
    expect = np.array([[-sign * mag, 0.0, 0.0], [sign * mag, 0.0, 0.0]])
    np.testing.assert_allclose(f, expect, rtol=1e-12, atol=1e-12)
    g.close()


def test_crowded_cells_match_oracle(oracle_lib):
    """Three cells per dimension of edge 4.48 hold about 76 sites each: the
    Verlet build runs its two-home form (two passes for cells of more than 64
    sites), and the per-step pair kernel stages each 27-cell neighbourhood
    (about 2,000 sites) in several rounds.  Both paths give the oracle's
    forces, and the Verlet path's trajectory stays on the per-step path's."""
    from komd_gb300 import gpu, lattice
    s = lattice.argon_fcc(8, rho=0.8442, t_star=0.722, seed=61, jitter=0.05)   # 2048 sites, L = 13.44
    L = float(s.high[0])
    cell = L / 3.0
    ref = _oracle_forces(oracle_lib, s, cell)
    a = gpu.GpuSystem(s, _physics(s, cell, 0.3))
    b = gpu.GpuSystem(s, _physics(s, cell, 0.0))
    for g in (a, b):
        g.update_container()
        g.forces()
        _, _, f = g.download()
        assert rel_rmse(f, ref) < FP32_FORCE_RMSE
    a.step(40)
    b.step(40)
    ra, _, fa = a.download()
    rb, _, fb = b.download()
    assert np.abs(ra - rb).max() < 1e-4
    assert rel_rmse(fa, fb) < 1e-4
    a.close()
    b.close()


def test_list_capacity_grows_for_a_cluster(oracle_lib):
    """All sites packed in a quarter of the box (liquid density there, empty
    elsewhere): the Verlet row capacity sized from the mean density (64) is
    below the cluster's rows (about 80), so the first rebuild overflows and the
    engine grows the list and rebuilds.  The forces are then the oracle's, and
    the steps that follow run."""
    from komd_gb300 import gpu, lattice
    c = lattice.argon_fcc(6, rho=0.8442, t_star=0.722, seed=62, jitter=0.05)   # 864 sites, L = 10.08
    L = float(c.high[0])
    s = _sites(c.r, c.v, [4.0 * L + 3.0, L, L])   # a gap wider than the cutoff on both sides in x
    s.r[:, 0] += 1.5
    cell = float(s.high[1]) / 3.0
    g = gpu.GpuSystem(s, _physics(s, cell, 0.3))
    g.update_container()
    g.forces()
    _, _, f = g.download()
    assert rel_rmse(f, _oracle_forces(oracle_lib, s, cell)) < FP32_FORCE_RMSE
    g.step(20)
    g.close()
