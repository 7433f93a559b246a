"""The labelled switched-cutoff option (komd_config::switch_width > 0).

The reference truncates LJ and ATM without a shift (potentials/LJ12_6.cpp:28,
potentials/ATM.cpp:43): every pair or triplet that crosses a cutoff makes the
total energy jump, and NVE runs drift.  The option multiplies each LJ pair
energy by S(r^2) and each ATM triplet energy by the product of S over its
three sides, S the C1 smoothstep of the squared distance over the last
`switch_width` below each cutoff, with forces the exact gradients.  It is off
by default (the engine then reproduces the reference, as the parity tests
show), and here the engine's switched forces and energies are compared with
the oracle's switched restatement, which is itself checked against central
differences of its energy.
"""
import numpy as np
import pytest

FP32_FORCE_RMSE = 1e-5


def rel_rmse(a, b):
    return float(np.sqrt(((a - b) ** 2).sum(1).mean()) / np.sqrt((b ** 2).sum(1).mean()))


def _cfg(s, cell, width, skin=0.3):
    from komd_gb300 import gpu
    return gpu.make_config(s.low, s.high, cell, cutoff=2.5, cutoff_3b=2.0, nu=0.073, dt=0.005,
                           terms=gpu.TERM_LJ | gpu.TERM_ATM, precision=gpu.FP32, atm_sign=gpu.ATM_SIGN_PHYSICAL,
                           atm_enum=gpu.ATM_ENUM_FULL, virial_mode=gpu.VIRIAL_CORRECT, skin=skin,
                           switch_width=width)


def _oracle(oracle_lib, s, r, v, cell, width):
    from komd_gb300 import lattice
    at = lattice.System(r=r, v=v, m=s.m, eps=s.eps, sig=s.sig, mol_id=s.mol_id, low=s.low, high=s.high)
    sim = oracle_lib.OracleSim(at, cell, 2.5, nu=0.073, cutoff_atm=2.0, atm=True, atm_mode="full",
                               atm_sign=oracle_lib.ATM_SIGN_PHYSICAL, virial_mode=oracle_lib.VIRIAL_CORRECT,
                               switch_width=width)
    sim.update_container()
    sim.forces(listless=True)
    return sim


def test_switch_is_off_by_default_and_validated():
    """CPU: the default configuration keeps the truncated potentials, and the
    option is refused outside the path that implements it."""
    import ctypes
    from komd_gb300 import gpu
    cfg = gpu.make_config([0, 0, 0], [20, 20, 20], 2.8, cutoff=2.5)
    assert cfg.switch_width == 0.0
    lib = gpu.load()
    h = ctypes.c_void_p()
    bad = gpu.make_config([0, 0, 0], [20, 20, 20], 2.8, cutoff=2.5, switch_width=0.3)   # skin 0
    assert lib.komd_gpu_create(ctypes.byref(bad), 0, ctypes.byref(h)) == 1
    assert b"switch_width" in lib.komd_gpu_last_error()
    bad = gpu.make_config([0, 0, 0], [20, 20, 20], 2.9, cutoff=2.5, terms=gpu.TERM_LJ | gpu.TERM_LIMIT, skin=0.3,
                          virial_mode=gpu.VIRIAL_CORRECT, switch_width=0.3)
    assert lib.komd_gpu_create(ctypes.byref(bad), 0, ctypes.byref(h)) == 1
    assert b"switch_width" in lib.komd_gpu_last_error()


def test_oracle_switched_forces_are_minus_gradient(oracle_lib):
    """CPU: the oracle's switched forces are minus the gradient of its switched
    energy (LJ + ATM), by central differences."""
    from komd_gb300 import lattice
    s = lattice.argon_fcc(4, rho=0.8442, t_star=0.722, seed=5, jitter=0.08)
    L = float((s.high - s.low)[0])
    cell = L / np.floor(L / 2.5)

    def ef(r):
        sim = _oracle(oracle_lib, s, r, s.v, cell, 0.3)
        return sim.lj_out.u_total + sim.atm_out.energy, sim.f.copy()

    _, f0 = ef(s.r.copy())
    h = 1e-6
    for i, d in ((0, 0), (5, 1), (17, 2), (100, 0), (200, 2)):
        rp, rm = s.r.copy(), s.r.copy()
        rp[i, d] += h
        rm[i, d] -= h
        fd = -(ef(rp)[0] - ef(rm)[0]) / (2 * h)
        assert abs(f0[i, d] - fd) <= 1e-6 * max(1.0, abs(fd)), (i, d, f0[i, d], fd)


@pytest.mark.gpu
def test_switched_forces_and_energies_match_oracle(oracle_lib):
    """GPU: 4,000 argon atoms on the Verlet path with switch_width 0.3: the
    half-list pass's forces and the measure passes' energies equal the oracle's
    switched restatement, at the start and after 100 steps."""
    from komd_gb300 import gpu, lattice
    s = lattice.argon_fcc(10, rho=0.8442, t_star=0.9, seed=71, jitter=0.05)
    L = float((s.high - s.low)[0])
    cell = L / np.floor(L / 2.8)
    g = gpu.GpuSystem(s, _cfg(s, cell, 0.3))
    g.update_container()
    g.forces()
    for steps in (0, 100):
        if steps:
            g.step(steps)
        r, v, f = g.download()
        obs = g.measure(gpu.MEASURE_ENERGY | gpu.MEASURE_PRESSURE)
        _, _, f_meas = g.download()
        sim = _oracle(oracle_lib, s, r, v, cell, 0.3)
        assert rel_rmse(f, sim.f) < FP32_FORCE_RMSE
        assert rel_rmse(f_meas, sim.f) < FP32_FORCE_RMSE   # the measure passes switch their forces too
        assert obs["u_lj"] == pytest.approx(sim.lj_out.u_total, rel=1e-5)
        assert obs["u_atm"] == pytest.approx(sim.atm_out.energy, rel=1e-5)
        truncated = _oracle(oracle_lib, s, r, v, cell, 0.0)
        assert rel_rmse(f, truncated.f) > 1e-3   # the option does change the forces
    g.close()


@pytest.mark.gpu
def test_switch_with_learned_term_switches_the_lj_part(oracle_lib):
    """With the learned three-body term the option switches the LJ pair
    energy: the forces of the learned form with and without the switch
    differ by exactly what the switch changes in the LJ forces (the oracle's
    switched and truncated LJ at the same positions), and the LJ energy
    matches the oracle's switched LJ."""
    from komd_gb300 import gpu, lattice, surrogate
    s = lattice.argon_fcc(10, rho=0.8442, t_star=1.0, seed=71, jitter=0.05)    # 4000 sites, L = 16.8
    cell = 2.8
    terms = gpu.TERM_LJ | gpu.TERM_ATM | gpu.TERM_ATM_SURROGATE
    forces, u_lj = {}, {}
    model = None
    for width in (0.0, 0.3):
        cfg = surrogate.physics_config(s, cell, skin=0.3, terms=terms)
        cfg.switch_width = width
        g = gpu.GpuSystem(s, cfg)
        g.update_container()
        g.forces()
        if model is None:
            x, e3, _ = g.surrogate_sample()
            model = dict(params=surrogate.init_params(5), fmean=x.mean(0).astype(np.float32),
                         fstd=(x.std(0) + 1e-6).astype(np.float32), e_scale=float(e3.std()), e_shift=float(e3.mean()))
        g.surrogate_load(model, probe_every=0)
        g.update_container()
        g.forces()
        _, _, forces[width] = g.download()
        u_lj[width] = g.measure(gpu.MEASURE_ENERGY)["u_lj"]
        g.close()
    lj = {}
    for width in (0.0, 0.3):
        at = lattice.System(r=s.r, v=s.v, m=s.m, eps=s.eps, sig=s.sig, mol_id=s.mol_id, low=s.low, high=s.high)
        sim = oracle_lib.OracleSim(at, cell, 2.5, nu=0.073, cutoff_atm=2.0, atm=False,
                                   virial_mode=oracle_lib.VIRIAL_CORRECT, switch_width=width)
        sim.update_container()
        sim.forces(listless=True)
        lj[width] = (sim.f.copy(), sim.lj_out.u_total)
    d_gpu = forces[0.3] - forces[0.0]
    d_ref = lj[0.3][0] - lj[0.0][0]
    scale = np.sqrt((lj[0.0][0] ** 2).sum(1).mean())
    assert np.sqrt((d_ref ** 2).sum(1).mean()) > 1e-3 * scale        # the switch changes the LJ forces
    assert np.sqrt(((d_gpu - d_ref) ** 2).sum(1).mean()) < 1e-5 * scale
    assert u_lj[0.3] == pytest.approx(lj[0.3][1], rel=1e-5)
