"""CUDA engine vs the reference (golden fixtures) and the CPU oracle, through
the C ABI (komd_gb300/_build/libkomd_gpu.so via ctypes).

Bars (from the engine's contract):
  * cell lists (incl. halo copies) and neighbour counts: bit-exact;
  * FP32 pair/triplet forces: relative RMSE <= 1e-5 against the reference's FP64;
  * FP64 mode: relative RMSE <= 1e-12;
  * temperature, potential energy, pressure: FP64 reductions, tolerances below;
  * RDF histogram counts: bit-exact for the same configuration.
"""
import numpy as np
import pytest

from conftest import CASES, case_system, load_case

pytestmark = pytest.mark.gpu

FP32_FORCE_RMSE = 1e-5
FP64_FORCE_RMSE = 1e-12


def rel_rmse(a, b):
    return float(np.sqrt(((a - b) ** 2).sum(1).mean()) / np.sqrt((b ** 2).sum(1).mean()))


def gpu_for_case(z, precision=None, **over):
    from komd_gb300 import gpu, lattice
    s = case_system(z)
    terms = gpu.TERM_LJ | gpu.TERM_FENE | gpu.TERM_LIMIT
    if int(z["p_enable_3b"]):
        terms |= gpu.TERM_ATM
    if int(z.get("p_enable_3b_approx", 0)):
        terms |= gpu.TERM_ATM2B
    if "table_x" in z:   # the tabulated force in LJ12_6's place
        terms = (terms & ~gpu.TERM_LJ) | gpu.TERM_TABULATED
    kw = dict(cutoff=float(z["p_cutoff"]), cutoff_3b=float(z["p_cutoff"]), nu=lattice.energy_3b_to_nu(float(z["p_energy_3b"])),
              dt=float(z["p_delta_t"]), terms=terms, precision=gpu.FP32 if precision is None else precision,
              atm_direct=int(z["p_enable_3b_direct"]), stiffness=float(z.get("p_stiffness", 30.0)),
              limit=float(z["p_limit"]), rdf_max=float(z.get("p_sensor_rdf_max", 0.0)),
              rdf_dr=float(z.get("p_sensor_rdf_dr", 0.0)), thermostat=int(z.get("p_thermostat", 0)),
              temperature_target=float(z.get("p_temperature", 0.0)))
    kw.update(over)
    cfg = gpu.make_config(z["low"], z["high"], float(z["p_cell_size"]), **kw)
    g = gpu.GpuSystem(s, cfg)
    if "table_x" in z:
        g.set_pair_table(z["table_x"], z["table_y"], 1e6, 0.0)
    return g, s


def _state_at(z, step):
    return (z["r0"], z["v0"]) if step == 0 else (z[f"s{step}_R"], z[f"s{step}_V"])


@pytest.mark.parametrize("name", CASES)
def test_cells_and_neighbour_counts_bitexact(name):
    z = load_case(name)
    g, _ = gpu_for_case(z)
    for step in [int(d) for d in z["dumps"]]:
        r, v = _state_at(z, step)
        g.set_state(r, v)
        g.update_container()
        count, idx = g.cells()
        assert np.array_equal(count, z[f"s{step}_cell_count"]), f"{name} step {step}"
        assert np.array_equal(idx, z[f"s{step}_cell_idx"]), f"{name} step {step}"
        r_gpu, _, _ = g.download()
        assert np.array_equal(r_gpu, z[f"s{step}_R"]), "periodic wrap must be bit-exact"
        assert np.array_equal(g.neighbour_counts(), z[f"s{step}_ncount"])
    g.close()


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_forces_match_reference(name, prec):
    from komd_gb300 import gpu
    z = load_case(name)
    g, _ = gpu_for_case(z, precision=gpu.FP32 if prec == "fp32" else gpu.FP64)
    tol = FP32_FORCE_RMSE if prec == "fp32" else FP64_FORCE_RMSE
    for step in [int(d) for d in z["dumps"]]:
        r, v = _state_at(z, step)
        g.set_state(r, v)
        g.update_container()
        g.forces()
        _, _, f = g.download()
        ref = z[f"s{step}_F"]
        finite = np.all(np.abs(ref) < 1e29, axis=1)     # FENE overstretch rows are 1e30 by design
        err = rel_rmse(f[finite], ref[finite])
        assert err < tol, f"{name} step {step} {prec}: rel RMSE {err:.3e}"
    g.close()


@pytest.mark.parametrize("name", ["lj864", "ljatm864", "atmlist500", "fene375"])
def test_sensors_match_reference(name):
    from komd_gb300 import gpu
    z = load_case(name)
    for prec, rtol in ((gpu.FP64, 1e-11), (gpu.FP32, 2e-5)):
        g, _ = gpu_for_case(z, precision=prec)
        step = int(z["dumps"][0])
        r, v = _state_at(z, step)
        g.set_state(r, v)
        g.update_container()
        g.forces()
        obs = g.measure(gpu.MEASURE_TEMPERATURE | gpu.MEASURE_ENERGY | gpu.MEASURE_PRESSURE | gpu.MEASURE_RDF)
        assert obs["temperature"] == pytest.approx(float(z[f"s{step}_temp"]), rel=1e-13)
        assert obs["u_lj"] == pytest.approx(float(z[f"s{step}_upot"]), rel=rtol)
        pres = z[f"s{step}_pressure"]
        scale = np.abs(pres).max()
        np.testing.assert_allclose(obs["pressure"], pres, rtol=0, atol=rtol * 10 * scale)
        if f"s{step}_rdf" in z:
            assert np.array_equal(obs["rdf"], z[f"s{step}_rdf"])
        g.close()


@pytest.mark.parametrize("name", ["lj864", "ljatm864", "fene375", "edge_box"])
def test_lj_histograms_match_reference(name):
    """KOMD_MEASURE_LJ_HIST against the reference's LJ12_6_Sensor histograms
    (LJ12_6_Sensor.cpp:47-84: per bin of r over 3 max_sigma, the sums of
    u and of F(r) = 24 eps (2 s12 - s6) / r and their counts, over the pairs
    the sensor counts once), at every dumped state.  FP64 mode: the same bins
    and counts, sums to rounding; FP32 mode: counts within the pairs that sit
    on a bin edge, sums to FP32 accuracy."""
    from komd_gb300 import gpu
    z = load_case(name)
    for step in (int(d) for d in z["dumps"]):
        ref = z[f"s{step}_ljhist"]
        nb = ref.shape[1]
        for prec in (gpu.FP64, gpu.FP32):
            g, _ = gpu_for_case(z, precision=prec, lj_bins=nb, max_sigma=1.0)
            r, v = _state_at(z, step)
            g.set_state(r, v)
            g.update_container()
            g.forces()
            h = g.measure(gpu.MEASURE_ENERGY | gpu.MEASURE_LJ_HIST)["lj_hist"]
            g.close()
            if prec == gpu.FP64:
                assert np.array_equal(h[2], ref[2]) and np.array_equal(h[3], ref[3]), f"{name} step {step}"
                np.testing.assert_allclose(h[0], ref[0], rtol=1e-11, atol=1e-11 * np.abs(ref[0]).max())
                np.testing.assert_allclose(h[1], ref[1], rtol=1e-11, atol=1e-11 * np.abs(ref[1]).max())
            else:
                assert np.abs(h[2] - ref[2]).sum() <= 4 and h[2].sum() == ref[2].sum(), f"{name} step {step}"
                scale_u, scale_f = np.abs(ref[0]).max(), np.abs(ref[1]).max()
                np.testing.assert_allclose(h[0].sum(), ref[0].sum(), rtol=2e-5)
                assert np.abs(h[0] - ref[0]).max() <= 1e-3 * scale_u
                assert np.abs(h[1] - ref[1]).max() <= 1e-3 * scale_f


def test_fp64_trajectory_follows_reference():
    """100 NVE steps in FP64 mode through the graph-replayed step: positions
    stay on the reference's trajectory."""
    from komd_gb300 import gpu
    z = load_case("lj864")
    g, _ = gpu_for_case(z, precision=gpu.FP64)
    g.update_container()
    g.forces()
    g.step(1)
    r1, v1, _ = g.download()
    assert np.abs(r1 - z["s1_R"]).max() < 1e-12
    g.step(99)
    r, v, f = g.download()
    assert np.abs(r - z["s100_R"]).max() < 1e-8
    assert rel_rmse(f, z["s100_F"]) < 1e-6
    g.close()


def test_atm2b_trajectory_follows_reference():
    """ATM2B (enable_3b_approx) in FP64: the engine's factor and scaled LJ
    forces keep the reference's trajectory for 20 steps."""
    from komd_gb300 import gpu
    z = load_case("atm2b864")
    g, _ = gpu_for_case(z, precision=gpu.FP64)
    g.update_container()
    g.forces()
    _, _, f0 = g.download()
    assert rel_rmse(f0, z["s0_F"]) < 1e-12
    g.step(20)
    r, v, f = g.download()
    assert np.abs(r - z["s20_R"]).max() < 1e-8
    assert rel_rmse(f, z["s20_F"]) < 1e-6
    g.close()


def test_tabulated_force_and_rdf_profiler_follow_reference(oracle_lib):
    """ibi864: the tabulated pair force (IBI_ForceFunctor with a 100-node
    table) keeps the reference's trajectory for 20 steps in FP64, and the
    RDF_Profiler histogram matches it; replacing the table between steps
    reaches the captured step graph."""
    from komd_gb300 import gpu
    z = load_case("ibi864")
    g, s = gpu_for_case(z, precision=gpu.FP64)
    g.update_container()
    g.forces()
    _, _, f0 = g.download()
    assert rel_rmse(f0, z["s0_F"]) < 1e-13
    g.step(1)
    r1, _, _ = g.download()
    assert np.abs(r1 - z["s1_R"]).max() < 1e-12
    nb = z["s1_ibirdf"].size
    bins = g.rdf_profile(float(z["p_cutoff"]), nb)
    gr = oracle_lib.rdf_profile_normalise(bins, 1, float(z["p_cutoff"]), nb, s.n, float(np.prod(z["high"] - z["low"])))
    np.testing.assert_allclose(gr, z["s1_ibirdf"], rtol=1e-14, atol=0)
    g.step(19)
    r, _, f = g.download()
    assert np.abs(r - z["s20_R"]).max() < 1e-8
    assert rel_rmse(f, z["s20_F"]) < 1e-6
    # a zero table switches the pair force off inside the same graph
    g.set_pair_table(z["table_x"], np.zeros_like(z["table_y"]), 1e6, 0.0)
    g.step(1)
    _, _, fz = g.download()
    assert np.abs(fz).max() == 0.0
    g.close()


def test_thermostat_trajectory_follows_reference():
    """The always-on VelocityScaling thermostat: the initial application
    through komd_gpu_scale_velocities (Simulation.cpp:42) and the per-step
    device-side application inside the step graph follow the reference's
    thermostatted trajectory for 50 steps (FP64)."""
    from komd_gb300 import gpu
    z = load_case("thermo864")
    t_target = float(z["p_temperature"])
    g, _ = gpu_for_case(z, precision=gpu.FP64)
    g.update_container()
    g.forces()
    t0 = g.measure(gpu.MEASURE_TEMPERATURE)["temperature"]
    g.scale_velocities(np.sqrt(t_target / t0))
    _, v0, _ = g.download()
    assert np.abs(v0 - z["s0_V"]).max() < 1e-13
    g.step(1)
    r1, v1, _ = g.download()
    assert np.abs(r1 - z["s1_R"]).max() < 1e-12
    assert np.abs(v1 - z["s1_V"]).max() < 1e-12
    g.step(49)
    r, v, _ = g.download()
    assert np.abs(r - z["s50_R"]).max() < 1e-8
    assert np.abs(v - z["s50_V"]).max() < 1e-7
    assert g.measure(gpu.MEASURE_TEMPERATURE)["temperature"] == pytest.approx(t_target, rel=1e-10)
    g.close()


def test_fp32_trajectory_close_to_reference():
    from komd_gb300 import gpu
    z = load_case("ljatm864")
    g, _ = gpu_for_case(z, precision=gpu.FP32)
    g.update_container()
    g.forces()
    g.step(20)
    r, v, f = g.download()
    assert np.abs(r - z["s20_R"]).max() < 1e-4
    assert rel_rmse(f, z["s20_F"]) < 1e-3
    g.close()


def _oracle_vertex(oracle_lib, s, cell, rc3, nu, full=True):
    sim = oracle_lib.OracleSim(s, cell, rc3, nu=nu, lj=False, atm=True, atm_mode="full" if full else "vertex_compat",
                               atm_sign=oracle_lib.ATM_SIGN_PHYSICAL, virial_mode=oracle_lib.VIRIAL_CORRECT)
    sim.update_container()
    sim.forces()
    return sim


def test_atm_full_physical_vs_oracle(oracle_lib):
    """FULL enumeration with F = -grad V (the physics mode): forces, energy,
    triplet count and virial against the oracle's vertex enumeration."""
    from komd_gb300 import gpu, lattice
    s = lattice.argon_fcc(6, rho=0.8442, t_star=0.722, seed=21, jitter=0.06)
    nu = 0.073
    sim = _oracle_vertex(oracle_lib, s, 2.0, 2.0, nu)
    cfg = gpu.make_config(s.low, s.high, 2.0, cutoff=2.0, cutoff_3b=2.0, nu=nu, terms=gpu.TERM_ATM,
                          atm_sign=gpu.ATM_SIGN_PHYSICAL, atm_enum=gpu.ATM_ENUM_FULL, virial_mode=gpu.VIRIAL_CORRECT)
    g = gpu.GpuSystem(s, cfg)
    g.update_container()
    g.forces()
    _, _, f = g.download()
    assert rel_rmse(f, sim.f) < FP32_FORCE_RMSE
    obs = g.measure(gpu.MEASURE_ENERGY | gpu.MEASURE_PRESSURE)
    assert obs["triplets"] == sim.atm_out.triplets
    assert obs["u_atm"] == pytest.approx(sim.atm_out.energy, rel=1e-5)
    np.testing.assert_allclose(obs["virial"], np.array(sim.atm_out.virial[:]), rtol=0,
                               atol=1e-4 * np.abs(np.array(sim.atm_out.virial[:])).max())
    g.close()


def test_atm_physical_is_minus_gradient():
    """Central differences of the GPU ATM energy equal the GPU physical force
    (FP64 mode, step 1e-6: small enough that no triplet side crosses the
    truncation at cutoff_3b, where the energy jumps)."""
    from komd_gb300 import gpu, lattice
    s = lattice.argon_fcc(4, rho=0.8442, t_star=0.722, seed=22, jitter=0.08)
    cfg = gpu.make_config(s.low, s.high, 2.0, cutoff=2.0, cutoff_3b=2.0, nu=0.073, terms=gpu.TERM_ATM,
                          precision=gpu.FP64, atm_sign=gpu.ATM_SIGN_PHYSICAL, atm_enum=gpu.ATM_ENUM_FULL)
    g = gpu.GpuSystem(s, cfg)
    g.update_container()
    g.forces()
    _, _, f = g.download()
    h = 1e-6
    for atom in (0, 7, 31, 100):
        for d in range(3):
            e = []
            for sgn in (1, -1):
                r = s.r.copy()
                r[atom, d] += sgn * h
                g.set_state(r, None)
                g.update_container()
                e.append(g.measure(gpu.MEASURE_ENERGY)["u_atm"])
            fd = -(e[0] - e[1]) / (2 * h)
            assert fd == pytest.approx(f[atom, d], rel=1e-5, abs=1e-7)
    g.close()


def test_bonded_vs_oracle(oracle_lib):
    from komd_gb300 import gpu, lattice
    s = lattice.triatomic_sc(5, rho_site=0.5, t_star=1.0, seed=23)
    s.r = s.r + np.random.default_rng(5).normal(0, 0.03, s.r.shape)   # strain bonds and angles
    th0 = np.deg2rad(109.47)
    cfg = gpu.make_config(s.low, s.high, 2.5, cutoff=2.5, terms=gpu.TERM_LJ | gpu.TERM_BONDED, bond_k=1000.0,
                          bond_r0=1.0, angle_k=100.0, angle_theta0=th0, virial_mode=gpu.VIRIAL_CORRECT)
    g = gpu.GpuSystem(s, cfg)
    g.update_container()
    g.forces()
    _, _, f = g.download()
    sim = oracle_lib.OracleSim(s, 2.5, 2.5, bonded=dict(bonds=s.bonds, angles=s.angles, kb=1000.0, r0=1.0, ka=100.0,
                                                        theta0=th0))
    sim.update_container()
    sim.forces()
    assert rel_rmse(f, sim.f) < 2e-5
    obs = g.measure(gpu.MEASURE_ENERGY)
    assert obs["u_bonded"] == pytest.approx(sim.e_bonded, rel=1e-4)
    assert obs["u_lj"] == pytest.approx(sim.lj_out.u_total, rel=1e-5)
    g.close()


def test_graph_step_equals_manual_sequence():
    from komd_gb300 import gpu
    z = load_case("ljatm864")
    a, _ = gpu_for_case(z)
    b, _ = gpu_for_case(z)
    for g in (a, b):
        g.update_container()
        g.forces()
    a.step(5)
    for _ in range(5):
        b.integrate0()
        b.update_container()
        b.forces()
        b.integrate1()
    ra, va, fa = a.download()
    rb, vb, fb = b.download()
    assert np.abs(ra - rb).max() < 1e-9
    assert rel_rmse(fa, fb) < 1e-6


def test_full_size_binning_and_momentum():
    """256,000-site FCC LJ+ATM (the benchmark size): the cell lists agree with
    a numpy restatement of the binning formula, every site is in exactly one
    domain cell in ascending order, and the physical force sums to zero."""
    from komd_gb300 import gpu, lattice
    s = lattice.argon_fcc(40, rho=0.8442, t_star=0.722, seed=4, jitter=0.02)
    cfg = gpu.make_config(s.low, s.high, 2.5, cutoff=2.5, cutoff_3b=2.0, nu=0.073,
                          terms=gpu.TERM_LJ | gpu.TERM_ATM, atm_sign=gpu.ATM_SIGN_PHYSICAL,
                          atm_enum=gpu.ATM_ENUM_FULL, virial_mode=gpu.VIRIAL_CORRECT)
    g = gpu.GpuSystem(s, cfg)
    g.update_container()
    nd = np.array(g.grid_dims())
    count, idx = g.cells()
    b = np.clip(np.trunc((s.r - s.low) / 2.5).astype(np.int64), 0, nd - 1) + 1
    lin = b[:, 0] + (nd[0] + 2) * (b[:, 1] + (nd[1] + 2) * b[:, 2])
    expect = np.bincount(lin, minlength=count.size)
    c3 = count.reshape(nd[2] + 2, nd[1] + 2, nd[0] + 2)
    dom = np.zeros_like(c3, dtype=bool)
    dom[1:-1, 1:-1, 1:-1] = True
    assert np.array_equal(count.reshape(c3.shape)[dom], expect.reshape(c3.shape)[dom])
    starts = np.concatenate(([0], np.cumsum(count)))
    dom_flat = dom.ravel()
    seen = np.concatenate([idx[starts[c]:starts[c + 1]] for c in np.flatnonzero(dom_flat)])
    assert np.array_equal(np.sort(seen), np.arange(s.n))
    for c in np.flatnonzero(dom_flat)[:2000]:
        seg = idx[starts[c]:starts[c + 1]]
        assert np.all(np.diff(seg) > 0)
    g.forces()
    _, _, f = g.download()
    assert np.abs(f.sum(0)).max() < 1e-3 * np.sqrt(s.n) * np.abs(f).mean()
    obs = g.measure(gpu.MEASURE_ENERGY | gpu.MEASURE_TEMPERATURE)
    assert obs["n_in_box"] == s.n
    assert obs["triplets"] > 15 * s.n     # thermalised FCC: 18 neighbours inside 2.0
    g.close()


def _physics_cfg(s, skin, cell):
    from komd_gb300 import gpu
    return gpu.make_config(s.low, s.high, cell, cutoff=2.5, cutoff_3b=2.0, nu=0.073, dt=0.005,
                           terms=gpu.TERM_LJ | gpu.TERM_ATM, atm_sign=gpu.ATM_SIGN_PHYSICAL,
                           atm_enum=gpu.ATM_ENUM_FULL, virial_mode=gpu.VIRIAL_CORRECT, skin=skin)


def test_verlet_path_matches_rebuild_every_step(oracle_lib):
    """The Verlet list (skin 0.3, rebuilt on demand inside the graph) gives the
    forces of a per-step rebuild: same trajectory over 60 steps, and forces at
    the end equal a fresh rebuild's and the oracle's."""
    from komd_gb300 import gpu, lattice
    s = lattice.argon_fcc(10, rho=0.8442, t_star=1.2, seed=41, jitter=0.05)    # 4000 sites, L = 16.8
    a = gpu.GpuSystem(s, _physics_cfg(s, 0.3, 2.8))
    b = gpu.GpuSystem(s, _physics_cfg(s, 0.0, 2.8))
    for g in (a, b):
        g.update_container()
        g.forces()
    for _ in range(6):
        a.step(10)
        b.step(10)
    ra, va, fa = a.download()
    rb, vb, fb = b.download()
    assert np.abs(ra - rb).max() < 1e-4
    assert rel_rmse(fa, fb) < 1e-4
    # list-based forces of the last step == forces after a fresh rebuild
    a.update_container()
    a.forces()
    _, _, fresh = a.download()
    assert rel_rmse(fa, fresh) < 2e-6
    sim = oracle_lib.OracleSim(lattice.System(r=ra, v=va, m=s.m, eps=s.eps, sig=s.sig, mol_id=s.mol_id, low=s.low,
                                              high=s.high), 2.8, 2.5, nu=0.073, cutoff_atm=2.0, atm=True,
                               atm_mode="full", atm_sign=oracle_lib.ATM_SIGN_PHYSICAL,
                               virial_mode=oracle_lib.VIRIAL_CORRECT)
    sim.update_container()
    sim.forces()
    assert rel_rmse(fresh, sim.f) < FP32_FORCE_RMSE
    obs = a.measure(gpu.MEASURE_ENERGY | gpu.MEASURE_PRESSURE)
    assert obs["u_lj"] == pytest.approx(sim.lj_out.u_total, rel=1e-5)
    assert obs["u_atm"] == pytest.approx(sim.atm_out.energy, rel=1e-5)
    a.close()
    b.close()


def test_binary_mixture_half_list_pass(oracle_lib):
    """Two species (sigma 1.0 / 0.88, epsilon 1.0 / 0.6; the reference's
    combining rules, LJ12_6.cpp:22-25: sigma = (s_i + s_j) / 2, epsilon =
    sqrt(e_i e_j)) on the benchmark's path: Verlet list with skin, the
    half-list LJ + ATM pass in its per-pair-parameter form, the fused step
    kernels.  After 50 steps the forces, the LJ and ATM energies and the
    virial match the oracle at the engine's positions."""
    from komd_gb300 import gpu, lattice
    s = lattice.argon_fcc(10, rho=0.8442, t_star=0.9, seed=43, jitter=0.05)    # 4000 sites, L = 16.8
    rng = np.random.default_rng(44)
    b_mask = rng.random(s.n) < 0.3
    s.sig = np.where(b_mask, 0.88, 1.0)
    s.eps = np.where(b_mask, 0.6, 1.0)
    g = gpu.GpuSystem(s, _physics_cfg(s, 0.3, 2.8))
    g.update_container()
    g.forces()
    g.step(50)
    r, v, f = g.download()
    obs = g.measure(gpu.MEASURE_ENERGY | gpu.MEASURE_PRESSURE)
    g.close()
    sim = oracle_lib.OracleSim(lattice.System(r=r, v=v, m=s.m, eps=s.eps, sig=s.sig, mol_id=s.mol_id, low=s.low,
                                              high=s.high), 2.8, 2.5, nu=0.073, cutoff_atm=2.0, atm=True,
                               atm_mode="full", atm_sign=oracle_lib.ATM_SIGN_PHYSICAL,
                               virial_mode=oracle_lib.VIRIAL_CORRECT)
    sim.update_container()
    sim.forces()
    assert rel_rmse(f, sim.f) < FP32_FORCE_RMSE
    assert obs["u_lj"] == pytest.approx(sim.lj_out.u_total, rel=1e-5)
    assert obs["u_atm"] == pytest.approx(sim.atm_out.energy, rel=1e-5)
    vir = np.array(sim.lj_out.virial[:]) + np.array(sim.atm_out.virial[:])
    np.testing.assert_allclose(obs["virial"], vir, rtol=0, atol=2e-5 * np.abs(vir).max())
    # Newton's third law of the once-per-pair and once-per-triplet sums
    assert np.abs(f.sum(0)).max() < 1e-3 * np.sqrt(s.n) * np.abs(f).mean()


def test_atm_only_on_the_half_list_pass(oracle_lib):
    """ATM without LJ on the Verlet path: the half-list pass in its general
    form (the LJ switch read per pair; the one-species LJ + ATM case runs a
    form without it).  4,000 sites, skin 0.3, FULL triplets, physical sign.
    The forces match the per-step cell lists' and the oracle's, and after 50
    steps the oracle's at the engine's positions."""
    from komd_gb300 import gpu, lattice
    s = lattice.argon_fcc(10, rho=0.8442, t_star=0.9, seed=47, jitter=0.05)

    def cfg(skin):
        return gpu.make_config(s.low, s.high, 2.8, cutoff=2.0, cutoff_3b=2.0, nu=0.073, dt=0.005,
                               terms=gpu.TERM_ATM, atm_sign=gpu.ATM_SIGN_PHYSICAL, atm_enum=gpu.ATM_ENUM_FULL,
                               virial_mode=gpu.VIRIAL_CORRECT, skin=skin)

    def oracle_forces(r, v):
        sim = oracle_lib.OracleSim(lattice.System(r=r, v=v, m=s.m, eps=s.eps, sig=s.sig, mol_id=s.mol_id,
                                                  low=s.low, high=s.high), 2.8, 2.0, nu=0.073, cutoff_atm=2.0,
                                   lj=False, atm=True, atm_mode="full", atm_sign=oracle_lib.ATM_SIGN_PHYSICAL,
                                   virial_mode=oracle_lib.VIRIAL_CORRECT)
        sim.update_container()
        sim.forces()
        return sim.f

    a = gpu.GpuSystem(s, cfg(0.3))
    b = gpu.GpuSystem(s, cfg(0.0))
    for g in (a, b):
        g.update_container()
        g.forces()
    r0, v0, fa = a.download()
    _, _, fb = b.download()
    assert rel_rmse(fa, fb) < 2e-6
    assert rel_rmse(fa, oracle_forces(r0, v0)) < FP32_FORCE_RMSE
    a.step(50)
    r, v, f = a.download()
    assert np.isfinite(r).all()
    assert rel_rmse(f, oracle_forces(r, v)) < FP32_FORCE_RMSE
    a.close()
    b.close()


def test_verlet_requires_cell_for_skin():
    from komd_gb300 import gpu, lattice
    s = lattice.argon_fcc(10, seed=1)
    with pytest.raises(gpu.KomdError, match="cutoff \\+ skin"):
        gpu.GpuSystem(s, _physics_cfg(s, 0.3, 2.5))


def test_multisite_300k_full_size(oracle_lib):
    """The multi-site workload at its full size: 100,000 flexible 3-site
    molecules (300,000 sites) on a simple-cubic lattice at site density 0.8,
    one seeded orientation for all molecules, harmonic bonds (k 1000, r0 1) and angles (k 100, theta0
    109.47 deg), intermolecular LJ with cutoff 2.5, FP32 forces.  The forces of
    256 random sites match an FP64 restatement (LJ over a periodic k-d tree in
    numpy, bonded terms by the oracle), the total force vanishes, and 500 NVE
    steps at dt 0.002 stay stable and keep the molecules' shape."""
    from scipy.spatial import cKDTree
    from komd_gb300 import gpu, lattice
    # one orientation for all molecules: with random ones, sites of neighbouring
    # molecules start a fraction of sigma apart at this density
    s = lattice.triatomic_count(100000, rho_site=0.8, t_star=1.0, seed=31, aligned=True)
    assert s.n == 300000
    L = np.asarray(s.high - s.low)
    # cells bin molecules by their centre of mass, as the reference does: with
    # cell >= cutoff + the molecule's diameter every site pair inside the
    # cutoff is in adjacent cells, so the minimum-image restatement below
    # sees the same pairs
    cell = float(L[0] / np.floor(L[0] / 4.2))
    th0 = np.deg2rad(109.47)
    cfg = gpu.make_config(s.low, s.high, cell, cutoff=2.5, dt=0.002, terms=gpu.TERM_LJ | gpu.TERM_BONDED,
                          bond_k=1000.0, bond_r0=1.0, angle_k=100.0, angle_theta0=th0,
                          virial_mode=gpu.VIRIAL_CORRECT)
    g = gpu.GpuSystem(s, cfg)
    g.update_container()
    g.forces()
    r, _, f = g.download()
    # bonded forces of every site in FP64 (the oracle's restatement)
    fb = np.zeros_like(r)
    w = np.zeros(6)
    L_ = oracle_lib.lib()
    bonds = np.ascontiguousarray(s.bonds, np.int64)
    angles = np.ascontiguousarray(s.angles, np.int64)
    rr = np.ascontiguousarray(r)
    L_.kor_bonded(bonds.shape[0], oracle_lib._p(bonds), 1000.0, 1.0, angles.shape[0], oracle_lib._p(angles), 100.0,
                  th0, oracle_lib._p(rr), None, oracle_lib._p(fb), oracle_lib._p(w))
    # intermolecular LJ of sampled sites in FP64, minimum image
    mol = s.mol_id
    tree = cKDTree(np.mod(r - s.low, L), boxsize=L)
    sample = np.random.default_rng(7).choice(s.n, 256, replace=False)
    ref = np.zeros((sample.size, 3))
    for k, i in enumerate(sample):
        js = np.asarray(tree.query_ball_point(np.mod(r[i] - s.low, L), 2.5), np.int64)
        js = js[mol[js] != mol[i]]
        dr = r[i] - r[js]
        dr -= L * np.round(dr / L)
        r2 = (dr * dr).sum(1)
        keep = r2 <= 6.25
        inv = 1.0 / r2[keep]
        s6 = inv ** 3
        ref[k] = ((24.0 * (2.0 * s6 * s6 - s6) * inv)[:, None] * dr[keep]).sum(0)
    ref += fb[sample]
    rms = np.sqrt((f * f).sum(1).mean())
    assert np.abs(f[sample] - ref).max() < 1e-4 * rms
    assert np.abs(f.sum(0)).max() < 1e-5 * rms * np.sqrt(s.n)

    def energy():
        o = g.measure(gpu.MEASURE_ENERGY | gpu.MEASURE_TEMPERATURE)
        return 0.5 * o["mv2"] + o["u_lj"] + o["u_bonded"]

    e0 = energy()
    g.step(500)
    e1 = energy()
    r1, v1, _ = g.download()
    assert np.isfinite(r1).all() and np.isfinite(v1).all()
    # the reference's LJ is truncated without a shift: while the lattice
    # disorders, pairs entering the cutoff change the energy by V(2.5) = -0.016
    # each (about -0.01 per site over these 500 steps); a broken integration
    # would be orders of magnitude off
    assert abs(e1 - e0) / s.n < 0.05
    b = np.linalg.norm(r1[s.bonds[:, 0]] - r1[s.bonds[:, 1]], axis=1)
    assert 0.8 < b.min() and b.max() < 1.2
    g.close()


def test_multisite_verlet_matches_cell_lists():
    """Molecules on the Verlet path: 8,000 flexible 3-site molecules (24,000
    sites, the multi-site workload's density, bonds and angles), binned by
    their centre of mass on cells >= cutoff + skin + 2.0 (twice a site's
    largest distance from its molecule's centre, 0.84 at rest), with the
    same-molecule pairs in the rows but excluded from LJ.  Over 200 steps with
    list rebuilds the trajectory follows the per-step cell lists' (skin 0, the
    same cells), the list's forces equal a fresh rebuild's, and the energies
    agree."""
    from komd_gb300 import gpu, lattice
    s = lattice.triatomic_count(8000, rho_site=0.8, t_star=1.0, seed=37, aligned=True)
    L = float((s.high - s.low)[0])
    th0 = np.deg2rad(109.47)

    def cfg(skin, reach):
        return gpu.make_config(s.low, s.high, L / np.floor(L / reach), cutoff=2.5, dt=0.002,
                               terms=gpu.TERM_LJ | gpu.TERM_BONDED, bond_k=1000.0, bond_r0=1.0, angle_k=100.0,
                               angle_theta0=th0, virial_mode=gpu.VIRIAL_CORRECT, skin=skin)

    a = gpu.GpuSystem(s, cfg(0.3, 4.8))
    b = gpu.GpuSystem(s, cfg(0.0, 4.8))
    for g in (a, b):
        g.update_container()
        g.forces()
    _, _, fa0 = a.download()
    _, _, fb0 = b.download()
    assert rel_rmse(fa0, fb0) < 2e-6
    a.set_profiling(False)
    for _ in range(20):
        a.step(10)
        b.step(10)
    assert a.profile().get("list_rebuilds", (0, 0.0))[0] >= 2   # the lists were rebuilt on the way
    ra, va, fa = a.download()
    rb, vb, fb = b.download()
    assert np.isfinite(ra).all() and np.isfinite(va).all()
    assert np.abs(ra - rb).max() < 1e-4
    assert rel_rmse(fa, fb) < 1e-4
    oa = a.measure(gpu.MEASURE_ENERGY | gpu.MEASURE_TEMPERATURE)
    ob = b.measure(gpu.MEASURE_ENERGY | gpu.MEASURE_TEMPERATURE)
    for key in ("u_lj", "u_bonded", "mv2"):
        assert oa[key] == pytest.approx(ob[key], rel=1e-4)
    a.update_container()
    a.forces()
    _, _, fresh = a.download()
    assert rel_rmse(fa, fresh) < 2e-6
    a.close()
    b.close()


def test_molecules_with_atm_on_the_half_list_pass():
    """LJ + ATM (FULL, physical sign) + bonds and angles on the Verlet path:
    the half-list pass writes f itself (the bonded kernels add to it before
    the flush) instead of its per-slot FP32 buffer.  2,000 flexible 3-site
    molecules (6,000 sites, site density 0.8), cells >= cutoff + skin + 2.0.
    The forces match the per-step cell lists' (skin 0, the same cells) at the
    start, the trajectories agree over 100 steps with list rebuilds, and the
    energies agree."""
    from komd_gb300 import gpu, lattice
    s = lattice.triatomic_count(2000, rho_site=0.8, t_star=1.0, seed=41, aligned=True)
    L = float((s.high - s.low)[0])
    th0 = np.deg2rad(109.47)

    def cfg(skin):
        return gpu.make_config(s.low, s.high, L / np.floor(L / 4.8), cutoff=2.5, cutoff_3b=2.0, nu=0.073, dt=0.002,
                               terms=gpu.TERM_LJ | gpu.TERM_ATM | gpu.TERM_BONDED, atm_sign=gpu.ATM_SIGN_PHYSICAL,
                               atm_enum=gpu.ATM_ENUM_FULL, virial_mode=gpu.VIRIAL_CORRECT, bond_k=1000.0,
                               bond_r0=1.0, angle_k=100.0, angle_theta0=th0, skin=skin)

    a = gpu.GpuSystem(s, cfg(0.3))
    b = gpu.GpuSystem(s, cfg(0.0))
    for g in (a, b):
        g.update_container()
        g.forces()
    _, _, fa0 = a.download()
    _, _, fb0 = b.download()
    assert rel_rmse(fa0, fb0) < 2e-6
    a.set_profiling(False)
    for _ in range(10):
        a.step(10)
        b.step(10)
    assert a.profile().get("list_rebuilds", (0, 0.0))[0] >= 1
    ra, va, fa = a.download()
    rb, vb, fb = b.download()
    assert np.isfinite(ra).all() and np.isfinite(va).all()
    assert np.abs(ra - rb).max() < 1e-4
    assert rel_rmse(fa, fb) < 1e-4
    oa = a.measure(gpu.MEASURE_ENERGY | gpu.MEASURE_TEMPERATURE)
    ob = b.measure(gpu.MEASURE_ENERGY | gpu.MEASURE_TEMPERATURE)
    for key in ("u_lj", "u_atm", "u_bonded", "mv2"):
        assert oa[key] == pytest.approx(ob[key], rel=1e-4)
    a.close()
    b.close()


def test_plain_lj_4000_fp64_1000_steps(oracle_lib):
    """The plain LJ workload at its full size and length: 4,000 argon atoms
    (FCC 10^3, rho* 0.8442, T* 0.722), cutoff 2.5, 1000 NVE steps of dt 0.005,
    all FP64.  After the 1000 steps the engine's positions follow the oracle's
    (the reference's pair sweep) to 1e-5 (the FP64 forces agree to ~1e-12 and
    chaos amplifies that by ~1e4 over this run), and the energy, the virial
    pressure and the RDF (200 bins to 2.5) agree."""
    from komd_gb300 import gpu, lattice
    s = lattice.argon_fcc(10, rho=0.8442, t_star=0.722, seed=51)
    L = float((s.high - s.low)[0])
    cell = L / np.floor(L / 2.5)
    cfg = gpu.make_config(s.low, s.high, cell, cutoff=2.5, dt=0.005, terms=gpu.TERM_LJ, precision=gpu.FP64,
                          virial_mode=gpu.VIRIAL_CORRECT, rdf_max=2.5, rdf_dr=0.0125)
    g = gpu.GpuSystem(s, cfg)
    g.update_container()
    g.forces()
    g.step(1000)
    r, v, f = g.download()
    sim = oracle_lib.OracleSim(s, cell, 2.5, dt=0.005, limit=1e30, virial_mode=oracle_lib.VIRIAL_CORRECT)
    sim.update_container()
    sim.forces()
    for _ in range(1000):
        sim.step()
    assert np.abs(r - sim.r).max() < 1e-5
    assert np.abs(v - sim.v).max() < 1e-5
    obs = g.measure(gpu.MEASURE_ENERGY | gpu.MEASURE_PRESSURE | gpu.MEASURE_RDF)
    sim.update_container()
    sim.forces()
    assert obs["u_lj"] == pytest.approx(sim.lj_out.u_total, rel=1e-8)
    pres = sim.momentum(s.n) + np.array(sim.lj_out.virial[:])
    np.testing.assert_allclose(obs["pressure"], pres, rtol=1e-6, atol=1e-6 * np.abs(pres).max())
    rdf = sim.rdf(2.5, 0.0125)
    assert obs["rdf"].size == rdf.size == 200
    assert np.abs(obs["rdf"] - rdf).max() <= 4    # a pair or two may sit within 1e-7 of a bin edge
    assert obs["rdf"].sum() == pytest.approx(rdf.sum(), abs=4)
    g.close()


def test_lj_atm_32k_fp32_against_fp64_oracle(oracle_lib):
    """The LJ + ATM workload at its full size: 32,000 argon atoms (FCC 20^3),
    LJ cutoff 2.5, ATM nu* 0.073 with cutoff 2.0 on all sides, FULL triplets
    and F = -grad V, FP32 forces with FP64 integration.  At the start and
    after 100 steps the forces, LJ and ATM energies and the virial match the
    FP64 oracle evaluated at the engine's positions."""
    from komd_gb300 import gpu, lattice
    s = lattice.argon_fcc(20, rho=0.8442, t_star=0.722, seed=52, jitter=0.05)   # off the symmetric lattice
    L = float((s.high - s.low)[0])
    cell = L / np.floor(L / 2.5)
    cfg = gpu.make_config(s.low, s.high, cell, cutoff=2.5, cutoff_3b=2.0, nu=0.073, dt=0.005,
                          terms=gpu.TERM_LJ | gpu.TERM_ATM, atm_sign=gpu.ATM_SIGN_PHYSICAL,
                          atm_enum=gpu.ATM_ENUM_FULL, virial_mode=gpu.VIRIAL_CORRECT)
    g = gpu.GpuSystem(s, cfg)
    g.update_container()
    g.forces()
    for steps in (0, 100):
        if steps:
            g.step(steps)
        r, v, f = g.download()
        at = lattice.System(r=r, v=v, m=s.m, eps=s.eps, sig=s.sig, mol_id=s.mol_id, low=s.low, high=s.high)
        sim = oracle_lib.OracleSim(at, cell, 2.5, nu=0.073, cutoff_atm=2.0, atm=True, atm_mode="full",
                                   atm_sign=oracle_lib.ATM_SIGN_PHYSICAL, virial_mode=oracle_lib.VIRIAL_CORRECT)
        sim.update_container()
        sim.forces()
        assert rel_rmse(f, sim.f) < FP32_FORCE_RMSE
        obs = g.measure(gpu.MEASURE_ENERGY | gpu.MEASURE_PRESSURE)
        assert obs["u_lj"] == pytest.approx(sim.lj_out.u_total, rel=1e-5)
        assert obs["u_atm"] == pytest.approx(sim.atm_out.energy, rel=1e-5)
        assert obs["triplets"] == sim.atm_out.triplets
        vir = np.array(sim.lj_out.virial[:]) + np.array(sim.atm_out.virial[:])
        np.testing.assert_allclose(obs["virial"], vir, rtol=0, atol=2e-5 * np.abs(vir).max())
    g.close()
