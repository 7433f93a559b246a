"""The CPU oracle against the reference itself (CPU, no GPU).

The fixtures under tests/golden/ were produced by the reference's own code
(oracle/ref/harness.cpp linked against the reference sources; see
tests/golden/make_golden.py).  The oracle must reproduce them bit for bit:
positions, forces, cell lists incl. halo copies, neighbour counts,
temperature, the LJ sensor potential, the pressure tensor and the RDF
histogram, along 0, 1 and up to 100 steps of NVE dynamics.
"""
import numpy as np
import pytest

from conftest import CASES, case_system, load_case


def atm2b_factor(oracle_lib, z, s):
    """The ATM2B factor as the reference's constructor forms it from the COMP
    line (epsilon in J times conv_J_Ei) and the loaded molecule count."""
    from komd_gb300 import lattice
    if not int(z.get("p_enable_3b_approx", 0)):
        return 1.0
    nu = float(z["p_energy_3b"]) * 1e+9 * lattice.CONV_J_EI
    eps = (1.0 / lattice.CONV_J_EI) * lattice.CONV_J_EI      # COMP epsilon of the fixtures, J -> internal
    vol = float(np.prod(z["high"] - z["low"]))
    return oracle_lib.atm2b_factor(nu, len(np.unique(z["mol_id"])), vol, eps, 1.0)


def _sim(oracle_lib, z, **kw):
    from komd_gb300 import lattice
    s = case_system(z)
    nu = lattice.energy_3b_to_nu(float(z["p_energy_3b"]))
    table = (z["table_x"], z["table_y"], 1e6, 0.0) if "table_x" in z else None
    return oracle_lib.OracleSim(s, float(z["p_cell_size"]), float(z["p_cutoff"]), dt=float(z["p_delta_t"]), nu=nu,
                                limit=float(z["p_limit"]), stiffness=float(z.get("p_stiffness", 30.0)),
                                atm=bool(z["p_enable_3b"]), fene=True, lj_force_scale=atm2b_factor(oracle_lib, z, s),
                                lj=table is None, table=table, **kw)


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_bitwise(oracle_lib, name):
    oracle_lib.set_threads(1)   # the reference harness runs Kokkos Serial: same summation order
    z = load_case(name)
    sim = _sim(oracle_lib, z)
    dumps = [int(d) for d in z["dumps"]]
    list_atm = bool(z["p_enable_3b"]) and not bool(z["p_enable_3b_direct"])
    rdf_sum, n_rdf = None, 0
    # the LJ sensor's U(r) / F(r) histograms of each dumped measure (sensor_lj_bins
    # over 3 max_sigma; max_sigma is the COMP sigma, 1)
    nbins = int(z["s0_ljhist"].shape[1]) if "s0_ljhist" in z else 0
    for step in range(max(dumps) + 1):
        if step > 0:
            sim.integrate0()
        sim.update_container()
        sim.forces(nbins=nbins, max_sigma=1.0, ncount=True, with_atm_virial=list_atm)
        if step > 0:
            sim.integrate1()
        if int(z.get("p_thermostat", 0)):
            sim.thermostat(float(z["p_temperature"]))
        if step not in dumps:
            continue
        p = f"s{step}_"
        count, _, idx = sim.cell_lists()
        assert np.array_equal(count, z[p + "cell_count"]), f"{name} step {step}: cell counts"
        assert np.array_equal(idx, z[p + "cell_idx"]), f"{name} step {step}: cell lists"
        assert np.array_equal(sim.r, z[p + "R"]), f"{name} step {step}: positions"
        assert np.array_equal(sim.v, z[p + "V"]), f"{name} step {step}: velocities"
        assert np.array_equal(sim.f, z[p + "F"]), f"{name} step {step}: forces"
        assert sim.temperature() == z[p + "temp"]
        if "table_x" in z:
            # the tabulated force replaces LJ12_6, whose pass also counts the
            # neighbours; the LJ and pressure sensors re-run LJ12_6 itself
            _, g = sim.rdf_profile(float(z["p_cutoff"]), z[p + "ibirdf"].size)
            np.testing.assert_allclose(g, z[p + "ibirdf"], rtol=1e-14, atol=0)
            continue
        assert np.array_equal(sim.ncount, z[p + "ncount"]), f"{name} step {step}: neighbour counts"
        assert sim.lj_out.u_total == pytest.approx(float(z[p + "upot"]), rel=1e-13, abs=1e-12)
        if nbins:
            # LJ12_6_Sensor::LJ12_6_Pot (LJ12_6_Sensor.cpp:47-84): same bins, sums and counts
            hu, hf, cu, cf = sim.hist
            ref = z[p + "ljhist"]
            assert np.array_equal(cu, ref[2].astype(np.uint64)) and np.array_equal(cf, ref[3].astype(np.uint64))
            np.testing.assert_allclose(hu, ref[0], rtol=1e-12, atol=1e-12 * np.abs(ref[0]).max())
            np.testing.assert_allclose(hf, ref[1], rtol=1e-12, atol=1e-12 * np.abs(ref[1]).max())
        # PressureSensor: momentum over the first getNumMolecules() sites + LJ
        # list virial (+ ATM_Pressure for the list-based ATM only)
        pres = sim.momentum() + np.array(sim.lj_out.virial[:])
        if list_atm:
            pres = pres + np.array(sim.atm_out.virial[:])
        np.testing.assert_allclose(pres, z[p + "pressure"], rtol=1e-12, atol=1e-9)
        if p + "rdf" in z:
            # RDFSensor accumulates its bins over every measure() and writes the
            # running mean bins / samples with 6 significant digits
            rdf = sim.rdf(float(z["p_sensor_rdf_max"]), float(z["p_sensor_rdf_dr"]))
            rdf_sum = rdf if rdf_sum is None else rdf_sum + rdf
            n_rdf += 1
            if n_rdf == 1:
                assert np.array_equal(rdf, z[p + "rdf"])
            np.testing.assert_allclose(rdf_sum / n_rdf, z[p + "rdf"], rtol=1e-5, atol=1e-5)


def test_halo_copies_and_stretched_cells(oracle_lib):
    """edge_box: non-zero domain_low, non-cubic box and a stretched last cell."""
    z = load_case("edge_box")
    sim = _sim(oracle_lib, z)
    sim.update_container()
    nd = sim.nd
    count, start, idx = sim.cell_lists()
    nx, ny, nz = (d + 2 for d in nd)
    c3 = count.reshape(nz, ny, nx)
    # every halo cell repeats its periodic source cell
    assert np.array_equal(c3[:, :, 0], c3[:, :, nx - 2]) and np.array_equal(c3[:, :, nx - 1], c3[:, :, 1])
    # every site appears exactly once in the domain cells
    dom = c3[1:-1, 1:-1, 1:-1].sum()
    assert dom == sim.n


def test_momentum_conservation_full_atm(oracle_lib):
    """FULL enumeration, physical sign: total force vanishes (Newton's third law
    holds per triplet), and the vertex form with the COMPAT restriction equals
    the reference's enumeration."""
    z = load_case("ljatm864")
    from komd_gb300 import lattice
    nu = lattice.energy_3b_to_nu(float(z["p_energy_3b"]))
    s = case_system(z)
    ref = oracle_lib.OracleSim(s, 2.0, 2.0, nu=nu, lj=False, atm=True, atm_mode="compat")
    ref.update_container()
    ref.forces()
    vc = oracle_lib.OracleSim(s, 2.0, 2.0, nu=nu, lj=False, atm=True, atm_mode="vertex_compat")
    vc.update_container()
    vc.forces()
    scale = np.sqrt((ref.f ** 2).sum(1).mean())
    assert np.sqrt(((vc.f - ref.f) ** 2).sum(1).mean()) / scale < 1e-12
    full = oracle_lib.OracleSim(s, 2.0, 2.0, nu=nu, lj=False, atm=True, atm_mode="full",
                                atm_sign=oracle_lib.ATM_SIGN_PHYSICAL)
    full.update_container()
    full.forces()
    assert np.abs(full.f.sum(0)).max() < 1e-10 * np.abs(full.f).max()
    # the COMPAT set misses the (A,A,B) classes: it holds fewer triplets
    assert full.atm_out.triplets > vc.atm_out.triplets


@pytest.mark.parametrize("sign", ["physical", "reference"])
def test_oracle_atm_force_is_gradient(oracle_lib, sign):
    """ATM force of the oracle against central differences of its energy:
    PHYSICAL is -grad V; REFERENCE reproduces the reference kernel's +grad V."""
    from komd_gb300 import lattice
    s = lattice.argon_fcc(4, rho=0.8442, t_star=0.722, seed=22, jitter=0.08)
    sg = oracle_lib.ATM_SIGN_PHYSICAL if sign == "physical" else oracle_lib.ATM_SIGN_REFERENCE

    def run(r):
        s2 = lattice.System(r=r, v=s.v, m=s.m, eps=s.eps, sig=s.sig, mol_id=s.mol_id, low=s.low, high=s.high)
        o = oracle_lib.OracleSim(s2, 2.0, 2.0, nu=0.073, lj=False, atm=True, atm_mode="full", atm_sign=sg,
                                 virial_mode=oracle_lib.VIRIAL_CORRECT)
        o.update_container()
        o.forces()
        return o
    o = run(s.r.copy())
    h = 1e-6
    for atom in (0, 7, 31):
        for d in range(3):
            e = []
            for k in (1, -1):
                r = s.r.copy()
                r[atom, d] += k * h
                e.append(run(r).atm_out.energy)
            grad = (e[0] - e[1]) / (2 * h)
            expect = -grad if sign == "physical" else grad
            assert o.f[atom, d] == pytest.approx(expect, rel=1e-6, abs=1e-9)


def test_oracle_surrogate_is_consistent(oracle_lib):
    """The FP64 surrogate restatement: forces are -grad of its energy, the
    parameter gradient matches finite differences, and forces sum to zero."""
    from komd_gb300 import lattice
    rng = np.random.default_rng(0)
    params = rng.normal(0, 0.3, oracle_lib.SUR_NPARAM)
    s = lattice.argon_fcc(3, rho=0.8442, seed=2, jitter=0.1)
    fm, fs = np.zeros(32), np.ones(32)
    et, e, f = oracle_lib.sur_energy_forces(s.r, s.box, params, fm, fs, 0.1, 0.2)
    assert et == pytest.approx(e.sum())
    h = 1e-6
    for a, d in ((0, 0), (5, 1), (17, 2)):
        rp, rm = s.r.copy(), s.r.copy()
        rp[a, d] += h
        rm[a, d] -= h
        fd = -(oracle_lib.sur_energy_forces(rp, s.box, params, fm, fs, 0.1, 0.2)[0] -
               oracle_lib.sur_energy_forces(rm, s.box, params, fm, fs, 0.1, 0.2)[0]) / (2 * h)
        assert f[a, d] == pytest.approx(fd, rel=1e-6, abs=1e-9)
    assert np.abs(f.sum(0)).max() < 1e-12
    x = rng.normal(0, 1, 32)
    g = oracle_lib.sur_mlp_param_grad(params, x)
    for k in (0, 100, 2100, 6300, oracle_lib.SUR_NPARAM - 1):
        p2 = params.copy()
        p2[k] += 1e-6
        e1, _ = oracle_lib.sur_mlp(p2, x)
        p2[k] -= 2e-6
        e2, _ = oracle_lib.sur_mlp(p2, x)
        assert g[k] == pytest.approx((e1 - e2) / 2e-6, rel=1e-5, abs=1e-8)


def _file_close(got, want, name):
    """IBI's files carry 6 significant digits (FunctionPL::write, default stream format)."""
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    assert got.shape == want.shape, name
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-9, err_msg=name)


@pytest.mark.parametrize("name", ["ibirun864", "ibistop864"])
def test_oracle_ibi_plugin_matches_stock_main(oracle_lib, name):
    """The oracle's restatement of the IBI plugin (RDF sampling, U0 = -T ln g0,
    corrections, F = -dU/dr, convergence and stopping) under the stock main's
    loop with the VelocityScaling thermostat, against the files, the
    convergence log and the final checkpoint of the reference's own stock main."""
    z = load_case(name)
    sim = _sim(oracle_lib, z)
    gs = lambda k, d: z[k].item() if k in z else d   # noqa: E731
    files, conv, stopped, steps = oracle_lib.run_ibi(
        sim, float(z["p_temperature"]), int(z["p_timesteps"]), int(z["p_IBI_bins"]), float(z["p_IBI_alpha"]),
        int(z["p_IBI_steps_equil"]), int(z["p_IBI_steps_measure"]), conv_mode=str(gs("p_IBI_conv_mode", "integral")),
        conv_stop=str(gs("p_IBI_conv_stop", "worse")), conv_threshold=float(gs("p_IBI_conv_threshold", 0.99)),
        conv_window=int(gs("p_IBI_conv_window", 10)))
    assert sorted(files) == sorted(str(f)[:-4] for f in z["files"])
    for k, (x, y) in files.items():
        _file_close(np.stack([x, y], 1), z["file_" + k], f"{name}: {k}.txt")
    np.testing.assert_allclose(conv, z["conv"], rtol=1e-5)
    assert bool(stopped) == bool(z["stopped"])
    assert steps == int(z["ckpt_step"])
    assert np.abs(sim.r - z["ckpt_R"]).max() <= 1e-5 * max(1.0, np.abs(z["ckpt_R"]).max())


def test_oracle_ibi_reload_matches_stock_main(oracle_lib):
    """IBI_reload: the tabulated force read from a file replaces every functor."""
    z = load_case("ibireload864")
    sim = _sim(oracle_lib, z)
    f = z["in_force"]
    sim.use_lj = sim.use_fene = False
    sim.limit = np.inf
    sim.table = (f[:, 0].copy(), f[:, 1].copy(), 1e6, 0.0)
    t = float(z["p_temperature"])
    sim.update_container()
    sim.forces()
    sim.thermostat(t)
    for _ in range(int(z["p_timesteps"])):
        sim.integrate0()
        sim.update_container()
        sim.forces()
        sim.integrate1()
        sim.thermostat(t)
    assert int(z["ckpt_step"]) == int(z["p_timesteps"])
    assert np.abs(sim.r - z["ckpt_R"]).max() <= 1e-5 * max(1.0, np.abs(z["ckpt_R"]).max())
