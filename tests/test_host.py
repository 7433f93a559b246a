"""The C++ host layer and the `komd` executable (komd_gb300/csrc/host/):
KoMD's input parser, checkpoint IO, Registry and Simulation::run over the
engine.  CPU tests cover the parser's checks (they fail before any GPU use);
the GPU test runs a reference fixture's input end to end and lands on the
reference's thermostatted trajectory."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, case_system, load_case

EXE = os.path.join(ROOT, "komd_gb300", "_build", "komd")


@pytest.fixture(scope="module")
def komd_exe():
    from komd_gb300 import build
    build.build()
    assert os.path.exists(EXE)
    return EXE


def _write_case(tmp_path, z, extra=None, steps=None):
    from komd_gb300 import komd_io, lattice
    s = case_system(z)
    ps = str(tmp_path / "in.ps")
    komd_io.write_checkpoint(ps, s)
    values = dict(temperature=float(z["p_temperature"]), delta_t=float(z["p_delta_t"]),
                  cutoff=float(z["p_cutoff"]), cell_size=float(z["p_cell_size"]),
                  timesteps=int(steps if steps is not None else max(z["dumps"])), limit=float(z["p_limit"]),
                  energy_3b=float(z["p_energy_3b"]), domain_low=tuple(z["low"]), domain_high=tuple(z["high"]),
                  write_freq=100000000, enable_3b=int(z["p_enable_3b"]), store_checkpoint=1)
    values.update(extra or {})
    inp = tmp_path / "in.dat"
    inp.write_text(komd_io.format_input(values, ps, [(0, 1.0 / lattice.CONV_J_EI, 1.0, 1.0)]))
    return str(inp)


def test_usage_and_parser_checks(komd_exe, tmp_path):
    out = subprocess.run([komd_exe], capture_output=True, text=True)
    assert out.returncode == 0 and "Run program with" in out.stdout
    bad = tmp_path / "bad.dat"
    bad.write_text("temperature 100\ncutoff 2.5\ncell_size 2.5")
    out = subprocess.run([komd_exe, str(bad)], capture_output=True, text=True)
    assert out.returncode == 0 and "no components defined" in out.stderr
    bad.write_text("cutoff 2.5\ncell_size 2.0\ncheckpoint_file x.ps 0 0 0\nCOMP 0 1e-21 1.0 1.0 0 0 0")
    out = subprocess.run([komd_exe, str(bad)], capture_output=True, text=True)
    assert "cell size must be larger or equal to cutoff radius" in out.stderr
    bad.write_text("cutoff 2.5\ncell_size 2.5\nCOMP 0 1e-21 1.0 1.0 0 0 0")
    out = subprocess.run([komd_exe, str(bad)], capture_output=True, text=True)
    assert "No phasespace data specified" in out.stderr
    bad.write_text("cutoff 2.5\ncell_size 2.5\ncheckpoint_file x.ps 0 0 0\nCOMP 0 1e-21 1.0 1.0 0 0 0\n"
                   "gpu_precision fp16")
    out = subprocess.run([komd_exe, str(bad)], capture_output=True, text=True)
    assert "invalid value for gpu_precision" in out.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("fused", [False, True])
def test_komd_executable_follows_reference(komd_exe, tmp_path, fused):
    """thermo864: 50 thermostatted steps through FileInput, CheckpointIO,
    the adapters and Simulation::run (per-call or fused) end on the
    reference's positions (the checkpoint is written with the reference's
    6-digit stream format)."""
    from komd_gb300 import komd_io
    z = load_case("thermo864")
    inp = _write_case(tmp_path, z, extra=dict(gpu_precision="fp64"))
    cmd = [komd_exe, inp] + (["--fused"] if fused else [])
    out = subprocess.run(cmd, capture_output=True, text=True, cwd=tmp_path, timeout=300)
    assert out.returncode == 0, out.stderr
    assert "Initial temperature T=" in out.stdout
    ck = tmp_path / "ckpt_50.ps"
    assert ck.exists()
    assert not ck.read_text().endswith("\n")
    s = komd_io.read_checkpoint(str(ck), low=z["low"], high=z["high"])
    ref = z["s50_R"]
    assert np.abs(s.r - ref).max() <= 1e-5 * max(1.0, np.abs(ref).max())


@pytest.mark.gpu
def test_viscosity_sensor_matches_restatement(komd_exe, tmp_path, oracle_lib):
    """The host layer's Green-Kubo viscosity sensor against the oracle's
    restatement applied to the same per-step pressure tensors (taken through
    the C ABI along the same thermostatted FP64 trajectory)."""
    from komd_gb300 import gpu
    z = load_case("thermo864")
    steps = 30
    inp = _write_case(tmp_path, z, extra=dict(gpu_precision="fp64", enable_sensor_visc=1, sensor_visc_no_orig=1),
                      steps=steps)
    out = subprocess.run([komd_exe, inp], capture_output=True, text=True, cwd=tmp_path, timeout=300)
    assert out.returncode == 0, out.stderr
    vals = dict(ln.split(": ") for ln in (tmp_path / f"viscosity_{steps}.txt").read_text().split("\n") if ln)
    # the same loop through the Python binding
    from test_gpu_parity import gpu_for_case
    g, _ = gpu_for_case(z, precision=gpu.FP64, thermostat=0)
    t_target = float(z["p_temperature"])
    g.update_container()
    g.forces()
    g.scale_velocities(np.sqrt(t_target / g.measure(gpu.MEASURE_TEMPERATURE)["temperature"]))
    vol = float(np.prod(z["high"] - z["low"]))
    series = []
    for _ in range(steps):
        g.integrate0()
        g.update_container()
        g.forces()
        g.integrate1()
        o = g.measure(gpu.MEASURE_PRESSURE | gpu.MEASURE_TEMPERATURE)
        series.append(np.asarray(o["pressure"]) / vol)
        g.scale_velocities(np.sqrt(t_target / o["temperature"]))
    g.close()
    b, s = oracle_lib.visc_green_kubo(series, float(z["p_delta_t"]), True)
    f = oracle_lib.visc_factor(vol, t_target)
    assert float(vals["b"]) == pytest.approx(b * f, rel=1e-4)
    assert float(vals["s"]) == pytest.approx(s * f, rel=1e-4)


def _write_stock_case(tmp_path, z, extra=None):
    """The input file of a stock-main fixture (its p_* keys), the checkpoint and
    any FunctionPL files the run reads."""
    from komd_gb300 import komd_io, lattice
    ps = str(tmp_path / "in.ps")
    komd_io.write_checkpoint(ps, case_system(z))
    values = {k[2:]: z[k].item() for k in z if k.startswith("p_")}
    values.update(domain_low=tuple(z["low"]), domain_high=tuple(z["high"]))
    values.update(extra or {})
    for k in z:
        if k.startswith("in_"):   # "x\ty" per line, no trailing newline
            (tmp_path / (k[3:] + ".txt")).write_text("\n".join("%.17g\t%.17g" % (a, b) for a, b in z[k]))
    inp = tmp_path / "in.dat"
    inp.write_text(komd_io.format_input(values, ps, [(0, 1.0 / lattice.CONV_J_EI, 1.0, 1.0)]))
    return str(inp)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["ibirun864", "ibistop864", "ibireload864"])
def test_komd_ibi_plugins_follow_reference(komd_exe, tmp_path, name):
    """The IBI plugin (RDF sampling on the engine, the tabulated force swapped in
    through komd_gpu_set_terms / komd_gpu_set_pair_table, corrections and the
    convergence stop) and IBI_reload, run by `komd` on the stock-main
    fixtures' inputs: every file IBI writes, the convergence log and the final
    checkpoint match the reference's (files carry 6 significant digits)."""
    from komd_gb300 import komd_io
    z = load_case(name)
    inp = _write_stock_case(tmp_path, z, extra=dict(gpu_precision="fp64"))
    out = subprocess.run([komd_exe, inp], capture_output=True, text=True, cwd=tmp_path, timeout=300)
    assert out.returncode == 0, out.stderr
    for f in z["files"]:
        f = str(f)
        got = np.atleast_2d(np.loadtxt(tmp_path / f))
        np.testing.assert_allclose(got, z["file_" + f[:-4]], rtol=1e-5, atol=1e-9, err_msg=f)
        assert not (tmp_path / f).read_text().endswith("\n")
    conv = [float(ln.split("value=")[1]) for ln in out.stdout.splitlines() if "[IBI] Convergence: target" in ln]
    np.testing.assert_allclose(conv, z["conv"], rtol=1e-5)
    assert ("stopping criterion reached" in out.stdout) == bool(z["stopped"])
    ck = tmp_path / f"ckpt_{int(z['ckpt_step'])}.ps"
    assert ck.exists()
    s = komd_io.read_checkpoint(str(ck), low=z["low"], high=z["high"])
    assert np.abs(s.r - z["ckpt_R"]).max() <= 1e-5 * max(1.0, np.abs(z["ckpt_R"]).max())


def test_ibi_parser_checks(komd_exe, tmp_path):
    """IBI input errors are reported before any GPU use."""
    base = "cutoff 2.5\ncell_size 2.5\ncheckpoint_file x.ps 0 0 0\nCOMP 0 1e-21 1.0 1.0 0 0 0\n"
    bad = tmp_path / "bad.dat"
    bad.write_text(base + "IBI_enable 1\ngpu_skin 0.3")
    out = subprocess.run([komd_exe, str(bad)], capture_output=True, text=True)
    assert out.returncode == 1 and "gpu_skin 0" in out.stderr
    bad.write_text(base + "IBI_enable 1")
    out = subprocess.run([komd_exe, str(bad), "--fused"], capture_output=True, text=True)
    assert out.returncode == 1 and "per-step hooks" in out.stderr
    bad.write_text(base + "ADR_enable 1")
    out = subprocess.run([komd_exe, str(bad)], capture_output=True, text=True)
    assert out.returncode == 1 and "AdResS" in out.stderr


@pytest.mark.gpu
def test_komd_vtk_output(komd_exe, tmp_path):
    """gpu_vtk 1: VTK_Output_<step>.vtu at step 0 (after the first container
    update, forces still zero) and every write_freq steps, sites in molecule
    order; the last one holds the final checkpoint's state in Float32."""
    from komd_gb300 import komd_io
    z = load_case("thermo864")
    inp = _write_case(tmp_path, z, extra=dict(gpu_precision="fp64", gpu_vtk=1, write_freq=25))
    out = subprocess.run([komd_exe, inp], capture_output=True, text=True, cwd=tmp_path, timeout=300)
    assert out.returncode == 0, out.stderr
    assert sorted(p.name for p in tmp_path.glob("VTK_Output_*.vtu")) == [
        "VTK_Output_0000.vtu", "VTK_Output_0025.vtu", "VTK_Output_0050.vtu"]
    d0 = komd_io.read_vtu(str(tmp_path / "VTK_Output_0000.vtu"))
    assert np.array_equal(d0["points"], z["r0"].astype(np.float32))
    assert np.array_equal(d0["velocity"], z["v0"].astype(np.float32))
    assert not d0["force"].any()
    assert np.array_equal(d0["id"], z["mol_id"].astype(np.int64))
    d50 = komd_io.read_vtu(str(tmp_path / "VTK_Output_0050.vtu"))
    ck = komd_io.read_checkpoint(str(tmp_path / "ckpt_50.ps"), low=z["low"], high=z["high"])
    np.testing.assert_allclose(d50["points"], ck.r, rtol=1e-5, atol=1e-5)
    assert np.isfinite(d50["force"]).all() and np.abs(d50["force"]).max() > 0


@pytest.mark.gpu
def test_komd_sensor_files_follow_reference(komd_exe, tmp_path):
    """sensors864: the reference's stock main with the LJ, pressure and
    viscosity sensors on wrote pot_LJ12_6_<step> (the U(r) and F(r) histogram
    means of LJ12_6_Sensor / Potential_Sensor), pot_history_LJ12_6_<step>,
    pressures_<step> and viscosity_<step> (the Green-Kubo integrals of
    ViscositySensor) every 10 steps.  `komd` on the same input writes the same
    files with the same numbers (6 printed digits; empty histogram bins are
    NaN on both sides)."""
    def file_tokens(path):   # as tests/golden/make_golden.py reads them: labels skipped, "-nan" is NaN
        with open(path) as fh:
            return np.array([float(t) for t in fh.read().split() if not t.endswith(":")])

    z = load_case("sensors864")
    inp = _write_stock_case(tmp_path, z, extra=dict(gpu_precision="fp64"))
    out = subprocess.run([komd_exe, inp], capture_output=True, text=True, cwd=tmp_path, timeout=300)
    assert out.returncode == 0, out.stderr
    for f in z["files"]:
        f = str(f)
        assert (tmp_path / f).exists(), f
        got = file_tokens(str(tmp_path / f))
        ref = z["tok_" + f[:-4]]
        assert got.shape == ref.shape, f
        # viscosity: correlation sums of the pressure series (6 digits each side)
        rtol = 2e-4 if f.startswith("viscosity") else 2e-5
        np.testing.assert_allclose(got, ref, rtol=rtol, atol=1e-9 * np.nanmax(np.abs(ref)), err_msg=f)


def test_phasespace_generator_follows_reference(komd_exe, tmp_path):
    """ps_gen_region (util/PhasespaceGenerator.cpp:27-95): `komd --phasespace`
    writes the generated molecules of the psgen3site input -- a bent
    three-site component on the generator's grid, random Euler rotations from
    the static engine seeded 43, Maxwell-Boltzmann velocities from the one
    seeded 42 -- and they equal the reference's generated state (dumped by
    the harness at step 0) to the last bit.  CPU only: the mode stops before
    any GPU work."""
    from komd_gb300 import komd_io
    z = load_case("psgen3site")
    comps = [(int(c[0]), float(c[1]), float(c[2]), float(c[3]), tuple(c[4:7])) for c in z["comps"]]
    regions = [(tuple(r[0:3]), tuple(r[3:6]), int(r[6])) for r in z["regions"]]
    values = {k[2:]: z[k].item() for k in z if k.startswith("p_") and k != "p_thermostat"}
    values.update(domain_low=tuple(z["low"]), domain_high=tuple(z["high"]), timesteps=5)
    inp = tmp_path / "in.dat"
    inp.write_text(komd_io.format_input(values, None, comps, regions))
    out = subprocess.run([komd_exe, str(inp), "--phasespace", str(tmp_path / "gen.ps")], capture_output=True,
                         text=True, cwd=tmp_path, timeout=120)
    assert out.returncode == 0, out.stderr
    s = komd_io.read_checkpoint(str(tmp_path / "gen.ps"), low=z["low"], high=z["high"])
    assert s.n == z["s0_R"].shape[0]
    assert np.array_equal(s.r, z["s0_R"])
    assert np.array_equal(s.v, z["s0_V"])
    assert np.array_equal(np.unique(s.mol_id), np.arange(1, s.n // 3 + 1))   # ids 1.. as Molecule::NEXT_ID gives
