"""The KoMD-side adapters (komd_gb300/csrc/komd_adapters/GpuKoMD.h) compile
against the reference's own headers, override its interfaces
(MoleculeContainer::init/updateContainer, ForceFunctor::handlePairList(
PairList&), Integrator::integrate0/1, TemperatureSensor::measure,
VelocityScaling::apply) and link with its library objects and
libkomd_gpu.so (oracle/ref/Makefile, target `adapters`).  The resulting
program is KoMD's start-up with the adapters registered in the Registry; it
reads a KoMD input file and checkpoint and runs Simulation::run.  Without a
GPU the engine's creation fails and the adapter reports it the way KoMD
reports errors, as a std::runtime_error with the engine's message.

Needs the reference sources (KOMD_REFERENCE_SRC, else the build container's
checkout); skipped where they are absent.
"""
import os
import subprocess

import pytest

from conftest import ROOT

REF = os.environ.get("KOMD_REFERENCE_SRC", "/root/reference")
EXE = os.path.join(ROOT, "oracle", "_ref", "komd_adapters_check")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")), reason="reference sources absent")
def test_adapters_build_against_reference_headers(tmp_path):
    from komd_gb300 import build, komd_io, lattice
    build.build()
    res = subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle", "ref"), "REF=" + REF, "adapters"],
                         capture_output=True, text=True, timeout=1200)
    assert res.returncode == 0, res.stdout[-3000:] + res.stderr[-3000:]
    assert os.path.exists(EXE)
    s = lattice.argon_fcc(5, rho=0.8442, t_star=0.722, seed=2)   # L = 8.4: three cells of 2.5
    ps = str(tmp_path / "in.ps")
    komd_io.write_checkpoint(ps, s)
    values = dict(temperature=0.868, delta_t=0.005, cutoff=2.5, cell_size=2.5, timesteps=5, limit=1e30,
                  energy_3b=0.0, domain_low=tuple(s.low), domain_high=tuple(s.high), write_freq=100000000,
                  enable_3b=0)
    (tmp_path / "in.dat").write_text(komd_io.format_input(values, ps, [(0, 1.0 / lattice.CONV_J_EI, 1.0, 1.0)]))
    out = subprocess.run([EXE, "in.dat"], capture_output=True, text=True, cwd=tmp_path, timeout=300)
    import torch
    if torch.cuda.is_available():
        assert out.returncode == 0, out.stdout + out.stderr
        assert "adapters ran: T=" in out.stdout
    else:
        # the adapter turned the engine's status into KoMD's exception
        assert out.returncode == 3, out.stdout + out.stderr
        assert "engine error:" in out.stdout and "cuda" in out.stdout.lower(), out.stdout
