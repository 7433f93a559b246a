"""The C ABI library loads and exports every entry point include/komd_gpu.h
declares (CPU only: no compute call is made)."""
import ctypes
import os
import re

from conftest import ROOT


def declared_symbols():
    with open(os.path.join(ROOT, "include", "komd_gpu.h")) as fh:
        text = fh.read()
    return sorted(set(re.findall(r"\b(komd_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from komd_gb300 import build, gpu
    build.build()
    lib = ctypes.CDLL(gpu.library_path())
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # the Python binding covers the same surface
    assert set(syms) <= set(gpu.EXPORTS) | {s for s in syms if s not in gpu.EXPORTS and hasattr(lib, s)}


def test_abi_version_and_error_reporting_without_gpu():
    from komd_gb300 import gpu
    lib = gpu.load()
    assert lib.komd_gpu_abi_version() == 2
    # argument validation happens before any device work
    cfg = gpu.make_config([0, 0, 0], [5, 5, 5], 2.5, cutoff=2.5)    # only 2 cells per dimension
    h = ctypes.c_void_p()
    rc = lib.komd_gpu_create(ctypes.byref(cfg), 0, ctypes.byref(h))
    assert rc == 1
    assert b"at least 3 domain cells" in lib.komd_gpu_last_error()
    cfg = gpu.make_config([0, 0, 0], [20, 20, 20], 2.0, cutoff=2.5)  # cell smaller than cutoff
    assert lib.komd_gpu_create(ctypes.byref(cfg), 0, ctypes.byref(h)) == 1
    assert b"cell size" in lib.komd_gpu_last_error()
    cfg = gpu.make_config([0, 0, 0], [20, 20, 20], 2.5, cutoff=2.5, thermostat=1)   # no target temperature
    assert lib.komd_gpu_create(ctypes.byref(cfg), 0, ctypes.byref(h)) == 1
    assert b"temperature_target" in lib.komd_gpu_last_error()
    cfg = gpu.make_config([0, 0, 0], [20, 20, 20], 2.8, cutoff=2.5, terms=gpu.TERM_TABULATED, skin=0.3)
    assert lib.komd_gpu_create(ctypes.byref(cfg), 0, ctypes.byref(h)) == 1
    assert b"tabulated" in lib.komd_gpu_last_error()
    cfg = gpu.make_config([0, 0, 0], [20, 20, 20], 2.5, cutoff=2.5, terms=gpu.TERM_ATM2B)   # ATM2B without LJ
    assert lib.komd_gpu_create(ctypes.byref(cfg), 0, ctypes.byref(h)) == 1
    assert b"ATM2B" in lib.komd_gpu_last_error()
    b = ctypes.c_void_p()
    assert lib.komd_batch_create(None, 0, 1, 1, None, ctypes.byref(b)) == 1   # no replicas


def test_sci_temperature_returns_for_every_input():
    """The SciValue temperature conversion is bounded: the device thermostat
    evaluates it inside the step graph, where an infinite kinetic sum (an
    overflowed force upstream) must not spin.  The host instantiation is the
    same function; each call runs in a child process under a time limit."""
    import subprocess
    import sys
    code = (
        "import math, sys; sys.path.insert(0, %r)\n"
        "from komd_gb300 import gpu\n"
        "L = gpu.load()\n"
        "for mv2 in (float('inf'), float('-inf'), float('nan'), 1e308, 0.0, 5e-324, -1e308):\n"
        "    t = L.komd_sci_temperature(mv2, 4000.0)\n"
        "    print(mv2, t)\n"
        "assert math.isinf(L.komd_sci_temperature(float('inf'), 4000.0))\n"
        "assert math.isnan(L.komd_sci_temperature(float('nan'), 4000.0))\n"
        "assert L.komd_sci_temperature(0.0, 4000.0) == 0.0\n"
        "assert L.komd_sci_temperature(1.0, 0.0) == 0.0\n"
        "assert math.isfinite(L.komd_sci_temperature(1e308, 4000.0))\n"
    ) % ROOT
    res = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stdout + res.stderr


def test_sci_temperature_matches_the_oracle():
    """Finite inputs keep the reference's SciValue rounding (the oracle is
    pinned to the reference's TemperatureSensor bit for bit)."""
    import numpy as np
    from komd_gb300 import gpu, lattice
    import pyoracle
    lib = gpu.load()
    s = lattice.argon_fcc(3, rho=0.8442, t_star=0.722, seed=3)
    sim = pyoracle.OracleSim(s, 2.5, 2.5, dt=0.005)
    sim.update_container()
    t_ref = sim.temperature()
    mv2 = 0.0
    for k in range(s.n):   # the oracle's summation order, site by site
        vx, vy, vz = (float(c) for c in sim.v[k])
        mv2 += float(sim.m[k]) * (vx * vx + vy * vy + vz * vz)
    t = lib.komd_sci_temperature(mv2, float(s.n))
    assert t == t_ref, (t, t_ref)
