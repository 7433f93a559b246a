"""Times the reference's own CPU path against the oracle's port of it, on the
same host cores, so that the port's timing (the benchmark's CPU baseline on
hosts where the reference cannot be built) can be tied to the reference.

TEST INFRASTRUCTURE ONLY.  Needs the stock main built with Kokkos' OpenMP
back end (oracle/_ref/komd_ref_main_omp, `make -C oracle/ref REF=<KoMD>`).

    python oracle/ref/calibrate_cpu.py [--threads 8] [--steps 10]

Workload: LJ + ATM argon, 32,000 atoms (FCC 20^3, rho* 0.8442, T* 0.722,
seeded), one cutoff of 2.0 for both terms (the reference has a single
cutoff), cells of 2.0, ATM by the direct cell-triple sweep (ATM_NOLIST).
The reference runs its stock main as users run it (OpenMP, pair_steps 8 and
triple_steps 4 as in its argon examples, the always-on thermostat); its time
per step is the difference of two runs of different length (so that set-up
and the first list build cancel).  The port runs the same system with the
same cutoffs and COMPAT triplets on the same number of threads.  Writes
oracle/ref/cpu_calibration.json.
"""
import argparse
import json
import os
import platform
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

STOCK_OMP = os.path.join(ROOT, "oracle", "_ref", "komd_ref_main_omp")


def reference_seconds(sysm, steps, threads):
    from komd_gb300 import komd_io, lattice
    tmp = tempfile.mkdtemp(prefix="komd_calib_")
    ps = os.path.join(tmp, "in.ps")
    komd_io.write_checkpoint(ps, sysm)
    values = dict(temperature=0.722 * 1.2027235, delta_t=0.005, cutoff=2.0, cell_size=2.0, timesteps=steps,
                  density=0.8442, limit=1e30, energy_3b=lattice.nu_star_to_energy_3b(0.073),
                  domain_low=tuple(sysm.low), domain_high=tuple(sysm.high), pair_steps=8, triple_steps=4,
                  write_freq=100000000, enable_3b=1, enable_3b_direct=1)
    with open(os.path.join(tmp, "in.dat"), "w") as fh:
        fh.write(komd_io.format_input(values, ps, [(0, 1.0 / lattice.CONV_J_EI, 1.0, 1.0)]))
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), OMP_PROC_BIND="spread", OMP_PLACES="cores")
    t0 = time.perf_counter()
    res = subprocess.run([STOCK_OMP, "in.dat"], cwd=tmp, capture_output=True, text=True, env=env)
    dt = time.perf_counter() - t0
    if res.returncode != 0:
        raise RuntimeError(res.stdout[-2000:] + res.stderr[-2000:])
    return dt


def port_seconds_per_step(sysm, steps, threads):
    import pyoracle
    pyoracle.build()
    pyoracle.set_threads(threads)
    sim = pyoracle.OracleSim(sysm, 2.0, 2.0, dt=0.005, nu=0.073, cutoff_atm=2.0, atm=True, atm_mode="compat")
    sim.update_container()
    sim.forces(listless=True)
    t0 = time.perf_counter()
    for _ in range(steps):
        sim.step(listless=True)
    return (time.perf_counter() - t0) / steps


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--steps", type=int, default=10)
    a = ap.parse_args()
    from komd_gb300 import lattice
    s = lattice.argon_fcc(20, rho=0.8442, t_star=0.722, seed=1)
    short = reference_seconds(s, 2, a.threads)
    long = reference_seconds(s, 2 + a.steps, a.threads)
    ref = (long - short) / a.steps
    port = port_seconds_per_step(s, a.steps, a.threads)
    out = {"workload": "LJ + ATM argon 32,000 atoms, one cutoff 2.0 (LJ and ATM), cells 2.0, direct ATM",
           "threads": a.threads, "host": platform.machine(), "steps": a.steps,
           "reference_s_per_step": ref, "port_s_per_step": port,
           "reference_atom_steps_per_s": s.n / ref, "port_atom_steps_per_s": s.n / port,
           "port_over_reference": ref / port,
           "reference_build": "stock main, Kokkos 4.3.1 OpenMP back end, g++ -O2, pair_steps 8, triple_steps 4",
           "port": "oracle/komd_oracle.c, OpenMP, COMPAT triplets, per-step cell lists"}
    with open(os.path.join(HERE, "cpu_calibration.json"), "w") as fh:
        json.dump(out, fh, indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
