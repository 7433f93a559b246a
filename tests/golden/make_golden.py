"""Generates the golden fixtures under tests/golden/ by running the reference.

The reference harness (oracle/ref/harness.cpp, built by oracle/ref/Makefile
from the reference's own sources into oracle/_ref/) is fed seeded synthetic
inputs in KoMD's own input and checkpoint formats (the plugin cases run the
reference's unmodified stock main, oracle/_ref/komd_ref_main, on whole input
files); its dumps (positions,
velocities, forces, cell lists incl. halo copies, neighbour counts,
temperature, LJ potential, pressure tensor, RDF histogram) are stored as
compressed .npz files together with the inputs that produced them.

Run from the repo root in a container where the reference is present:

    make -C oracle/ref REF=<KoMD checkout> -j8 && python tests/golden/make_golden.py [case ...]

The fixtures are then read by the tests without the reference.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from komd_gb300 import lattice, komd_io  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "komd_ref_harness")
STOCK = os.path.join(ROOT, "oracle", "_ref", "komd_ref_main")
OUT = os.path.dirname(os.path.abspath(__file__))
EPS_J = 1.0 / lattice.CONV_J_EI          # eps* = 1 as the COMP line's Joule value


def parse_dump(path):
    steps = {}
    with open(path) as fh:
        lines = fh.read().split("\n")
    i = 0
    cur = None
    while i < len(lines):
        ln = lines[i].split()
        i += 1
        if not ln:
            continue
        key = ln[0]
        if key == "STEP":
            cur = steps.setdefault(int(ln[1]), {})
        elif key in ("R", "V", "F"):
            n = int(ln[1])
            cur[key] = np.array([[float(x) for x in lines[i + k].split()] for k in range(n)]).reshape(n, 3)
            i += n
        elif key == "CELLS":
            n = int(ln[1])
            counts, idx = [], []
            for k in range(n):
                p = [int(x) for x in lines[i + k].split()]
                counts.append(p[0])
                idx.extend(p[1:])
            cur["cell_count"] = np.array(counts, np.int64)
            cur["cell_idx"] = np.array(idx, np.int64)
            i += n
        elif key == "NCOUNT":
            n = int(ln[1])
            cur["ncount"] = np.array([int(lines[i + k]) for k in range(n)], np.int64)
            i += n
        elif key == "PRESSURE":
            cur["pressure"] = np.array([float(lines[i + k]) for k in range(6)])
            i += 6
        elif key == "IBIRDF":
            n = int(ln[1])
            cur["ibirdf"] = np.array([float(lines[i + k]) for k in range(n)])
            i += n
        elif key == "LJHIST":
            n = int(ln[1])
            cur["ljhist"] = np.array([[float(x) for x in lines[i + k].split()] for k in range(n)]).T.copy()
            i += n
        elif key in ("TEMP", "UPOT"):
            cur[key.lower()] = float(ln[1])
        elif key == "NPAIRS":
            cur["npairs"] = int(ln[1])
    return steps


def run_case(name, sysm, values, steps, dumps, comps=None, thermostat=False, table=None, regions=()):
    tmp = tempfile.mkdtemp(prefix=f"komd_golden_{name}_")
    try:
        ps = None
        if sysm is not None:   # else the phase space comes from ps_gen_region entries alone
            ps = os.path.join(tmp, "in.ps")
            komd_io.write_checkpoint(ps, sysm)
        comps = comps or [(0, EPS_J, 1.0, 1.0)]
        with open(os.path.join(tmp, "in.dat"), "w") as fh:
            fh.write(komd_io.format_input(values, ps, comps, regions))
        env = dict(os.environ, KOMD_HARNESS_THERMOSTAT="1" if thermostat else "0")
        if table is not None:
            tab = os.path.join(tmp, "force.txt")
            with open(tab, "w") as fh:   # FunctionPL::write layout: "x\ty" per line
                fh.write("\n".join("%.17g\t%.17g" % (x, y) for x, y in zip(*table)))
            env["KOMD_HARNESS_IBI_TABLE"] = tab
        res = subprocess.run([HARNESS, "in.dat", "out.txt", str(steps)] + [str(d) for d in dumps], cwd=tmp,
                             capture_output=True, text=True, env=env)
        if res.returncode != 0:
            raise RuntimeError(f"{name}: harness failed\n{res.stdout}\n{res.stderr}")
        dump = parse_dump(os.path.join(tmp, "out.txt"))
        arrays = dict(low=np.asarray(values["domain_low"], float), high=np.asarray(values["domain_high"], float),
                      dumps=np.array(dumps, np.int64))
        if sysm is not None:
            arrays.update(r0=sysm.r, v0=sysm.v, m=sysm.m, eps=sysm.eps, sig=sysm.sig, mol_id=sysm.mol_id)
        if regions:
            arrays["regions"] = np.array([[*b, *e, c] for b, e, c in regions], float)
            arrays["comps"] = np.array([[c[0], c[1], c[2], c[3], *c[4]] for c in comps], float)
        arrays["p_thermostat"] = np.int64(1 if thermostat else 0)
        if table is not None:
            arrays["table_x"], arrays["table_y"] = np.asarray(table[0]), np.asarray(table[1])
        for k in ("cutoff", "cell_size", "delta_t", "limit", "energy_3b", "stiffness", "sensor_rdf_max",
                  "sensor_rdf_dr", "temperature", "density"):
            if k in values:
                arrays["p_" + k] = np.float64(values[k])
        for k in ("enable_3b", "enable_3b_direct", "enable_sensor_rdf", "enable_sensor_lj", "enable_sensor_pres",
                  "enable_3b_approx"):
            if k in values:
                arrays["p_" + k] = np.int64(values[k])
        for s, d in dump.items():
            for k, v in d.items():
                arrays[f"s{s}_{k}"] = np.asarray(v)
            rdf = os.path.join(tmp, f"rdf_{s}.txt")
            if os.path.exists(rdf):
                tab = np.loadtxt(rdf)
                arrays[f"s{s}_rdf"] = tab[:, 2].copy()
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **arrays)
        n = sysm.n if sysm is not None else len(dump[dumps[0]]["R"])
        print(f"{name}: n={n} steps={steps} dumps={dumps} -> {name}.npz")
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def file_tokens(path):
    """The numbers of a sensor file in reading order; labels such as the
    viscosity file's "b:" are skipped, the reference's "-nan" reads as NaN."""
    with open(path) as fh:
        return np.array([float(t) for t in fh.read().split() if not t.endswith(":")])


def run_stock(name, sysm, values, comps=None, tables=None, tokens=False):
    """Runs the reference's unmodified stock main (oracle/_ref/komd_ref_main)
    on a whole input file (plugins included) and stores every text file it
    writes (IBI's rdf_/pot_/force_/update_<iteration>.txt, final_pot.txt), the
    final checkpoint and the IBI convergence log lines."""
    tmp = tempfile.mkdtemp(prefix=f"komd_golden_{name}_")
    try:
        ps = os.path.join(tmp, "in.ps")
        komd_io.write_checkpoint(ps, sysm)
        comps = comps or [(0, EPS_J, 1.0, 1.0)]
        arrays = dict(r0=sysm.r, v0=sysm.v, m=sysm.m, eps=sysm.eps, sig=sysm.sig, mol_id=sysm.mol_id,
                      low=np.asarray(values["domain_low"], float), high=np.asarray(values["domain_high"], float))
        for fname, (x, y) in (tables or {}).items():   # FunctionPL files read by the run
            with open(os.path.join(tmp, fname), "w") as fh:
                fh.write("\n".join("%.17g\t%.17g" % (a, b) for a, b in zip(x, y)))
            arrays["in_" + fname.replace(".txt", "")] = np.stack([np.asarray(x), np.asarray(y)], 1)
        with open(os.path.join(tmp, "in.dat"), "w") as fh:
            fh.write(komd_io.format_input(values, ps, comps))
        res = subprocess.run([STOCK, "in.dat"], cwd=tmp, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"{name}: stock main failed\n{res.stdout[-2000:]}\n{res.stderr[-2000:]}")
        for k, v in values.items():
            if isinstance(v, (tuple, list)):
                continue
            arrays["p_" + k] = np.asarray(v) if not isinstance(v, str) else np.asarray(v)
        conv = [float(ln.split("value=")[1]) for ln in res.stdout.splitlines() if "[IBI] Convergence: target" in ln]
        arrays["conv"] = np.asarray(conv, float)
        arrays["stopped"] = np.int64("stopping criterion reached" in res.stdout)
        names = sorted(f for f in os.listdir(tmp) if f.endswith(".txt") and f not in (tables or {}))
        arrays["files"] = np.asarray(names)
        for f in names:
            if tokens:   # sensor files with ragged rows or labels: their numbers in order
                arrays["tok_" + f[:-4]] = file_tokens(os.path.join(tmp, f))
            else:
                arrays["file_" + f[:-4]] = np.atleast_2d(np.loadtxt(os.path.join(tmp, f)))
        ck = [f for f in os.listdir(tmp) if f.startswith("ckpt_") and f.endswith(".ps")]
        if len(ck) != 1:
            raise RuntimeError(f"{name}: expected one checkpoint, found {ck}")
        arrays["ckpt_step"] = np.int64(int(ck[0][5:-3]))
        arrays["ckpt_R"] = komd_io.read_checkpoint(os.path.join(tmp, ck[0]), low=values["domain_low"],
                                                   high=values["domain_high"]).r
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **arrays)
        print(f"{name}: n={sysm.n} files={names} ckpt={ck[0]} conv={conv} -> {name}.npz")
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def base_values(sysm, cutoff, cell, dt, steps, **kw):
    v = dict(temperature=100.0, delta_t=dt, cutoff=cutoff, cell_size=cell, timesteps=steps, density=0.8,
             limit=1e30, energy_3b=0.0, domain_low=tuple(sysm.low), domain_high=tuple(sysm.high),
             pair_steps=1, triple_steps=1, write_freq=100000000, enable_3b=0, enable_3b_direct=1,
             enable_sensor_lj=1, enable_sensor_pres=1, enable_sensor_rdf=0)
    v.update(kw)
    return v


def main(selected):
    if not os.path.exists(HARNESS) or not os.path.exists(STOCK):
        raise SystemExit("build the reference harness and stock main first: make -C oracle/ref -j8")
    e3b = lattice.nu_star_to_energy_3b(0.073)

    def lj864():
        # plain LJ argon, 864 atoms, jittered FCC, rc = cell = 2.5, RDF 200 bins
        s = lattice.argon_fcc(6, rho=0.8442, t_star=0.722, seed=11, jitter=0.05)
        run_case("lj864", s, base_values(s, 2.5, 2.5, 0.005, 100, enable_sensor_rdf=1, sensor_rdf_max=2.5,
                                          sensor_rdf_dr=0.0125), 100, [0, 1, 100])

    def ljatm864():
        # LJ + ATM (direct enumeration), single cutoff 2.0 (the reference has one cutoff)
        s = lattice.argon_fcc(6, rho=0.8442, t_star=0.722, seed=12, jitter=0.05)
        run_case("ljatm864", s, base_values(s, 2.0, 2.0, 0.005, 20, enable_3b=1, enable_3b_direct=1,
                                             energy_3b=e3b), 20, [0, 1, 20])

    def atmlist500():
        # ATM via the triplet list (ATM + ATM_Pressure), 500 atoms, stretched last cell
        s = lattice.argon_fcc(5, rho=0.8442, t_star=0.722, seed=13, jitter=0.05)
        run_case("atmlist500", s, base_values(s, 2.0, 2.0, 0.005, 5, enable_3b=1, enable_3b_direct=0,
                                               energy_3b=e3b), 5, [0, 1, 5])

    def fene375():
        # three-site molecules with FENE (all same-molecule pairs) and intermolecular LJ
        s = lattice.triatomic_sc(5, rho_site=0.25, t_star=0.5, seed=14, r0=0.97, theta0_deg=90.0)
        run_case("fene375", s, base_values(s, 2.5, 2.5, 0.002, 20, stiffness=30.0), 20, [0, 1, 20])

    def edge_box():
        # non-cubic box, non-zero domain_low, atoms on the domain faces, hot gas so
        # that sites cross the periodic boundary; small force clamp (Limit)
        rng = np.random.default_rng(15)
        low = np.array([-2.0, 0.5, 1.0])
        box = np.array([10.3, 11.1, 9.7])
        g = np.stack(np.meshgrid(*(np.arange(int(b // 1.15)) for b in box), indexing="ij"), -1).reshape(-1, 3)
        r = low + (g + 0.5) * (box / np.floor(box / 1.15)) + rng.normal(0, 0.04, g.shape)
        r[0] = low                  # exactly on the low corner
        r[1] = low + box * np.array([1.0, 0.5, 0.5])   # exactly on the high x face
        n = r.shape[0]
        s = lattice.System(r=r, v=lattice.maxwell_boltzmann(n, 2.0, np.ones(n), rng), m=np.ones(n),
                           eps=np.ones(n), sig=np.ones(n), mol_id=np.arange(1, n + 1, dtype=np.uint64), low=low,
                           high=low + box)
        run_case("edge_box", s, base_values(s, 2.5, 2.5, 0.004, 50, limit=40.0), 50, [0, 1, 50])

    def atm2b864():
        # ATM2B effective pair force (enable_3b_approx) in place of LJ12_6, nu* = 0.073
        s = lattice.argon_fcc(6, rho=0.8442, t_star=0.722, seed=16, jitter=0.05)
        run_case("atm2b864", s, base_values(s, 2.5, 2.5, 0.005, 20, enable_3b_approx=1, energy_3b=e3b),
                 20, [0, 1, 20])

    def thermo864():
        # the always-on VelocityScaling thermostat: target 1.2 K (T* ~ 1.0) from T* = 0.722
        s = lattice.argon_fcc(6, rho=0.8442, t_star=0.722, seed=17, jitter=0.05)
        run_case("thermo864", s, base_values(s, 2.5, 2.5, 0.005, 50, temperature=1.2), 50, [0, 1, 50],
                 thermostat=True)

    def ibi864():
        # tabulated pair force (IBI_ForceFunctor) in place of LJ: the LJ force
        # sampled on IBI_bins = 100 nodes (i + 1/2) * 2.5/100, linear in between;
        # plus the RDF_Profiler histogram (100 bins to the cutoff)
        s = lattice.argon_fcc(6, rho=0.8442, t_star=0.722, seed=18, jitter=0.05)
        x = (np.arange(100) + 0.5) * 2.5 / 100
        y = 24.0 * (2.0 * x ** -13 - x ** -7)
        run_case("ibi864", s, base_values(s, 2.5, 2.5, 0.005, 20), 20, [0, 1, 20], table=(x, y))

    def ibi_values(s, steps, **kw):
        v = dict(temperature=1.2, delta_t=0.005, cutoff=2.5, cell_size=2.5, timesteps=steps, density=0.8,
                 limit=1e30, energy_3b=0.0, domain_low=tuple(s.low), domain_high=tuple(s.high), pair_steps=1,
                 triple_steps=1, write_freq=100000000, enable_3b=0, enable_3b_direct=1, store_checkpoint=1)
        v.update(kw)
        return v

    def ibirun864():
        # the IBI plugin under the stock main: 9 RDF samples with LJ, then
        # U0 = -T ln g0 as a tabulated force and three correction iterations
        # (5 equilibration + 10 measurement steps each); integral criterion
        s = lattice.argon_fcc(6, rho=0.8442, t_star=0.722, seed=19, jitter=0.05)
        run_stock("ibirun864", s, ibi_values(s, 60, IBI_enable=1, IBI_bins=50, IBI_alpha=0.2, IBI_steps_equil=5,
                                             IBI_steps_measure=10))

    def ibistop864():
        # l2 criterion with a 2-iteration window under a loose threshold: the
        # plugin stops the run after the second iteration (Simulation::stop)
        s = lattice.argon_fcc(6, rho=0.8442, t_star=0.722, seed=20, jitter=0.05)
        run_stock("ibistop864", s, ibi_values(s, 80, IBI_enable=1, IBI_bins=40, IBI_alpha=0.3, IBI_steps_equil=4,
                                              IBI_steps_measure=8, IBI_conv_mode="l2", IBI_conv_stop="window",
                                              IBI_conv_window=2, IBI_conv_threshold=1e6))

    def ibireload864():
        # IBI_reload: a tabulated force and potential read from files replace
        # every functor from the first step (no exclusion zone)
        s = lattice.argon_fcc(6, rho=0.8442, t_star=0.722, seed=21, jitter=0.05)
        x = (np.arange(60) + 0.5) * 2.5 / 60
        f = 24.0 * (2.0 * x ** -13 - x ** -7)
        u = 4.0 * (x ** -12 - x ** -6)
        run_stock("ibireload864", s, ibi_values(s, 30, IBI_reload=1, IBI_bins=60, IBI_reload_fpath="force.txt",
                                                IBI_reload_ppath="pot.txt"),
                  tables={"force.txt": (x, f), "pot.txt": (x, u)})

    def psgen3site():
        # PhasespaceGenerator (ps_gen_region, no checkpoint): a bent three-site
        # component on the generator's grid at density 0.05 per cubic Angstrom in
        # a 14 x 14 x 14 box, rotated at random, Maxwell-Boltzmann at 120 K;
        # the harness dumps the generated state at step 0 (and after 5 steps)
        box = 14.0
        comps = [(0, EPS_J, 1.0, 1.0, (0.0, 0.0, 0.0)), (0, EPS_J, 1.0, 1.0, (0.97, 0.0, 0.0)),
                 (0, EPS_J, 1.0, 1.0, (-0.3, 0.92, 0.0))]
        values = base_values(lattice.System(r=np.zeros((1, 3)), v=np.zeros((1, 3)), m=np.ones(1), eps=np.ones(1),
                                            sig=np.ones(1), mol_id=np.ones(1, np.uint64), low=np.zeros(3),
                                            high=np.full(3, box)),
                             2.5, 2.8, 0.002, 5, density=0.05, temperature=120.0, stiffness=30.0)
        run_case("psgen3site", None, values, 5, [0, 5], comps=comps,
                 regions=[((0.0, 0.0, 0.0), (box, box, box), 0)])

    def sensors864():
        # the stock main with the LJ, pressure and viscosity sensors on (and the
        # always-on thermostat): every file they write at write_freq 10 over 30 steps
        # -- pot_LJ12_6_<step> (U(r), F(r) histogram means), pot_history_LJ12_6_<step>,
        # pressures_<step>, viscosity_<step> (Green-Kubo over the per-step tensors)
        s = lattice.argon_fcc(6, rho=0.8442, t_star=0.722, seed=22, jitter=0.05)
        run_stock("sensors864", s, ibi_values(s, 30, write_freq=10, enable_sensor_lj=1, enable_sensor_pres=1,
                                              enable_sensor_visc=1, sensor_visc_no_orig=1, sensor_lj_bins=60),
                  tokens=True)

    cases = dict(psgen3site=psgen3site, sensors864=sensors864, ibirun864=ibirun864, ibistop864=ibistop864, ibireload864=ibireload864, ibi864=ibi864, lj864=lj864, ljatm864=ljatm864, atmlist500=atmlist500, fene375=fene375, edge_box=edge_box,
                 atm2b864=atm2b864, thermo864=thermo864)
    for name in (selected or list(cases)):
        cases[name]()


if __name__ == "__main__":
    main(sys.argv[1:])
