"""Small fixed workloads for kernel profiling (ncu) and quick timing.

    python -m komd_gb300.profile_cases exact      [--ncell 40] [--steps 3] [--equil 0] [--skin 0.3] [--cell 2.8]
    python -m komd_gb300.profile_cases surrogate  [--ncell 40] [--steps 3]
    python -m komd_gb300.profile_cases replicas   [--count 64] [--steps 2] [--equil 0] [--groups 4]
    python -m komd_gb300.profile_cases tabulated  [--ncell 40] [--steps 3]
    python -m komd_gb300.profile_cases train      [--snaps 40] [--epochs 2] [--batch 4]

`exact`: LJ + FULL ATM argon (rho* 0.8442, T* 0.722, rc 2.5 / 2.0, nu* 0.073,
cell 2.8, skin 0.3 by default; the benchmark's timed configuration is
--skin 0.4 --cell 0 (cell 0: the smallest edge >= 2.5 + skin that divides the
box) --equil 400).  `surrogate`: the
same with the learned three-body term on Glorot-initialised weights (kernel
cost does not depend on the weights).  `replicas`: the first `count` of the
benchmark's uneven replicas (2000-20000 atoms) advanced by one batched graph
(`groups` packed groups) after `equil` steps.  `tabulated`: the IBI
tabulated pair force (FP64, per-step cells of edge >= 2.5, a 200-node table
of the LJ force) on the jittered lattice, then one RDF_Profiler sample (100
bins to 2.5).  `train`: force-matched training of the learned term on a small
dataset from the exact kernel.  Each prints its mean step
time; the launches before the measured steps are few, so that a profiler can
skip to them.
"""
from __future__ import annotations

import argparse
import time

import numpy as np

from . import gpu, lattice, surrogate


def exact(ncell, steps, equil, learned=False, skin=0.3, cell=2.8):
    s = lattice.argon_fcc(ncell, rho=0.8442, t_star=0.722, seed=1)
    terms = gpu.TERM_LJ | gpu.TERM_ATM | (gpu.TERM_ATM_SURROGATE if learned else 0)
    if cell <= 0:
        side = float(np.min(s.high - s.low))
        cell = side / np.floor(side / (2.5 + skin))
    g = gpu.GpuSystem(s, surrogate.physics_config(s, cell, skin=skin, terms=terms))
    g.update_container()
    g.forces()
    if learned:
        x, e3, _ = g.surrogate_sample()
        model = dict(params=surrogate.init_params(1), fmean=x.mean(0).astype(np.float32),
                     fstd=(x.std(0) + 1e-6).astype(np.float32), e_scale=float(e3.std()), e_shift=float(e3.mean()))
        g.surrogate_load(model, probe_every=0)
        g.forces()
    if equil:
        g.step(equil)
    t0 = time.perf_counter()
    g.step(steps)
    dt = (time.perf_counter() - t0) / steps
    print(f"{'surrogate' if learned else 'exact'} n={s.n}: {dt * 1e3:.3f} ms/step (host clock)")
    g.close()


def replicas(count, steps, equil=0, groups=4):
    reps = []
    for seed, n, rho, t_star in lattice.replica_specs(count, 2027):   # the benchmark's replicas
        s = lattice.trimmed_fcc(n, rho, t_star, seed)
        L = float(s.high[0])
        g = gpu.GpuSystem(s, surrogate.physics_config(s, L / np.floor(L / 2.8), skin=0.3))
        g.update_container()
        g.forces()
        reps.append(g)
    b = gpu.Batch(reps, n_streams=groups, steps_per_graph=1)
    if equil:
        b.step(equil)
    t0 = time.perf_counter()
    b.step(steps)
    dt = (time.perf_counter() - t0) / steps
    print(f"replicas x{count}: {dt * 1e3:.3f} ms/step (host clock)")
    b.close()
    for g in reps:
        g.close()


def train(snaps, epochs, batch):
    """Force-matched training on the GPU: a dataset of `snaps` snapshots of 500
    sites from the exact kernel (the benchmark's training set is 2000), then
    `epochs` passes of Adam steps over `batch` snapshots each (the network's
    kernels on the tensor cores)."""
    data = surrogate.capture(n_points=max(1, snaps // 10), snaps_per_point=10, ncell=5, equil=20, every=5)
    t0 = time.perf_counter()
    model = surrogate.fit_forces(data, epochs=epochs, snaps_per_batch=batch)
    dt = time.perf_counter() - t0
    print(f"train: {data.snapshots} snapshots x {data.sites} sites, {epochs} epochs: {dt:.3f} s "
          f"(loss {model['loss'][-1].tolist()})")
    data.close()


def tabulated(ncell, steps):
    s = lattice.argon_fcc(ncell, rho=0.8442, t_star=0.722, seed=3, jitter=0.02)
    side = float(np.min(s.high - s.low))
    cell = side / np.floor(side / 2.5)
    g = gpu.GpuSystem(s, gpu.make_config(s.low, s.high, cell, cutoff=2.5, terms=gpu.TERM_TABULATED,
                                         precision=gpu.FP64))
    x = np.linspace(0.6, 2.5, 200)
    g.set_pair_table(x, 24.0 * (2.0 * x ** -13 - x ** -7), 1e6, 0.0)
    g.update_container()
    g.forces()
    t0 = time.perf_counter()
    g.step(steps)
    dt = (time.perf_counter() - t0) / steps
    g.rdf_profile(2.5, 100)
    print(f"tabulated n={s.n}: {dt * 1e3:.3f} ms/step (host clock)")
    g.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["exact", "surrogate", "replicas", "tabulated", "train"])
    ap.add_argument("--ncell", type=int, default=40)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--equil", type=int, default=0)
    ap.add_argument("--count", type=int, default=64)
    ap.add_argument("--groups", type=int, default=4)
    ap.add_argument("--snaps", type=int, default=40)
    ap.add_argument("--epochs", type=int, default=2)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--skin", type=float, default=0.3)
    ap.add_argument("--cell", type=float, default=2.8)
    a = ap.parse_args()
    if a.case == "train":
        train(a.snaps, a.epochs, a.batch)
    elif a.case == "replicas":
        replicas(a.count, a.steps, a.equil, a.groups)
    elif a.case == "tabulated":
        tabulated(a.ncell, a.steps)
    else:
        exact(a.ncell, a.steps, a.equil, learned=a.case == "surrogate", skin=a.skin, cell=a.cell)


if __name__ == "__main__":
    main()
