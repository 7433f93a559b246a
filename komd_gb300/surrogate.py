"""Learned three-body term: data generation, training and evaluation.

The exact ATM kernel generates the training set: seeded LJ + ATM runs at
state points drawn from T* in [0.6, 1.2] and rho* in [0.75, 0.9], each started
on an FCC lattice (so lattice-like and liquid configurations are both
present), sampled every few steps.  Two trainers run on the GPU with the engine's own kernels:
fit_forces (komd_sur_fit) matches the exact three-body forces and the exact
per-site energies V/3 per vertex on snapshots kept on the device; fit
(komd_mlp_train) regresses per-site energies only.  Inference and forces run
in the engine (KOMD_TERM_ATM_SURROGATE).
"""
from __future__ import annotations

import time

import numpy as np

from . import gpu, lattice

NFEAT, NPARAM, HIDDEN = gpu.SUR_NFEAT, gpu.SUR_NPARAM, 64


def init_params(seed: int) -> np.ndarray:
    """Glorot-uniform weights, zero biases (layout W1 b1 W2 b2 w3 b3)."""
    rng = np.random.default_rng(seed)

    def glorot(o, i):
        a = np.sqrt(6.0 / (o + i))
        return rng.uniform(-a, a, (o, i))
    parts = [glorot(HIDDEN, NFEAT).ravel(), np.zeros(HIDDEN), glorot(HIDDEN, HIDDEN).ravel(), np.zeros(HIDDEN),
             glorot(1, HIDDEN).ravel(), np.zeros(1)]
    p = np.concatenate(parts).astype(np.float32)
    assert p.size == NPARAM
    return p


def physics_config(s, cell, nu=0.073, rc3=2.0, rc=2.5, dt=0.005, terms=None, skin=0.0):
    t = gpu.TERM_LJ | gpu.TERM_ATM if terms is None else terms
    return gpu.make_config(s.low, s.high, cell, cutoff=rc, cutoff_3b=rc3, nu=nu, dt=dt, terms=t,
                           atm_sign=gpu.ATM_SIGN_PHYSICAL, atm_enum=gpu.ATM_ENUM_FULL,
                           virial_mode=gpu.VIRIAL_CORRECT, skin=skin)


def generate(n_points=40, snaps_per_point=50, ncell=5, equil=100, every=10, seed=2026, nu=0.073, device=0):
    """Training set from the exact kernel.  Returns dict of arrays:
    X (samples x 32 raw features), e (per-site ATM energies), f (exact ATM
    forces), point (state-point index)."""
    rng = np.random.default_rng(seed)
    X, E, F, P = [], [], [], []
    for k in range(n_points):
        t_star = float(rng.uniform(0.6, 1.2))
        rho = float(rng.uniform(0.75, 0.90))
        s = lattice.argon_fcc(ncell, rho=rho, t_star=t_star, seed=int(rng.integers(1 << 30)), jitter=0.02)
        cell = float(s.high[0]) / np.floor(float(s.high[0]) / 2.5)
        g = gpu.GpuSystem(s, physics_config(s, cell, nu=nu), device=device)
        g.update_container()
        g.forces()
        g.step(equil)
        for _ in range(snaps_per_point):
            g.update_container()
            x, e3, f3 = g.surrogate_sample()
            X.append(x)
            E.append(e3)
            F.append(f3)
            P.append(np.full(s.n, k, np.int32))
            g.forces()
            g.step(every)
        g.close()
    return dict(X=np.concatenate(X), e=np.concatenate(E), f=np.concatenate(F), point=np.concatenate(P))


def capture(n_points=40, snaps_per_point=50, ncell=5, equil=100, every=10, seed=2026, nu=0.073, device=0,
            nl_cap=80, jitter=0.02):
    """Force-matching dataset, resident on the device: n_points state points
    (T*, rho*) drawn from [0.6, 1.2] x [0.75, 0.9], each run with the exact
    LJ + ATM forces and captured every `every` steps after `equil` steps
    (snapshots of 4 ncell^3 sites; per site the ATM neighbour list, raw
    features, exact per-site energy and exact three-body force)."""
    rng = np.random.default_rng(seed)
    data = gpu.SurData(device=device, nl_cap=nl_cap)
    for _ in range(n_points):
        t_star = float(rng.uniform(0.6, 1.2))
        rho = float(rng.uniform(0.75, 0.90))
        s = lattice.argon_fcc(ncell, rho=rho, t_star=t_star, seed=int(rng.integers(1 << 30)), jitter=jitter)
        cell = float(s.high[0]) / np.floor(float(s.high[0]) / 2.5)
        g = gpu.GpuSystem(s, physics_config(s, cell, nu=nu), device=device)
        g.update_container()
        g.forces()
        g.step(equil)
        for _ in range(snaps_per_point):
            g.update_container()
            g.surrogate_capture(data)
            g.forces()
            g.step(every)
        g.close()
    return data


def scaling(data: "gpu.SurData") -> dict:
    """Feature standardisation, energy scaling and the mean squared exact
    three-body force per site of a dataset."""
    x, e3, f3, _ = data.get(-1)
    x = x.astype(np.float64)
    return dict(fmean=x.mean(0).astype(np.float32), fstd=(x.std(0) + 1e-12).astype(np.float32),
                e_shift=float(e3.mean()), e_scale=float(e3.std() + 1e-12),
                f2=float((f3.astype(np.float64) ** 2).sum(1).mean()))


def fit_forces(data: "gpu.SurData", epochs=60, snaps_per_batch=4, lr=3e-3, lr_end=5e-5, lam_e=0.1, lam_f=1.0,
               seed=7, params=None):
    """Force-matched training on the GPU (komd_sur_fit): energy and force
    residuals against the exact kernel's per-site energies and forces."""
    sc = scaling(data)
    p0 = init_params(seed) if params is None else params
    t0 = time.perf_counter()
    params, loss = data.fit(p0, sc["fmean"], sc["fstd"], sc["e_scale"], sc["e_shift"], sc["f2"], epochs,
                            snaps_per_batch=snaps_per_batch, lr=lr, lr_end=lr_end, lam_e=lam_e, lam_f=lam_f,
                            seed=seed)
    return dict(params=params, fmean=sc["fmean"], fstd=sc["fstd"], e_scale=sc["e_scale"], e_shift=sc["e_shift"],
                loss=loss, train_s=time.perf_counter() - t0, snapshots=data.snapshots, sites=data.sites)


def fit(data, epochs=40, batch=1024, lr=2e-3, seed=7):
    """Standardises features and targets and trains on the GPU."""
    X = data["X"].astype(np.float64)
    fmean = X.mean(0)
    fstd = X.std(0) + 1e-12
    e = data["e"]
    e_shift, e_scale = float(e.mean()), float(e.std() + 1e-12)
    Xs = ((X - fmean) / fstd).astype(np.float32)
    ys = ((e - e_shift) / e_scale).astype(np.float32)
    t0 = time.perf_counter()
    params, loss = gpu.mlp_train(Xs, ys, init_params(seed), epochs=epochs, batch=batch, lr=lr, seed=seed)
    return dict(params=params, fmean=fmean.astype(np.float32), fstd=fstd.astype(np.float32), e_scale=e_scale,
                e_shift=e_shift, loss=loss, train_s=time.perf_counter() - t0, samples=int(Xs.shape[0]))


def force_rmse(f, ref):
    """|f - ref| RMS over |ref| RMS."""
    return float(np.sqrt(((f - ref) ** 2).sum(1).mean() / (ref ** 2).sum(1).mean()))


def save(path, model):
    np.savez(path, **{k: np.asarray(v) for k, v in model.items()})


def load(path):
    z = np.load(path)
    return {k: (z[k].item() if z[k].ndim == 0 else z[k]) for k in z.files}
