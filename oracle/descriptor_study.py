"""Descriptor study for the learned three-body term (analysis, not product code).

TEST INFRASTRUCTURE ONLY: uses the oracle (oracle/komd_oracle.c through
pyoracle) as the source of liquid configurations and exact ATM forces.

Question: how close can a per-site energy built from O(k) descriptors (sums
over the neighbours of one site, no explicit triplets) come to the exact
Axilrod-Teller-Muto forces?  For each descriptor family the per-site energy is
taken LINEAR in the descriptors, E = sum_i sum_k w_k D_ik, so the forces
F = -sum_k w_k dS_k/dr (S_k = sum_i D_ik) are linear in w and the best
weights are a least-squares fit of the exact three-body forces of training
snapshots; the score is the relative force RMSE on held-out snapshots
(|F_fit - F_exact| RMS / |F_exact| RMS).  A linear fit bounds what the family
carries to first order; the engine's MLP on the first family is the
comparison (its three-body force RMSE is the benchmark's
surrogate.force_rmse_3body).

Families (neighbours inside rc = 2.0, fc = (cos(pi r / rc) + 1) / 2):
  radial   G_k = sum_j exp(-50 (r - mu_k)^2) fc,  mu_k = 0.85 + k 1.15 / 15 (16 terms)
  channel  g_c(r) = exp(-eta (r - mu_c)^2) fc with moments
           M0_c = sum g_c, M1_c = sum g_c u, M2_c = sum g_c u u, M3_c = sum g_c u u u
  engine   radial + per channel (4, the engine's) |M1|^2, M2:M2, M1.M2.M1, tr M2^3      32 features
  crossL3  radial + for every channel pair (a <= b) of 3 channels M1a.M1b, M2a:M2b, M3a:M3b   34
  cross6   radial + for every pair of 6 channels M0aM0b, M1a.M1b, M2a:M2b, M3a:M3b      100
  cross8   the same over 8 channels                                                     160

Snapshots: 500-atom argon (FCC 5^3 start), LJ 2.5 + ATM 2.0 (FULL, physical
sign, nu* 0.073) with the oracle's reference-semantics MD at dt* 0.005,
state points (T*, rho*) in [0.6, 1.2] x [0.75, 0.9]; 300 steps to melt, then
one snapshot every 20 steps.  Even state points train, odd ones are held out.

    python oracle/descriptor_study.py [--points 6] [--snaps 5] [--families engine,crossL3,cross6,cross8]

prints one JSON line per family and a summary.  Needs torch (CPU autograd
for the descriptor Jacobians).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))

RC = 2.0
NU = 0.073


def snapshots(points: int, snaps: int, seed: int = 11, equil: int = 300, every: int = 20):
    """[(r, box, f3, point index)] from the oracle's MD."""
    import pyoracle
    from komd_gb300 import lattice
    pyoracle.build()
    rng = np.random.default_rng(seed)
    out = []
    for p in range(points):
        t_star = float(rng.uniform(0.6, 1.2))
        rho = float(rng.uniform(0.75, 0.90))
        s = lattice.argon_fcc(5, rho=rho, t_star=t_star, seed=int(rng.integers(1 << 30)), jitter=0.02)
        L = float(s.high[0] - s.low[0])
        cell = L / math.floor(L / 2.5)
        sim = pyoracle.OracleSim(s, cell, 2.5, dt=0.005, nu=NU, cutoff_atm=RC, atm=True, atm_mode="full",
                                 atm_sign=pyoracle.ATM_SIGN_PHYSICAL, virial_mode=pyoracle.VIRIAL_CORRECT)
        sim.step(first=True)
        for k in range(equil + snaps * every):
            sim.step()
            if k >= equil and (k - equil) % every == every - 1:
                three = pyoracle.OracleSim(
                    lattice.System(r=sim.r.copy(), v=sim.v.copy(), m=s.m, eps=s.eps, sig=s.sig, mol_id=s.mol_id,
                                   low=s.low, high=s.high),
                    cell, 2.5, nu=NU, cutoff_atm=RC, lj=False, atm=True, atm_mode="full",
                    atm_sign=pyoracle.ATM_SIGN_PHYSICAL, virial_mode=pyoracle.VIRIAL_CORRECT)
                three.update_container()
                three.forces()
                out.append((three.r.copy() - s.low, np.full(3, L), three.f.copy(), p))
    return out


def _channels(n):
    mu = np.linspace(0.95, 1.95, n)
    width = (mu[1] - mu[0]) if n > 1 else 0.25
    return mu, 1.0 / (2.0 * width * width)


def pair_list(r_np, box):
    """Directed pairs (i, j) with |r_j - r_i| < rc (minimum image) and the
    periodic shift of each, fixed for the snapshot."""
    d = r_np[None, :, :] - r_np[:, None, :]
    shift = -box * np.round(d / box)
    d = d + shift
    r2 = (d * d).sum(-1)
    np.fill_diagonal(r2, np.inf)
    i, j = np.nonzero(r2 < RC * RC)
    return i, j, shift[i, j]


def descriptor_sums(family: str, r, pairs):
    """S_k = sum over sites of each feature, as a torch function of the
    positions r (requires_grad), and the feature count."""
    import torch
    n = r.shape[0]
    i_np, j_np, sh = pairs
    i = torch.as_tensor(i_np)
    j = torch.as_tensor(j_np)
    d = r[j] - r[i] + torch.as_tensor(sh)
    rr = torch.sqrt((d * d).sum(-1))
    fc = 0.5 * (torch.cos(math.pi * rr / RC) + 1.0)
    u = d / rr[:, None]

    def site_sum(x):   # per-pair rows -> per-site sums
        out = torch.zeros((n,) + tuple(x.shape[1:]), dtype=x.dtype)
        return out.index_add(0, i, x)

    feats = []
    mu_r = 0.85 + np.arange(16) * 1.15 / 15.0
    for m in mu_r:
        feats.append(site_sum(torch.exp(-50.0 * (rr - m) ** 2) * fc))
    if family == "engine":
        mu_c, eta = 1.05 + 0.25 * np.arange(4), 22.222222
    else:
        nc = {"crossL3": 3, "cross6": 6, "cross8": 8}[family]
        mu_c, eta = _channels(nc)
    uu = u[:, :, None] * u[:, None, :]
    uuu = uu[:, :, :, None] * u[:, None, None, :]
    M0, M1, M2, M3 = [], [], [], []
    for m in mu_c:
        g = torch.exp(-eta * (rr - m) ** 2) * fc
        M0.append(site_sum(g))
        M1.append(site_sum(g[:, None] * u))
        M2.append(site_sum(g[:, None, None] * uu))
        M3.append(site_sum(g[:, None, None, None] * uuu))
    if family == "engine":
        for c in range(len(mu_c)):
            v, M = M1[c], M2[c]
            feats.append((v * v).sum(-1))
            feats.append((M * M).sum((-1, -2)))
            feats.append(torch.einsum("ix,ixy,iy->i", v, M, v))
            feats.append(torch.einsum("ixy,iyz,izx->i", M, M, M))
    else:
        C = len(mu_c)
        for a in range(C):
            for b in range(a, C):
                if family != "crossL3":
                    feats.append(M0[a] * M0[b])
                feats.append((M1[a] * M1[b]).sum(-1))
                feats.append((M2[a] * M2[b]).sum((-1, -2)))
                feats.append((M3[a] * M3[b]).sum((-1, -2, -3)))
    D = torch.stack(feats, 1)                                  # (n, K)
    return D.sum(0), D.shape[1]


def jacobian(family: str, r_np, box):
    """J (3n x K): dS_k / dr for every feature k."""
    import torch
    r = torch.tensor(r_np, dtype=torch.float64, requires_grad=True)
    S, K = descriptor_sums(family, r, pair_list(r_np, box))
    cols = []
    for k in range(K):
        (g,) = torch.autograd.grad(S[k], r, retain_graph=k + 1 < K)
        cols.append(g.reshape(-1).numpy())
    return np.stack(cols, 1)


def study(family: str, snaps, ridge: float = 1e-8):
    jac = [jacobian(family, r, box) for r, box, _, _ in snaps]
    train = [k for k, s in enumerate(snaps) if s[3] % 2 == 0]
    test = [k for k, s in enumerate(snaps) if s[3] % 2 == 1]
    A, b = [], []
    for k in train:
        A.append(-jac[k])
        b.append(snaps[k][2].reshape(-1))
    A, b = np.concatenate(A), np.concatenate(b)
    scale = np.sqrt((A * A).mean(0)) + 1e-300
    As = A / scale
    w = np.linalg.solve(As.T @ As + ridge * len(b) * np.eye(As.shape[1]), As.T @ b) / scale

    def rel(sets):
        num = den = 0.0
        for k in sets:
            f3 = snaps[k][2]
            fp = (-jac[k] @ w).reshape(-1, 3)
            num += ((fp - f3) ** 2).sum()
            den += (f3 ** 2).sum()
        return math.sqrt(num / den)

    return {"family": family, "features": int(A.shape[1]), "train_rel_rmse": rel(train), "held_out_rel_rmse": rel(test),
            "train_snapshots": len(train), "held_out_snapshots": len(test)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--points", type=int, default=6)
    ap.add_argument("--snaps", type=int, default=5)
    ap.add_argument("--families", default="engine,crossL3,cross6,cross8")
    a = ap.parse_args()
    t0 = time.time()
    snaps = snapshots(a.points, a.snaps)
    print(json.dumps({"snapshots": len(snaps), "atoms": int(snaps[0][0].shape[0]), "seconds": time.time() - t0}),
          flush=True)
    for fam in a.families.split(","):
        t1 = time.time()
        res = study(fam, snaps)
        res["seconds"] = time.time() - t1
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
