"""Learned three-body term on the GPU against the FP64 oracle (oracle/kor_sur_*).

The reference has no surrogate; these checks pin the CUDA descriptors, the
training kernels' gradients, the tensor-core inference and the analytic
forces to the FP64 restatement, and show what the trained network gains
over leaving the three-body term out.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _small_system(seed=51, ncell=4, jitter=0.06):
    from komd_gb300 import lattice
    return lattice.argon_fcc(ncell, rho=0.8442, t_star=0.9, seed=seed, jitter=jitter)   # 256 sites, L = 6.72


def _gpu(s, cell=2.2):
    from komd_gb300 import gpu, surrogate
    g = gpu.GpuSystem(s, surrogate.physics_config(s, cell, rc=2.0))   # LJ cutoff <= cell edge
    g.update_container()
    return g


def _min_image_neighbours(r, box, i, rc):
    d = r - r[i]
    d -= box * np.round(d / box)
    q = (d * d).sum(1)
    m = (q < rc * rc) & (np.arange(len(r)) != i)
    return d[m]


def test_descriptors_and_labels_match_oracle(oracle_lib):
    s = _small_system()
    g = _gpu(s)
    x, e3, f3 = g.surrogate_sample()
    r, _, _ = g.download()
    ref = np.array([oracle_lib.sur_features(_min_image_neighbours(r, s.box, i, 2.0)) for i in range(s.n)])
    scale = np.abs(ref).max(0) + 1e-12
    dev = (np.abs(x - ref) / (2e-4 * np.abs(ref) + 2e-4 * scale)).max(0)
    assert dev.max() < 1.0, f"feature deviations in units of the tolerance: {np.round(dev, 2).tolist()}"
    # exact per-site ATM energies sum to the oracle's ATM energy; forces match
    sim = oracle_lib.OracleSim(s, 2.2, 2.0, nu=0.073, lj=False, atm=True, atm_mode="full",
                               atm_sign=oracle_lib.ATM_SIGN_PHYSICAL, virial_mode=oracle_lib.VIRIAL_CORRECT)
    sim.update_container()
    sim.forces()
    assert e3.sum() == pytest.approx(sim.atm_out.energy, rel=1e-5)
    err = np.sqrt(((f3 - sim.f) ** 2).sum(1).mean() / (sim.f ** 2).sum(1).mean())
    assert err < 1e-5
    g.close()


def test_training_gradient_matches_oracle(oracle_lib):
    from komd_gb300 import gpu, surrogate
    rng = np.random.default_rng(3)
    params = surrogate.init_params(11)
    params[64 * 32:64 * 32 + 64] = rng.normal(0, 0.1, 64)          # non-zero biases
    X = rng.normal(0, 1, (96, 32)).astype(np.float32)
    y = rng.normal(0, 1, 96).astype(np.float32)
    g, loss = gpu.mlp_loss_grad(X, y, params)
    p64 = params.astype(np.float64)
    ref = np.zeros_like(p64)
    ref_loss = 0.0
    for k in range(len(y)):
        e, _ = oracle_lib.sur_mlp(p64, X[k].astype(np.float64))
        ref += 2.0 * (e - y[k]) / len(y) * oracle_lib.sur_mlp_param_grad(p64, X[k].astype(np.float64))
        ref_loss += (e - y[k]) ** 2 / len(y)
    assert loss == pytest.approx(ref_loss, rel=1e-4)
    assert np.abs(g - ref).max() < 1e-4 * np.abs(ref).max() + 1e-7


# (form, loss tolerance, gradient tolerance in units of the largest
# component): the FP32 SIMT form, and the tensor-core form that komd_sur_fit
# runs by default, whose BF16 operands (8-bit significands) round every
# activation, weight and gradient record to about 0.4 %
FIT_FORMS = [("fp32", 2e-3, 3e-3), ("bf16", 3e-2, 3e-2)]


@pytest.mark.parametrize("form,loss_tol,grad_tol", FIT_FORMS)
def test_force_matching_gradient_matches_oracle(oracle_lib, form, loss_tol, grad_tol):
    """komd_sur_fit's gradient (energy + force residuals through the
    descriptor Jacobian and the network's tangent pass) against central
    differences of the same loss evaluated by the FP64 oracle; the BF16
    tensor-core gradient also against the FP32 one, block by block."""
    from komd_gb300 import gpu, surrogate
    s = _small_system(seed=53)
    g = _gpu(s)
    data = gpu.SurData(nl_cap=80)
    g.surrogate_capture(data)
    r, _, _ = g.download()
    g.close()
    x, e3, f3, site = data.get(0)
    e3s = np.zeros(s.n)
    f3s = np.zeros((s.n, 3))
    e3s[site] = e3
    f3s[site] = f3
    fmean = x.mean(0).astype(np.float32)
    fstd = (x.std(0) + 1e-6).astype(np.float32)
    e_scale, e_shift = float(e3.std()), float(e3.mean())
    f2 = float((f3.astype(np.float64) ** 2).sum(1).mean())
    rng = np.random.default_rng(4)
    params = surrogate.init_params(8)
    params[64 * 32:64 * 32 + 64] = rng.normal(0, 0.1, 64)
    params[64 * 32 + 64 + 64 * 64:64 * 32 + 64 + 64 * 64 + 64] = rng.normal(0, 0.1, 64)
    lam_e, lam_f = 0.3, 1.0
    precision = gpu.FIT_BF16 if form == "bf16" else gpu.FIT_FP32
    grad, loss = data.fit_grad(params, fmean, fstd, e_scale, e_shift, f2, lam_e=lam_e, lam_f=lam_f,
                               precision=precision)
    blocks = [(0, 2048), (2048, 2112), (2112, 6208), (6208, 6272), (6272, 6336), (6336, 6337)]   # W1 b1 W2 b2 w3 b3
    if form == "bf16":
        g32, _ = data.fit_grad(params, fmean, fstd, e_scale, e_shift, f2, lam_e=lam_e, lam_f=lam_f,
                               precision=gpu.FIT_FP32)
        top = np.abs(g32).max()
        for a, b in blocks:   # each block against its own scale (at least 5 % of the largest component)
            ref = max(np.abs(g32[a:b]).max(), 0.05 * top)
            assert np.abs(grad[a:b] - g32[a:b]).max() < grad_tol * ref, (a, b)
    fm64, fs64 = fmean.astype(np.float64), fstd.astype(np.float64)
    y = (e3s - e_shift) / e_scale

    def oracle_loss(p64):
        _, e, f = oracle_lib.sur_energy_forces(r, s.box, p64, fm64, fs64, e_scale, e_shift)
        return (lam_e * np.mean(((e - e_shift) / e_scale - y) ** 2), lam_f * np.mean(((f - f3s) ** 2).sum(1)) / f2)

    p64 = params.astype(np.float64)
    le, lf = oracle_loss(p64)
    assert loss[0] == pytest.approx(le, rel=loss_tol)
    assert loss[1] == pytest.approx(lf, rel=loss_tol)
    idx = np.concatenate([rng.choice(np.arange(a, b), min(4, b - a), replace=False) for a, b in blocks])
    h = 1e-4
    num = []
    for q in idx:
        pp, pm = p64.copy(), p64.copy()
        pp[q] += h
        pm[q] -= h
        num.append((sum(oracle_loss(pp)) - sum(oracle_loss(pm))) / (2 * h))
    num = np.array(num)
    scale = max(np.abs(num).max(), np.abs(grad).max())
    assert np.abs(grad[idx] - num).max() < grad_tol * scale, (grad[idx], num)
    data.close()


def _model_from_sample(x, params, e3):
    fmean = x.mean(0)
    fstd = x.std(0) + 1e-6
    return dict(params=params, fmean=fmean.astype(np.float32), fstd=fstd.astype(np.float32),
                e_scale=float(e3.std()), e_shift=float(e3.mean()))


def test_inference_forces_match_oracle(oracle_lib):
    """Tensor-core inference (BF16 weights, FP32 accumulation) and the
    chain-rule forces against the FP64 energy and its analytic gradient."""
    from komd_gb300 import surrogate
    s = _small_system(seed=52)
    g = _gpu(s)
    x, e3, _ = g.surrogate_sample()
    model = _model_from_sample(x, surrogate.init_params(5), e3)
    g.surrogate_load(model, probe_every=0)
    f, e = g.surrogate_forces()
    r, _, _ = g.download()
    et, e_ref, f_ref = oracle_lib.sur_energy_forces(r, s.box, model["params"].astype(np.float64),
                                                    model["fmean"].astype(np.float64),
                                                    model["fstd"].astype(np.float64), model["e_scale"],
                                                    model["e_shift"])
    assert surrogate.force_rmse(f, f_ref) < 3e-2            # BF16 weights and activations
    assert np.abs(e - e_ref).max() < 3e-2 * np.abs(e_ref - model["e_shift"]).max() + 1e-6
    assert np.abs(f.sum(0)).max() < 1e-3 * np.abs(f).max()  # Newton's third law through the chain rule
    g.close()


@pytest.fixture(scope="module")
def trained():
    from komd_gb300 import surrogate
    data = surrogate.capture(n_points=8, snaps_per_point=10, ncell=5, equil=40, every=10, seed=99)
    model = surrogate.fit_forces(data, epochs=40, snaps_per_batch=4, lr=3e-3, seed=3)
    data.close()
    return None, model


def test_trained_surrogate_gains_over_no_threebody(trained):
    """On a held-out configuration (another seed and state point, run with
    the exact forces) the trained network's three-body forces sit far closer
    to the exact ones than the method without the learned term (three-body
    forces left out: relative error 1), and the per-site energies explain
    most of the variance."""
    from komd_gb300 import gpu, lattice, surrogate
    _, model = trained
    assert model["loss"][-1].sum() < 0.5 * model["loss"][0].sum()
    s = lattice.argon_fcc(5, rho=0.82, t_star=0.9, seed=777, jitter=0.02)
    cell = float(s.high[0]) / np.floor(float(s.high[0]) / 2.5)
    g = gpu.GpuSystem(s, surrogate.physics_config(s, cell))
    g.update_container()
    g.forces()
    g.step(150)
    g.update_container()
    _, e3, f3 = g.surrogate_sample()
    g.surrogate_load(model, probe_every=0)
    f, e = g.surrogate_forces()
    err = surrogate.force_rmse(f, f3)
    assert err < 0.35, f"surrogate three-body force RMSE {err:.3f}"
    r2 = 1.0 - ((e - e3) ** 2).sum() / ((e3 - e3.mean()) ** 2).sum()
    assert r2 > 0.8
    g.close()


def test_probe_and_fallback(trained):
    from komd_gb300 import gpu, surrogate
    _, model = trained
    s = _small_system(seed=31)
    for thr, expect_fallback in ((1e-9, 1), (10.0, 0)):
        cfg = surrogate.physics_config(s, 2.2, rc=2.0, terms=gpu.TERM_LJ | gpu.TERM_ATM | gpu.TERM_ATM_SURROGATE)
        g = gpu.GpuSystem(s, cfg)
        g.surrogate_load(model, probe_every=5, probe_threshold=thr)
        g.update_container()
        g.forces()
        g.step(12)
        st = g.surrogate_status()
        assert st["probes"] >= 1
        assert st["fallback"] == expect_fallback
        assert st["last_rmse"] > 0
        r, v, f = g.download()
        assert np.isfinite(r).all() and np.isfinite(f).all()
        g.close()
