"""Batched replicas (komd_batch_*): one CUDA graph advancing several engines
of uneven sizes must give every replica exactly the trajectory it gets when
stepped alone through the single-system path -- in the packed form (one
launch per stage of the step for all replicas) and in the branch form (each
replica's own kernels on parallel graph branches)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPECS = [(11, 2000, 0.75, 1.0), (12, 3100, 0.85, 0.7), (13, 2500, 0.90, 1.4), (14, 2222, 0.80, 0.6)]


def _replica(seed, n, rho, t_star, skin=0.3):
    from komd_gb300 import gpu, lattice, surrogate
    s = lattice.trimmed_fcc(n, rho, t_star, seed)
    cell = float(s.high[0]) / np.floor(float(s.high[0]) / 2.8)
    cfg = surrogate.physics_config(s, cell, skin=skin)
    g = gpu.GpuSystem(s, cfg)
    g.update_container()
    g.forces()
    return g


@pytest.mark.parametrize("groups", [1, 3])
def test_batch_matches_single_system_path(groups):
    """Packed form, all replicas in one group, and in three groups on parallel branches."""
    from komd_gb300 import gpu
    a = [_replica(*sp) for sp in SPECS]
    b = [_replica(*sp) for sp in SPECS]
    batch = gpu.Batch(a, n_streams=groups, steps_per_graph=5)
    assert batch.packed                             # the Verlet path's replicas: one launch per stage
    batch.step(6)                                   # 30 steps
    for g in b:
        g.step(30)
    for ga, gb in zip(a, b):
        ra, va, fa = ga.download()
        rb, vb, fb = gb.download()
        assert np.array_equal(ra, rb)
        assert np.array_equal(va, vb)
        assert np.array_equal(fa, fb)
    batch.close()
    for g in a + b:
        g.close()


def test_packed_mixture_replicas_match_single_path():
    """Replicas of a two-species LJ mixture (per-pair LJ parameters) take the
    packed form too: bitwise the single-system path after 20 steps."""
    from komd_gb300 import gpu, lattice, surrogate

    def make(seed, n, rho, t_star):
        s = lattice.trimmed_fcc(n, rho, t_star, seed)
        rng = np.random.default_rng(seed)
        mix = rng.random(s.n) < 0.4
        s.sig = np.where(mix, 0.9, 1.0)
        s.eps = np.where(mix, 0.7, 1.0)
        cfg = surrogate.physics_config(s, float(s.high[0]) / np.floor(float(s.high[0]) / 2.8), skin=0.3)
        g = gpu.GpuSystem(s, cfg)
        g.update_container()
        g.forces()
        return g

    a = [make(*sp) for sp in SPECS[:3]]
    b = [make(*sp) for sp in SPECS[:3]]
    batch = gpu.Batch(a, n_streams=2, steps_per_graph=4)
    assert batch.packed
    batch.step(5)
    batch.close()
    for ga, gb in zip(a, b):
        gb.step(20)
        ra, va, fa = ga.download()
        rb, vb, fb = gb.download()
        assert np.array_equal(ra, rb) and np.array_equal(va, vb) and np.array_equal(fa, fb)
        ga.close()
        gb.close()


def test_batch_measure_matches_replica_measures():
    """komd_batch_measure (every replica's measure enqueued on the batch's
    branches, one synchronisation) gives each replica what komd_gpu_measure
    gives it alone: energies, virial, pressure, temperature and the RDF.
    A measure with the RDF rebuilds the Verlet lists at the current positions
    (its cells may be stale), which moves the FP32 cell-local coordinates of
    the next measure's force pass by rounding: the first batched measure
    agrees with a measure alone to FP32 precision, a second one (lists of the
    same positions on both sides) to the last bits of the FP64 sums."""
    from komd_gb300 import gpu
    a = [_replica_rdf(*sp) for sp in SPECS]
    batch = gpu.Batch(a, n_streams=2, steps_per_graph=5)
    batch.step(2)
    mask = gpu.MEASURE_ENERGY | gpu.MEASURE_PRESSURE | gpu.MEASURE_TEMPERATURE | gpu.MEASURE_RDF
    first = batch.measure(mask)
    together = batch.measure(mask)
    batch.close()
    for g, t0, t in zip(a, first, together):
        alone = g.measure(mask)
        assert np.array_equal(t["rdf"], alone["rdf"]) and np.array_equal(t0["rdf"], alone["rdf"])
        assert t["rdf"].sum() > 0
        for k in ("u_lj", "u_atm", "temperature", "mv2", "pairs_in_cutoff", "triplets"):
            assert t[k] == pytest.approx(alone[k], rel=1e-12, abs=0), k
            assert t0[k] == pytest.approx(alone[k], rel=1e-6, abs=0), k
        np.testing.assert_allclose(t["pressure"], alone["pressure"], rtol=1e-12, atol=0)
        g.close()


def _replica_rdf(seed, n, rho, t_star):
    from komd_gb300 import gpu, lattice, surrogate
    s = lattice.trimmed_fcc(n, rho, t_star, seed)
    cfg = surrogate.physics_config(s, float(s.high[0]) / np.floor(float(s.high[0]) / 2.8), skin=0.3)
    cfg.rdf_max, cfg.rdf_dr = 2.5, 2.5 / 200
    g = gpu.GpuSystem(s, cfg)
    g.update_container()
    g.forces()
    return g


def test_branch_form_matches_single_system_path():
    """Replicas on the per-step-cell path (no skin) take the branch form."""
    from komd_gb300 import gpu
    a = [_replica(*sp, skin=0.0) for sp in SPECS[:3]]
    b = [_replica(*sp, skin=0.0) for sp in SPECS[:3]]
    batch = gpu.Batch(a, n_streams=2, steps_per_graph=4)
    assert not batch.packed
    batch.step(3)
    for g in b:
        g.step(12)
    for ga, gb in zip(a, b):
        ra, va, fa = ga.download()
        rb, vb, fb = gb.download()
        assert np.array_equal(ra, rb) and np.array_equal(va, vb) and np.array_equal(fa, fb)
    batch.close()
    for g in a + b:
        g.close()


def test_batch_rejects_bad_input():
    from komd_gb300 import gpu
    g = _replica(*SPECS[0])
    with pytest.raises(gpu.KomdError):
        gpu.Batch([g, g])                           # the same replica twice
    g.close()


def test_autotuner_picks_a_measured_shape():
    from komd_gb300 import autotune, gpu, lattice, surrogate
    reps = [_replica(*sp) for sp in SPECS[:3]]
    t = autotune.tune_batch(reps, streams=(2, 3), graph_steps=(1, 2), steps=4)
    assert len(t["table"]) == 4
    assert t["best"]["ms_per_step"] == min(r["ms_per_step"] for r in t["table"])
    for g in reps:
        g.close()
    s = lattice.argon_fcc(8, rho=0.8442, t_star=0.722, seed=5)          # 2048 atoms, L = 13.4

    def make_cfg(skin, cell):
        return surrogate.physics_config(s, cell, skin=skin)
    t = autotune.tune_skin(s, make_cfg, (0.2, 0.4), 2.5, steps=20, warmup=5)
    assert [r["skin"] for r in sorted(t["table"], key=lambda r: r["skin"])] == [0.2, 0.4]
    assert all(r["cell"] >= 2.5 + r["skin"] for r in t["table"])


@pytest.mark.parametrize("pinned", [True, False])
def test_step_host_matches_device_path(pinned):
    """komd_gpu_step_host on the fused path reads r, v from the caller's buffers
    and writes r, v, f back from inside the step's kernels (plain pageable
    memory where the GPU walks the host page tables; with pinned buffers the
    positions go back on the copy engine beside the force pass); the
    trajectory is bitwise the one of komd_gpu_step on device-resident state,
    for one step per call and for several."""
    import torch
    a = _replica(*SPECS[1])
    b = _replica(*SPECS[1])
    r0, v0, f0 = a.download()

    def buf(x):
        t = torch.from_numpy(np.ascontiguousarray(x))
        return (t.pin_memory() if pinned else t.clone()).numpy()

    r, v, f = buf(r0), buf(v0), buf(np.zeros_like(f0))
    for n in (1, 1, 2, 5, 1):
        a.step_host(n, r, v, f)
        b.step(n)
        rb, vb, fb = b.download()
        assert np.array_equal(r, rb)
        assert np.array_equal(v, vb)
        assert np.array_equal(f, fb)
    a.close()
    b.close()


def test_step_host_graph_follows_buffers_and_stream():
    """A one-step komd_gpu_step_host call replays a graph captured for the
    caller's buffers.  Calls that alternate between two pinned buffer sets, and
    calls after set_stream (which retires the step graph), stay bitwise on the
    trajectory of komd_gpu_step."""
    import torch
    a = _replica(*SPECS[1])
    b = _replica(*SPECS[1])
    r0, v0, f0 = a.download()

    def pin(x):
        return torch.from_numpy(np.ascontiguousarray(x)).pin_memory().numpy()

    sets = [(pin(r0), pin(v0), pin(np.zeros_like(f0))), (pin(r0), pin(v0), pin(np.zeros_like(f0)))]
    side = torch.cuda.Stream()
    cur = 0
    for k in range(8):
        if k == 4:
            a.set_stream(side.cuda_stream)
            b.set_stream(side.cuda_stream)
        r, v, f = sets[cur]
        a.step_host(1, r, v, f)
        b.step(1)
        rb, vb, fb = b.download()
        assert np.array_equal(r, rb), k
        assert np.array_equal(v, vb), k
        assert np.array_equal(f, fb), k
        if k % 2:   # the next call reads the other buffer set
            nr, nv, _ = sets[1 - cur]
            nr[:] = r
            nv[:] = v
            cur = 1 - cur
    a.close()
    b.close()


def test_batch_512_replicas_full_size():
    """The batched-replicas workload at its full size: 512 LJ + ATM boxes,
    N ~ U[2000, 20000] (FCC filled, trimmed by seed), rho* ~ U[0.70, 0.90],
    T* ~ U[0.6, 1.5], one graph over 32 branches.  After 10 steps, sampled
    replicas equal, bit for bit, the same replicas stepped alone, and every
    replica's RDF (200 bins to 2.5) and virial pressure are finite."""
    from komd_gb300 import gpu, lattice, surrogate
    rng = np.random.default_rng(2027)
    specs = [(int(rng.integers(1 << 30)), int(rng.integers(2000, 20001)), float(rng.uniform(0.70, 0.90)),
              float(rng.uniform(0.6, 1.5))) for _ in range(512)]

    def make(seed, n, rho, t_star):
        s = lattice.trimmed_fcc(n, rho, t_star, seed)
        L = float(s.high[0])
        cfg = surrogate.physics_config(s, L / np.floor(L / 2.8), skin=0.3)
        cfg.rdf_max, cfg.rdf_dr = 2.5, 2.5 / 200
        g = gpu.GpuSystem(s, cfg)
        g.update_container()
        g.forces()
        return g

    reps = [make(*sp) for sp in specs]
    assert 512 * 2000 <= sum(g.n for g in reps) <= 512 * 20000
    batch = gpu.Batch(reps, n_streams=32, steps_per_graph=5)
    assert batch.packed
    batch.step(2)
    batch.close()
    for k in (0, 137, 511):
        alone = make(*specs[k])
        alone.step(10)
        ra, va, fa = reps[k].download()
        rb, vb, fb = alone.download()
        assert np.array_equal(ra, rb) and np.array_equal(va, vb) and np.array_equal(fa, fb)
        alone.close()
    for g in reps:
        o = g.measure(gpu.MEASURE_PRESSURE | gpu.MEASURE_RDF)
        assert o["rdf"].size == 200 and np.isfinite(o["rdf"]).all() and o["rdf"].sum() > 0
        assert np.isfinite(o["pressure"]).all()
        g.close()
