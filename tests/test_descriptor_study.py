"""The descriptor study (oracle/descriptor_study.py) on a small sample: it
builds liquid snapshots with the oracle, the descriptor Jacobians by CPU
autograd, and linear force fits whose errors are finite and below the
zero-force baseline.  The full study's table is in the design notes."""
import numpy as np
import pytest


def test_descriptor_study_small_sample(oracle_lib):
    pytest.importorskip("torch")
    import descriptor_study as ds
    snaps = ds.snapshots(points=2, snaps=2, equil=100, every=10)
    assert len(snaps) == 4 and snaps[0][0].shape == (500, 3)
    assert all(np.abs(s[2]).max() > 0 for s in snaps)      # exact three-body forces
    for fam, nfeat in (("engine", 32), ("crossL3", 34)):
        res = ds.study(fam, snaps)
        assert res["features"] == nfeat
        assert 0.0 < res["train_rel_rmse"] < 1.0 and np.isfinite(res["held_out_rel_rmse"])
