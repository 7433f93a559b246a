"""Input-file and checkpoint formats (CPU)."""
import os

import numpy as np
import pytest

from komd_gb300 import komd_io, lattice


def test_checkpoint_roundtrip_exact(tmp_path):
    s = lattice.triatomic_sc(3, seed=9)
    p = tmp_path / "x.ps"
    komd_io.write_checkpoint(str(p), s)
    text = p.read_text()
    assert not text.endswith("\n")
    back = komd_io.read_checkpoint(str(p), s.low, s.high)
    assert np.array_equal(back.r, s.r) and np.array_equal(back.v, s.v)
    assert np.array_equal(back.mol_id, s.mol_id)
    assert np.array_equal(back.mol_off, s.mol_off)


def test_trailing_newline_adds_no_phantom_site(tmp_path):
    s = lattice.argon_fcc(2, seed=1)
    p = tmp_path / "x.ps"
    komd_io.write_checkpoint(str(p), s)
    with open(p, "a") as fh:
        fh.write("\n")
    assert komd_io.read_checkpoint(str(p)).n == s.n


def test_parse_reference_style_input():
    text = """# comment line
temperature 150
delta_t 0.0005
cutoff 8.525
cell_size 10
checkpoint_file ../examples/argon/ckpt_3b_eq.ps    0 0 0
energy_3b 7.32e-27
domain_low 0 0 0
domain_high 20 20 20
enable_3b 1
enable_3b_direct 0
IBI_alpha 0.2
COMP   0       1.661196877e-21      3.41    39.948        0           0           0
"""
    inp = komd_io.parse_input(text)
    assert inp["cutoff"] == 8.525 and inp["cell_size"] == 10.0
    assert inp["enable_3b"] == 1 and inp["enable_3b_direct"] == 0
    assert inp["domain_high"] == (20.0, 20.0, 20.0)
    assert inp.checkpoints[0][0].endswith("ckpt_3b_eq.ps")
    assert inp.max_sigma == 3.41


def test_parse_rejects_like_reference():
    with pytest.raises(ValueError, match="no components"):
        komd_io.parse_input("cutoff 2.5\ncheckpoint_file a.ps 0 0 0")
    with pytest.raises(ValueError, match="cell size"):
        komd_io.parse_input("cutoff 3\ncell_size 2\ncheckpoint_file a.ps 0 0 0\nCOMP 0 1 1 1 0 0 0")


def test_unit_mapping():
    assert lattice.energy_3b_to_nu(lattice.nu_star_to_energy_3b(0.073)) == pytest.approx(0.073, rel=1e-15)
    assert komd_io.rdf_nbins(2.5, 0.0125) in (199, 200)


def test_autotune_cell_edge():
    from komd_gb300 import autotune
    assert autotune.cell_for(67.184, 2.8) == pytest.approx(67.184 / 23)
    assert autotune.cell_for(10.0, 2.5) == pytest.approx(2.5)
    with pytest.raises(ValueError):
        autotune.cell_for(7.0, 2.5)


def test_vtu_round_trip(tmp_path):
    """write_vtu / read_vtu: KoMD's VTKWriter arrays as Float32 / Int32."""
    from komd_gb300 import komd_io, lattice
    s = lattice.argon_fcc(2, seed=3)
    f = np.random.default_rng(0).normal(size=(s.n, 3))
    p = tmp_path / "VTK_Output_0007.vtu"
    komd_io.write_vtu(str(p), s, f=f)
    d = komd_io.read_vtu(str(p))
    assert np.array_equal(d["points"], s.r.astype(np.float32))
    assert np.array_equal(d["velocity"], s.v.astype(np.float32))
    assert np.array_equal(d["force"], f.astype(np.float32))
    assert np.array_equal(d["mass"], s.m.astype(np.float32))
    assert np.array_equal(d["id"], s.mol_id.astype(np.int64))
    assert not d["cid"].any()
