"""KoMD's input-file and checkpoint formats (Python side).

Mirrors the reference's whitespace key/value parser (IO/FileInput.cpp:11-122)
and its `.ps` checkpoint format (IO/CheckpointIO.cpp:13-76):

    id <TAB> rx ry rz <TAB> vx vy vz <TAB> mass eps sig      (one site per line)

consecutive lines with the same id form one molecule.  Two reference quirks
are handled on purpose:

* the reference re-executes the last key or line when a file ends in a
  newline (its ``while(!eof())`` loops); files written here never end in one,
  and the readers here accept either form;
* checkpoints written by the reference use the stream's default 6 significant
  digits; files written here use 17 so that doubles round-trip exactly.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .lattice import System

# defaults, util/defaults.h:11-64 of the reference
DEFAULTS = dict(
    temperature=300.0, delta_t=0.001, timesteps=1, cutoff=2.5, cell_size=3.0, density=0.1,
    stiffness=30.0, limit=20.0, energy_3b=1.0, pair_steps=4, triple_steps=8,
    domain_low=(0.0, 0.0, 0.0), domain_high=(10.0, 10.0, 10.0), write_freq=10,
    enable_3b_approx=0, enable_3b=0, enable_3b_direct=1, enable_sensor_lj=0,
    enable_sensor_fene=0, enable_sensor_rdf=0, enable_sensor_disp=0, enable_sensor_pres=0,
    enable_sensor_visc=0, sensor_lj_bins=100, sensor_fene_bins=100, sensor_rdf_max=5.0,
    sensor_rdf_dr=0.1, store_checkpoint=0,
)

_FLOAT_KEYS = {"temperature", "delta_t", "cutoff", "cell_size", "density", "stiffness", "limit",
               "energy_3b", "sensor_rdf_max", "sensor_rdf_dr"}
_INT_KEYS = {"timesteps", "pair_steps", "triple_steps", "write_freq", "enable_3b_approx", "enable_3b",
             "enable_3b_direct", "enable_sensor_lj", "enable_sensor_fene", "enable_sensor_rdf",
             "enable_sensor_disp", "enable_sensor_pres", "enable_sensor_visc", "sensor_lj_bins",
             "sensor_fene_bins", "store_checkpoint"}
_VEC_KEYS = {"domain_low", "domain_high"}


@dataclass
class InputFile:
    values: Dict[str, object] = field(default_factory=lambda: dict(DEFAULTS))
    checkpoints: List[Tuple[str, Tuple[float, float, float]]] = field(default_factory=list)
    components: Dict[int, List[Tuple[float, float, float, Tuple[float, float, float]]]] = field(default_factory=dict)
    extra: Dict[str, List[str]] = field(default_factory=dict)

    def __getitem__(self, k):
        return self.values[k]

    @property
    def max_sigma(self) -> float:
        return max(s[1] for sites in self.components.values() for s in sites)


def parse_input(text: str) -> InputFile:
    """Token stream parser with the reference's key set; unknown keys are
    skipped token by token, '#' starts a comment running to the end of line."""
    inp = InputFile()
    lines = text.splitlines()
    toks: List[str] = []
    for ln in lines:
        parts = ln.split()
        for i, p in enumerate(parts):
            if p.startswith("#"):
                break
            toks.append(p)
    i = 0

    def take(k=1):
        nonlocal i
        out = toks[i:i + k]
        if len(out) < k:
            raise ValueError("truncated input")
        i += k
        return out

    while i < len(toks):
        key = take()[0]
        if key in _FLOAT_KEYS:
            inp.values[key] = float(take()[0])
        elif key in _INT_KEYS:
            inp.values[key] = int(float(take()[0]))
        elif key in _VEC_KEYS:
            inp.values[key] = tuple(float(x) for x in take(3))
        elif key == "checkpoint_file":
            p, *o = take(4)
            inp.checkpoints.append((p, tuple(float(x) for x in o)))
        elif key == "COMP":
            cid, eps, sig, mass, x, y, z = take(7)
            if int(cid) < 0:
                raise ValueError("negative component id not allowed")
            inp.components.setdefault(int(cid), []).append(
                (float(eps), float(sig), float(mass), (float(x), float(y), float(z))))
        else:
            # keys outside the hot path (plugins, IBI, ADR, ...) keep their tokens
            inp.extra.setdefault(key, [])
    if not inp.components:
        raise ValueError("no components defined")
    if not inp.checkpoints:
        raise ValueError("No phasespace data specified")
    if inp["cell_size"] < inp["cutoff"]:
        raise ValueError("cell size must be larger or equal to cutoff radius")
    return inp


def read_input(path: str) -> InputFile:
    with open(path) as fh:
        return parse_input(fh.read())


def format_input(values: dict, checkpoint: Optional[str], comps: List[tuple],
                 regions: Sequence[tuple] = ()) -> str:
    """Input file text without a trailing newline.  comps: (cid, eps in J,
    sigma, mass[, site position]) per COMP line; regions: (begin xyz, end xyz,
    cid) per ps_gen_region line; checkpoint None: no checkpoint_file line."""
    out = []
    for k, v in values.items():
        if isinstance(v, (tuple, list)):
            out.append(f"{k} " + " ".join(repr(float(x)) for x in v))
        elif isinstance(v, float):
            out.append(f"{k} {v!r}")
        else:
            out.append(f"{k} {v}")
    if checkpoint is not None:
        out.append(f"checkpoint_file {checkpoint} 0 0 0")
    for begin, end, cid in regions:
        out.append("ps_gen_region " + " ".join(repr(float(x)) for x in (*begin, *end)) + f" {int(cid)}")
    for c in comps:
        cid, eps_j, sig, mass = c[:4]
        r = c[4] if len(c) > 4 else (0.0, 0.0, 0.0)
        out.append(f"COMP {cid} {eps_j!r} {sig!r} {mass!r} " + " ".join(repr(float(x)) for x in r))
    return "\n".join(out)


def write_checkpoint(path: str, sysm: System) -> None:
    """17-significant-digit checkpoint, no trailing newline."""
    rows = []
    for s in range(sysm.n):
        r, v = sysm.r[s], sysm.v[s]
        rows.append("%d\t%.17g %.17g %.17g\t%.17g %.17g %.17g\t%.17g %.17g %.17g" % (
            int(sysm.mol_id[s]), r[0], r[1], r[2], v[0], v[1], v[2], sysm.m[s], sysm.eps[s], sysm.sig[s]))
    with open(path, "w") as fh:
        fh.write("\n".join(rows))


def read_checkpoint(path: str, low=(0, 0, 0), high=(10, 10, 10), offset=(0.0, 0.0, 0.0)) -> System:
    """Reads a `.ps` file; a trailing newline does not add a phantom site."""
    data = []
    with open(path) as fh:
        for ln in fh:
            p = ln.split()
            if not p:
                continue
            if len(p) != 10:
                raise ValueError(f"malformed checkpoint line: {ln!r}")
            data.append(p)
    ids = np.array([int(p[0]) for p in data], dtype=np.uint64)
    arr = np.array([[float(x) for x in p[1:]] for p in data], dtype=np.float64).reshape(-1, 9)
    off = np.asarray(offset, dtype=np.float64)
    return System(r=arr[:, 0:3] + off, v=arr[:, 3:6].copy(), m=arr[:, 6].copy(), eps=arr[:, 7].copy(),
                  sig=arr[:, 8].copy(), mol_id=ids, low=np.asarray(low, float), high=np.asarray(high, float))


def rdf_nbins(max_r: float, dr: float) -> int:
    """(uint64)(max_r / dr), RDFSensor.cpp:18."""
    return int(math.trunc(max_r / dr))


def rdf_normalise(bins: np.ndarray, samples: int, dr: float, volume: float, n: int):
    """(r, g(r)) from a raw histogram of ordered molecule pairs, as
    RDFSensor::write (RDFSensor.cpp:45-60): bin centres r = (k + 1/2) dr,
    g = (bins/samples) V / (shell volume * n (n - 1))."""
    b = np.asarray(bins, np.float64) / max(samples, 1)
    r = (np.arange(b.size) + 0.5) * dr
    v_bin = 4.0 / 3.0 * math.pi * ((r + 0.5 * dr) ** 3 - (r - 0.5 * dr) ** 3)
    return r, b * volume / (v_bin * n * (n - 1.0))


_VTU_ARRAYS = (("mass", "Float32", 1), ("velocity", "Float32", 3), ("force", "Float32", 3), ("id", "Int32", 1),
               ("cid", "Int32", 1))


def write_vtu(path: str, sysm: System, f=None, cid=None) -> None:
    """VTK UnstructuredGrid (.vtu, ASCII) of a snapshot with the arrays of
    KoMD's VTKWriter (IO/VTKWriter.cpp:44-123): points, and per site mass,
    velocity, force (Float32) and molecule id and component id (Int32).  The
    same layout as the `komd` executable's VTK_Output_<step>.vtu."""
    n = sysm.n
    f = np.zeros((n, 3)) if f is None else np.asarray(f)
    cid = np.zeros(n, np.int64) if cid is None else np.asarray(cid)
    cols = dict(mass=sysm.m, velocity=sysm.v, force=f, id=sysm.mol_id.astype(np.int64), cid=cid)

    def arr(name, typ, comps, data):
        a = np.asarray(data).reshape(-1)
        body = " ".join(repr(float(np.float32(x))) if typ == "Float32" else str(int(x)) for x in a)
        return (f'      <DataArray type="{typ}" Name="{name}" NumberOfComponents="{comps}" format="ascii">'
                f"{body + ' ' if body else ''}</DataArray>\n")

    out = ['<?xml version="1.0" encoding="UTF-8"?>\n',
           '<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian">\n',
           "  <UnstructuredGrid>\n", f'    <Piece NumberOfPoints="{n}" NumberOfCells="0">\n', "    <PointData>\n"]
    out += [arr(nm, t, c, cols[nm]) for nm, t, c in _VTU_ARRAYS]
    out += ["    </PointData>\n    <CellData/>\n    <Points>\n", arr("points", "Float32", 3, sysm.r),
            "    </Points>\n    <Cells>\n", arr("types", "Float32", 0, []),
            "    </Cells>\n    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n"]
    with open(path, "w") as fh:
        fh.write("".join(out))


def read_vtu(path: str) -> Dict[str, np.ndarray]:
    """The point arrays of an ASCII .vtu written by write_vtu or `komd`
    ({"points": (n, 3), "mass": (n,), "velocity": (n, 3), ...})."""
    import xml.etree.ElementTree as ET
    root = ET.parse(path).getroot()
    piece = root.find("UnstructuredGrid/Piece")
    n = int(piece.get("NumberOfPoints"))
    out = {}
    for da in piece.iter("DataArray"):
        comps = int(da.get("NumberOfComponents"))
        if comps == 0:
            continue
        dt = np.float32 if da.get("type") == "Float32" else np.int64
        vals = np.array((da.text or "").split(), dtype=np.float64).astype(dt)
        out[da.get("Name")] = vals.reshape(n, comps) if comps > 1 else vals.reshape(n)
    return out
