"""Measured choice of the engine's shape parameters.

The physics does not depend on these parameters; only the speed does:

* single system: the Verlet skin (list length against rebuild frequency) and
  with it the cell edge (the smallest edge >= cutoff + skin that divides the
  box, so that the 27-cell stencil covers the list range);
* batched replicas: the number of parallel graph branches (for a packed
  batch, the groups of replicas) and the steps captured per graph.

Each candidate is timed on the caller's actual state (positions and
velocities), after a warm-up that includes the graph capture, by the
device-synchronised wall time of komd_gpu_step / komd_batch_step.
"""
from __future__ import annotations

import time
from typing import Callable, Dict, List, Sequence

import numpy as np

from . import gpu


def cell_for(box_len: float, reach: float) -> float:
    """Smallest cell edge >= reach that divides box_len into whole cells."""
    k = int(np.floor(box_len / reach))
    if k < 3:
        raise ValueError("box too small for three cells of the requested reach")
    return box_len / k


def tune_skin(system, make_cfg: Callable[[float, float], "gpu.KomdConfig"], skins: Sequence[float],
              rc_max: float, steps: int = 100, warmup: int = 20, device: int = 0) -> Dict:
    """Times `steps` steps for each skin (cell = cell_for(min box edge, rc_max + skin))
    and returns {"best": {...}, "table": [...]} sorted by ms per step."""
    L = float(np.min(np.asarray(system.high) - np.asarray(system.low)))
    table: List[Dict] = []
    for skin in skins:
        try:
            cell = cell_for(L, rc_max + skin)
        except ValueError:
            continue
        g = gpu.GpuSystem(system, make_cfg(skin, cell), device=device)
        try:
            g.update_container()
            g.forces()
            g.step(warmup)
            t0 = time.perf_counter()
            g.step(steps)
            ms = (time.perf_counter() - t0) * 1e3 / steps
        finally:
            g.close()
        table.append({"skin": float(skin), "cell": float(cell), "ms_per_step": ms})
    table.sort(key=lambda r: r["ms_per_step"])
    return {"best": table[0] if table else None, "table": table}


def tune_batch(systems, streams: Sequence[int] = (16, 32, 64), graph_steps: Sequence[int] = (1, 5, 10),
               steps: int = 10) -> Dict:
    """Times each (n_streams, steps_per_graph) on the given replicas; the
    replicas advance by the timed steps (they are independent MD runs)."""
    table: List[Dict] = []
    for ns in streams:
        for spg in graph_steps:
            b = gpu.Batch(systems, n_streams=ns, steps_per_graph=spg)
            try:
                b.step(1)
                n = max(1, steps // spg)
                t0 = time.perf_counter()
                b.step(n)
                ms = (time.perf_counter() - t0) * 1e3 / (n * spg)
            finally:
                b.close()
            table.append({"streams": int(ns), "steps_per_graph": int(spg), "ms_per_step": ms})
    table.sort(key=lambda r: r["ms_per_step"])
    return {"best": table[0], "table": table}
