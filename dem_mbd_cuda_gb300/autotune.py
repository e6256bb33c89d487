"""Autotuner for the engine's runtime settings on a given scene.

Two settings change the speed of a step without changing its contact physics:

* the cell factor (cell edge = factor x the scene's largest radius): a smaller
  cell means fewer candidates per particle in the sweep but more cells to
  build and visit; the reference's 2.5 is the only value whose sorted cell
  keys match its own, so it stays the default;
* the particle-triangle crossover (contact items up to which the PT law runs
  one warp per item instead of one thread per item).

``autotune(scene)`` times graph-launched steps for each candidate (CUDA
events on the engine stream after warm-up steps) and returns the fastest
setting with the whole table.  Results are cached per scene signature and
precision for the process.
"""
from __future__ import annotations

import hashlib

import numpy as np

from .engine import CudaDemSolver

FACTORS = (2.0, 2.25, 2.5, 3.0, 3.5)
WARP_ITEMS = (512, 3072, 16384)
_cache: dict = {}


def _signature(scene, precision):
    h = hashlib.sha1()
    scenes = scene if isinstance(scene, (list, tuple)) else [scene]
    for s in scenes:
        h.update(np.ascontiguousarray(s.pos).tobytes()[:1 << 20])
        h.update(np.ascontiguousarray(s.owner_radius).tobytes()[:1 << 20])
        h.update(str((s.n, s.n_triangles, s.dt)).encode())
    h.update(precision.encode())
    return h.hexdigest()


def _time(scene, precision, factor, warp_items, steps, warmup):
    e = CudaDemSolver().initialize(scene, precision=precision, cell_factor=factor)
    if warp_items is not None:
        e.set_pt_warp_items(warp_items)
    e.run(max(1, warmup))
    return e.time_steps(steps) / steps


def autotune(scene, precision="mixed", factors=FACTORS, warp_items=WARP_ITEMS, steps=20, warmup=5):
    """Fastest (cell_factor, pt_warp_items) for `scene`; returns a dict with
    the choice, its ms per step, the default's ms per step and the table."""
    key = (_signature(scene, precision), tuple(factors), tuple(warp_items), steps)
    if key in _cache:
        return _cache[key]
    table = []
    for f in factors:
        table.append({"cell_factor": f, "pt_warp_items": None, "ms_per_step": _time(scene, precision, f, None, steps, warmup)})
    best = min(table, key=lambda r: r["ms_per_step"])
    has_bodies = any(s.n_bodies for s in (scene if isinstance(scene, (list, tuple)) else [scene]))
    if has_bodies:
        for w in warp_items:
            table.append({"cell_factor": best["cell_factor"], "pt_warp_items": w,
                          "ms_per_step": _time(scene, precision, best["cell_factor"], w, steps, warmup)})
        best = min(table, key=lambda r: r["ms_per_step"])
    default = next(r["ms_per_step"] for r in table if r["cell_factor"] == 2.5 and r["pt_warp_items"] is None)
    out = {"cell_factor": best["cell_factor"], "pt_warp_items": best["pt_warp_items"], "ms_per_step": best["ms_per_step"],
           "default_ms_per_step": default, "speedup_over_default": default / best["ms_per_step"], "table": table}
    _cache[key] = out
    return out
