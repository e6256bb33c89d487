"""Autotuner for the engine's runtime settings on a given scene.

Three settings change the speed of a step without changing its contact
physics:

* the cell factor (cell edge = factor x the scene's largest radius): a smaller
  cell means fewer candidates per particle in the sweep but more cells to
  build and visit; the reference's 2.5 is the only value whose sorted cell
  keys match its own, so it stays the default;
* the blocks per SM of the sweep and of the record gathers: they run
  grid-stride so that the kernels of the step's other branches
  (particle-triangle law, rotational advance, walls) find free warp slots
  beside them; the best share depends on how much work those branches carry;
* the particle-triangle crossover (contact items up to which the PT law runs
  one warp per item instead of one thread per item);
* the neighbour lists' skin (0: lists off, the cells swept every step): a
  wider skin means longer lists but fewer rebuilds.

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
SWEEP_BLOCKS = (2, 3, 4, 6, 8, 16, 24)
GATHER_BLOCKS = (2, 3, 4, 6, 8)
WARP_ITEMS = (512, 3072, 16384)
SKINS = (0, 250, 500, 900)  # per mille of the room the cell edge leaves beyond the largest pair
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


def _time(scene, precision, factor, sweep_blocks, gather_blocks, warp_items, skin, steps, warmup):
    e = CudaDemSolver().initialize(scene, precision=precision, cell_factor=factor)
    if skin is not None:
        e.set_neighbor_lists(skin > 0, skin if skin > 0 else None)
    if sweep_blocks is not None:
        e.set_sweep_blocks(sweep_blocks)
    if gather_blocks is not None:
        e.set_gather_blocks(gather_blocks)
    if warp_items is not None:
        e.set_pt_warp_items(warp_items)
    e.run(max(1, warmup))
    return min(e.time_steps(steps) / steps for _ in range(2))


def autotune(scene, precision="mixed", factors=FACTORS, sweep_blocks=SWEEP_BLOCKS, gather_blocks=GATHER_BLOCKS,
             warp_items=WARP_ITEMS, skins=SKINS, steps=100, warmup=5):
    """Fastest (cell_factor, nl_skin, sweep_blocks, gather_blocks,
    pt_warp_items) for `scene`, searched one setting at a time in that order;
    returns a dict with the choice, its ms per step, the default's ms per step
    and the table.  None in the choice means the engine's default.  The
    windows are long enough for the neighbour lists' movers to build up (on
    the 2M drum 20-step windows favoured 6 sweep blocks per SM, 200-step runs
    24)."""
    key = (_signature(scene, precision), tuple(factors), tuple(sweep_blocks), tuple(gather_blocks), tuple(warp_items),
           tuple(skins), steps)
    if key in _cache:
        return _cache[key]
    table = []

    def row(f, b, g, w, k=None):
        r = {"cell_factor": f, "nl_skin": k, "sweep_blocks": b, "gather_blocks": g, "pt_warp_items": w,
             "ms_per_step": _time(scene, precision, f, b, g, w, k, steps, warmup)}
        table.append(r)
        return r

    def pick(rows):
        return min(rows, key=lambda r: r["ms_per_step"])

    best = pick([row(f, None, None, None) for f in factors])
    default = next(r["ms_per_step"] for r in table if r["cell_factor"] == 2.5)
    best = pick([best] + [row(best["cell_factor"], None, None, None, k) for k in skins])
    sk = best["nl_skin"]
    best = pick([best] + [row(best["cell_factor"], b, None, None, sk) for b in sweep_blocks])
    best = pick([best] + [row(best["cell_factor"], best["sweep_blocks"], g, None, sk) for g in gather_blocks])
    has_bodies = any(s.n_bodies for s in (scene if isinstance(scene, (list, tuple)) else [scene]))
    if has_bodies:
        best = pick([best] + [row(best["cell_factor"], best["sweep_blocks"], best["gather_blocks"], w, sk)
                              for w in warp_items])
    out = {"cell_factor": best["cell_factor"], "nl_skin": best["nl_skin"], "sweep_blocks": best["sweep_blocks"],
           "gather_blocks": best["gather_blocks"], "pt_warp_items": best["pt_warp_items"],
           "ms_per_step": best["ms_per_step"], "default_ms_per_step": default,
           "speedup_over_default": default / best["ms_per_step"], "table": table}
    _cache[key] = out
    return out
