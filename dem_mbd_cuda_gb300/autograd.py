"""torch.autograd.Function over the engine's reverse mode.

``simulate(scene, steps, pp, pw, vel0)`` runs the reference's step sequence
(FP64 form) from ``scene`` with the particle-particle and particle-wall
materials ``pp`` / ``pw`` (tensors [kN, mu, epsN, epsS, muT, muR]) and initial
velocities ``vel0`` ([n, 3]), and returns the final positions and velocities.
Gradients flow back to the materials and the initial velocities through
dem_adjoint_forward / dem_adjoint_backward, so material calibration is an
ordinary torch optimisation loop.  Tensors live on the host; the engine keeps
its own device state.

``simulate_batch(scenes, steps, pp, pw, vel0)`` does the same for a batch of
independent scenes in one engine (one launch per kernel per step): ``pp`` and
``pw`` are [scenes, 6], ``vel0`` and the results are the scenes' owners one
after the other, and each scene's materials get their own gradients.
"""
from __future__ import annotations

import dataclasses

import numpy as np
import torch

from .engine import CudaDemSolver

FIELDS = ("kN", "mu", "epsN", "epsS", "muT", "muR")


def _with_materials(scene, pp, pw, vel0):
    def mech(m, v):
        return dataclasses.replace(m, **{f: float(x) for f, x in zip(FIELDS, v)})
    return dataclasses.replace(scene, pp=mech(scene.pp, pp), pw=mech(scene.pw, pw), pt=dataclasses.replace(scene.pt),
                               vel=np.asarray(vel0, dtype=np.float64).reshape(-1, 3).copy())


def _batch_with_materials(scenes, pp, pw, vel0):
    out, off = [], 0
    for k, s in enumerate(scenes):
        out.append(_with_materials(s, pp[k], pw[k], vel0[off:off + s.n]))
        off += s.n
    return out


class DemRun(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pp, pw, vel0, scene, steps, checkpoint_every, reverse_fp32=False):
        args = (pp.detach().cpu().numpy(), pw.detach().cpu().numpy(), vel0.detach().cpu().numpy().reshape(-1, 3))
        sc = _batch_with_materials(scene, *args) if isinstance(scene, (list, tuple)) else _with_materials(scene, *args)
        e = CudaDemSolver().initialize(sc, precision="fp64").set_adjoint_fp32(reverse_fp32)
        e.adjoint_forward(steps, checkpoint_every)
        st = e.downloadParticleState()
        ctx.engine = e
        ctx.dtype = pp.dtype
        return (torch.as_tensor(st["pos"], dtype=vel0.dtype), torch.as_tensor(st["vel"], dtype=vel0.dtype))

    @staticmethod
    def backward(ctx, gpos, gvel):
        g = ctx.engine.adjoint_backward(None if gpos is None else gpos.detach().cpu().numpy(),
                                        None if gvel is None else gvel.detach().cpu().numpy())
        per = g["dl_dparams"]
        rows = per if isinstance(per, list) else [per]
        pp = torch.tensor([[r["pp"][f] for f in FIELDS] for r in rows], dtype=ctx.dtype)
        pw = torch.tensor([[r["pw"][f] for f in FIELDS] for r in rows], dtype=ctx.dtype)
        if not isinstance(per, list):
            pp, pw = pp[0], pw[0]
        dv = torch.as_tensor(g["dl_dvel0"], dtype=gpos.dtype if gpos is not None else gvel.dtype)
        return pp, pw, dv, None, None, None, None


def materials(m):
    """A scene's Mech as the [kN, mu, epsN, epsS, muT, muR] tensor."""
    return torch.tensor([getattr(m, f) for f in FIELDS], dtype=torch.float64)


def simulate(scene, steps, pp, pw, vel0, checkpoint_every=100, reverse_fp32=False):
    """Final (positions, velocities) of `steps` steps, differentiable with
    respect to pp, pw and vel0.  reverse_fp32 runs the reverse law of the
    particle and wall contacts in FP32 (CudaDemSolver.set_adjoint_fp32)."""
    return DemRun.apply(pp, pw, vel0, scene, int(steps), int(checkpoint_every), bool(reverse_fp32))


def simulate_batch(scenes, steps, pp, pw, vel0, checkpoint_every=100, reverse_fp32=False):
    """Final (positions, velocities) of `steps` steps of a batch of scenes,
    differentiable with respect to the per-scene materials pp, pw
    ([scenes, 6]) and vel0 (the scenes' owners one after the other)."""
    return DemRun.apply(pp, pw, vel0, list(scenes), int(steps), int(checkpoint_every), bool(reverse_fp32))
