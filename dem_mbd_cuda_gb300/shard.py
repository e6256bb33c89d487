"""Batches of independent scenes over several GPUs: one process per GPU, each
running its share of the scenes as one batched engine.

Scenes do not interact, so the only exchange is on the host: per-scene
results (losses, gradients, final states) gathered to every rank, and the
slowest rank's time.  ``partition`` balances the shares by particle count
(greedy: the largest scene next to the least-loaded rank, ties to the lower
index), so every rank derives the same assignment without communication.
"""
from __future__ import annotations


def partition(counts, world):
    """Scene indices per rank ([world] sorted lists) balancing the sum of
    `counts` (particles per scene)."""
    if world < 1:
        raise ValueError("world must be at least 1")
    order = sorted(range(len(counts)), key=lambda i: (-counts[i], i))
    loads = [0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (loads[k], k))
        parts[r].append(i)
        loads[r] += counts[i]
    return [sorted(p) for p in parts]


def gather_per_scene(local_values, parts, group=None):
    """Every rank's per-scene values (in the order of its share) gathered
    into one list in scene order, on every rank (torch.distributed object
    gather; gloo or NCCL)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    if len(local_values) != len(parts[rank]):
        raise ValueError("one value per scene of this rank's share")
    got = [None] * world
    dist.all_gather_object(got, list(local_values), group=group)
    out = [None] * sum(len(p) for p in parts)
    for r, p in enumerate(parts):
        for k, i in enumerate(p):
            out[i] = got[r][k]
    return out


def max_over_ranks(x, group=None):
    """The largest of one float over the ranks (the slowest rank's time)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t[0])


def split_by_scene(array, counts):
    """Rows of a batch array ([sum(counts), ...], scenes one after the other)
    as one block per scene."""
    import numpy as np
    edges = np.cumsum([0] + list(counts))
    return [array[edges[k]:edges[k + 1]] for k in range(len(counts))]


def gather_batch_gradients(local, parts, counts, group=None):
    """The reverse-mode result of this rank's batch engine
    (CudaDemSolver.adjoint_backward over the scenes parts[rank], in that
    order) gathered into the whole batch's result on every rank: dl_dpos0,
    dl_dvel0 and dl_domega0 as [sum(counts), 3] arrays in scene order and
    dl_dparams as one entry per scene.  `counts` are the particles of every
    scene of the batch."""
    import numpy as np
    import torch.distributed as dist
    rank = dist.get_rank(group)
    mine = [counts[i] for i in parts[rank]]
    per = local["dl_dparams"]
    per = per if isinstance(per, list) else [per]
    if len(per) != len(mine):
        raise ValueError("one parameter gradient per scene of this rank's share")
    blocks = {k: split_by_scene(np.asarray(local[k]), mine) for k in ("dl_dpos0", "dl_dvel0", "dl_domega0")}
    rows = [{"dl_dparams": per[j], **{k: blocks[k][j] for k in blocks}} for j in range(len(mine))]
    allrows = gather_per_scene(rows, parts, group=group)
    out = {k: np.concatenate([r[k] for r in allrows]).reshape(-1, 3) for k in blocks}
    out["dl_dparams"] = [r["dl_dparams"] for r in allrows]
    return out
