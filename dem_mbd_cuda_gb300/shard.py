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
