"""Scene sharding of a batch over ranks (dem_mbd_cuda_gb300/shard.py): the
partition covers every scene once and balances particles; the per-scene
gather, the max over ranks and the gather of a batched reverse-mode result
(per-scene gradients shaped as CudaDemSolver.adjoint_backward returns them
for a rank's share) run as two gloo processes on the CPU."""
import os
import socket

import pytest

from dem_mbd_cuda_gb300.shard import partition


def test_partition_covers_and_balances():
    import random
    rng = random.Random(3)
    counts = [rng.randint(2000, 40000) for _ in range(256)]
    for world in (1, 2, 3, 4, 8):
        parts = partition(counts, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(256))
        loads = [sum(counts[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(counts)
    assert partition(counts, 4) == partition(counts, 4)
    assert partition([5, 5, 5], 5)[3:] == [[], []]
    with pytest.raises(ValueError):
        partition(counts, 0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, counts, out_dir):
    import torch.distributed as dist
    from dem_mbd_cuda_gb300.shard import gather_per_scene, max_over_ranks, partition
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    parts = partition(counts, world)
    mine = [10.0 * i + 0.5 for i in parts[rank]]     # a per-scene result of this rank's share
    allv = gather_per_scene(mine, parts)
    slowest = max_over_ranks(1.0 + rank)
    with open(os.path.join(out_dir, f"r{rank}.txt"), "w") as f:
        f.write(repr((allv, slowest)))
    dist.barrier()
    dist.destroy_process_group()


def test_gather_and_max_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    counts = [30000, 2000, 17000, 40000, 5000, 12000, 9000]
    port = _free_port()
    mp.spawn(_worker, args=(2, port, counts, str(tmp_path)), nprocs=2, join=True)
    for rank in range(2):
        allv, slowest = eval(open(tmp_path / f"r{rank}.txt").read())
        assert allv == [10.0 * i + 0.5 for i in range(len(counts))]
        assert slowest == 2.0


def _grad_worker(rank, world, port, counts, out_dir):
    import numpy as np
    import torch.distributed as dist
    from dem_mbd_cuda_gb300.shard import gather_batch_gradients, partition
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    parts = partition(counts, world)
    # this rank's batch engine result: its scenes one after the other, every
    # row tagged with (scene, row) so the assembly can be checked
    rows = []
    for i in parts[rank]:
        rows.append(np.stack([np.full(counts[i], float(i)), np.arange(counts[i], dtype=float),
                              np.full(counts[i], float(rank))], axis=1))
    dv = np.concatenate(rows)
    keys = ("kN", "mu", "epsN", "epsS", "muT", "muR")
    params = [{c: {k: 100.0 * i + j for j, k in enumerate(keys)} for c in ("pp", "pw", "pt")} for i in parts[rank]]
    local = {"dl_dpos0": 2 * dv, "dl_dvel0": dv, "dl_domega0": -dv, "dl_dparams": params}
    out = gather_batch_gradients(local, parts, counts)
    np.save(os.path.join(out_dir, f"g{rank}.npy"), out["dl_dvel0"])
    with open(os.path.join(out_dir, f"p{rank}.txt"), "w") as f:
        f.write(repr([p["pp"]["mu"] for p in out["dl_dparams"]]))
    assert np.array_equal(out["dl_dpos0"], 2 * out["dl_dvel0"])
    dist.barrier()
    dist.destroy_process_group()


def test_batched_gradients_gather_in_scene_order(tmp_path):
    import numpy as np
    import torch.multiprocessing as mp
    from dem_mbd_cuda_gb300 import generate as G
    counts = [s.n for s in G.batch(nscenes=6, nmin=200, nmax=900)]
    port = _free_port()
    mp.spawn(_grad_worker, args=(2, port, counts, str(tmp_path)), nprocs=2, join=True)
    for rank in range(2):
        g = np.load(tmp_path / f"g{rank}.npy")
        assert g.shape == (sum(counts), 3)
        scene = np.repeat(np.arange(len(counts)), counts)
        row = np.concatenate([np.arange(c) for c in counts])
        assert np.array_equal(g[:, 0], scene) and np.array_equal(g[:, 1], row)
        assert eval(open(tmp_path / f"p{rank}.txt").read()) == [100.0 * i + 1 for i in range(len(counts))]
