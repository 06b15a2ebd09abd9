"""Multi-GPU layout of the traversal: one process per GPU, no exchange on the data path.

Worlds are read-only during a frame and every ray, tile and view is independent, so
N ranks need no collective while they trace.  Two layouts:

* weak scaling (what `bench.py --gpus N` measures): every rank traces its own batch of
  the same shape, built from a seed derived from its rank;
* strong scaling: one batch is split by world across ranks (`shard_batch`), each rank
  holding the worlds it owns and the views that look into them.

The only collectives are outside the timed data path: a barrier around the timed
region and the maximum of the per-rank times.  They run over NCCL on GPUs and over
gloo in the CPU tests.
"""
from __future__ import annotations

import os

SEED_STRIDE = 1000


def env_rank() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def rank_seed(base_seed: int, rank: int) -> int:
    """Seed of a rank's own batch under weak scaling (rank 0 keeps the base seed)."""
    return base_seed + SEED_STRIDE * rank


def shard_worlds(world_sizes, rank: int, world_size: int) -> list[int]:
    """Worlds owned by `rank`: largest first, each to the rank with the least total so
    far (ties to the lower rank), so ranks hold similar brick volumes."""
    if not 0 <= rank < world_size:
        raise ValueError(f"rank {rank} outside world size {world_size}")
    order = sorted(range(len(world_sizes)), key=lambda i: (-world_sizes[i], i))
    load = [0] * world_size
    owner = [0] * len(world_sizes)
    for i in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += world_sizes[i]
    return [i for i in range(len(world_sizes)) if owner[i] == rank]


def shard_batch(worlds, views, rank: int, world_size: int, size_of=None):
    """(local worlds, local views, global world index of each local world) for `rank`.

    Views keep their order; their `world` field is re-indexed to the local list.  The
    views of a world all go to the rank that owns it, so a rank's records are whole
    views and the union over ranks is the full batch."""
    from .capi import View

    size_of = size_of or (lambda w: int(getattr(w, "n_bricks", 1)))
    own = shard_worlds([size_of(w) for w in worlds], rank, world_size)
    local_index = {g: k for k, g in enumerate(own)}
    local_views = []
    for vw in views:
        if vw.world in local_index:
            c = View.from_buffer_copy(vw)
            c.world = local_index[vw.world]
            local_views.append(c)
    return [worlds[g] for g in own], local_views, own


def _reduce(pg, x: float, op_name: str, device) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=getattr(pg.ReduceOp, op_name))
    return float(t.item())


def max_over_ranks(pg, x: float, device="cuda") -> float:
    """Largest per-rank value (the job's time is its slowest rank's)."""
    return _reduce(pg, x, "MAX", device)


def sum_over_ranks(pg, x: float, device="cuda") -> float:
    return _reduce(pg, x, "SUM", device)


def barrier(pg) -> None:
    if pg is not None:
        pg.barrier()
