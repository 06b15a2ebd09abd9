"""Multi-rank layout of the traversal on CPU: world sharding, per-rank seeds, and the
collectives around the timed region over gloo with two ranks (no GPU)."""
import json
import socket
from dataclasses import dataclass

import pytest

from voxelrt_gb300 import shard


@dataclass
class FakeWorld:
    n_bricks: int


def test_shard_worlds_partitions_and_balances():
    sizes = [900, 10, 500, 500, 30, 400, 7, 1000, 60, 60]
    for n in (1, 2, 3, 4):
        parts = [shard.shard_worlds(sizes, r, n) for r in range(n)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        loads = [sum(sizes[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(sizes)
    with pytest.raises(ValueError):
        shard.shard_worlds(sizes, 2, 2)


def test_rank_seed_distinct_and_rank0_is_base():
    assert shard.rank_seed(2, 0) == 2
    assert len({shard.rank_seed(2, r) for r in range(8)}) == 8


def _views(n_worlds, per_world):
    import voxelrt_gb300 as v
    views = []
    for w in range(n_worlds):
        for k in range(per_world[w]):
            cam = v.look_at((10.0 + k, 20.0, 5.0), (40.0, 10.0, 40.0 + w), 70.0, 16 + k, 8 + w)
            views.append(v.make_view(cam, world=w))
    return views


def test_shard_batch_reindexes_views():
    per_world = [3, 0, 2, 1, 4]
    worlds = [FakeWorld(b) for b in (50, 40, 30, 20, 10)]
    views = _views(len(worlds), per_world)
    seen = []
    for r in range(2):
        lw, lv, own = shard.shard_batch(worlds, views, r, 2)
        assert [worlds[g] for g in own] == lw
        for vw in lv:
            g = own[vw.world]
            seen.append((g, vw.cam.width, vw.cam.height))
            assert 0 <= vw.world < len(lw)
    want = sorted((vw.world, vw.cam.width, vw.cam.height) for vw in views)
    assert sorted(seen) == want


def _rank_main(rank, world_size, port, out_dir):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world_size)
    try:
        worlds = [FakeWorld(b) for b in (70, 5, 33, 33, 12, 90)]
        views = _views(len(worlds), [2, 1, 1, 3, 0, 2])
        lw, lv, own = shard.shard_batch(worlds, views, rank, world_size)
        shard.barrier(dist)
        t_max = shard.max_over_ranks(dist, 1.5 + rank, "cpu")
        rays = sum(vw.cam.width * vw.cam.height for vw in lv)
        total = shard.sum_over_ranks(dist, float(rays), "cpu")
        gathered = [None] * world_size
        dist.all_gather_object(gathered, own)
        with open(f"{out_dir}/rank{rank}.json", "w") as f:
            json.dump({"t_max": t_max, "total": total, "own": gathered,
                       "all_rays": sum(vw.cam.width * vw.cam.height for vw in views)}, f)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    res = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(2)]
    for r in res:
        assert r["t_max"] == 2.5                      # the slowest rank's time
        assert r["total"] == r["all_rays"]            # the job's rays: each view on exactly one rank
        assert sorted(r["own"][0] + r["own"][1]) == list(range(6))
        assert not set(r["own"][0]) & set(r["own"][1])
