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


class StubEngine:
    """CPU stand-in for bench.GpuEngine: the rank's own seeded workload (bench's weak-scaling
    layout), its primary rays as the rays of a step, and fixed per-rank times (the slower
    rank 1 sets the job's time)."""

    def __init__(self, args, rank, world_size, local):
        import bench
        self.args, self.rank = args, rank
        self.wl = bench.build_workload("uneven_batch", rank, args, world_size)
        self.rays_per_step = self.wl.primary_rays
        self.h2d_bytes = 128 * len(self.wl.views)
        self.d2h_bytes = 16 * self.rays_per_step

    def time_batched(self, sync):
        sync()
        return 2.0 + self.rank, {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}

    def time_per_view(self):
        return 5.0 + self.rank, 1

    def time_e2e(self, sync):
        sync()
        return 0.010 * (1 + self.rank)

    def d2h_link_gbs(self):
        return 100.0

    def config(self):
        return {"workload": self.wl.name, "rays_per_step": self.rays_per_step}

    def extras(self):
        return {"roofline": None, "cpu_baseline": None, "rank_rays": self.rays_per_step}

    def close(self):
        pass


def _bench_rank(rank, world_size, port, out_dir):
    import contextlib
    import io
    import os
    os.environ.update(WORLD_SIZE=str(world_size), RANK=str(rank), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    args = bench.parse(["--gpus", str(world_size), "--worlds", "3", "--max-views", "2"])
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_ours(args, engine_cls=StubEngine, backend="gloo", device="cpu")
    rays = StubEngine(args, rank, world_size, rank).rays_per_step
    with open(f"{out_dir}/bench{rank}.json", "w") as f:
        json.dump({"stdout": buf.getvalue(), "rays": rays}, f)


def test_bench_two_gloo_ranks(tmp_path):
    """bench.run_ours over two gloo ranks: one JSON line from rank 0 with n_gpus 2, the job's
    rays the sum of both ranks' rays and its time the slower rank's."""
    mp = pytest.importorskip("torch.multiprocessing")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.start_processes(_bench_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    res = [json.loads((tmp_path / f"bench{r}.json").read_text()) for r in range(2)]
    assert res[1]["stdout"] == ""
    lines = [ln for ln in res[0]["stdout"].splitlines() if ln.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    job = res[0]["rays"] + res[1]["rays"]
    assert res[0]["rays"] != res[1]["rays"]  # each rank traced its own seeded batch
    assert line["n_gpus"] == 2 and line["scaling"] == "weak"
    assert line["job_rays_per_step"] == job
    assert line["ms_per_step"] == 3.0
    assert abs(line["value"] - job / 3.0e-3 / 1e9) < 1e-12
    assert abs(line["per_view"]["value"] - job / 6.0e-3 / 1e9) < 1e-12
    assert abs(line["e2e"]["value"] - job / 0.020 / 1e9) < 1e-12
    assert line["e2e"]["d2h_bytes_per_step"] == 16 * job


def test_bench_rank_count_checks(monkeypatch):
    import bench
    cmd = bench.relaunch_cmd(4, ["--gpus", "4", "--steps", "5"], 29512)
    assert cmd[1:3] == ["-m", "torch.distributed.run"] and "--nproc-per-node=4" in cmd
    assert cmd[cmd.index("--master-addr") + 1] == "127.0.0.1" and cmd[-4:] == ["--gpus", "4", "--steps", "5"]
    monkeypatch.setenv("WORLD_SIZE", "2")
    assert bench.main(["--gpus", "4"]) == 2  # a torchrun job whose size disagrees is refused
