"""Autotuner for the batched persistent traversal.

Sweeps the launch structure of vrt_batch - ray tile shape (8x8, 8x8 Morton, 16x4,
32x1), warps per block, refill (compaction) threshold, DDA iterations between refill
checks and tiles per queue fetch - on a given batch, timing CUDA-graph launches with
CUDA events, and caches the winner per GPU name and workload.

Cache lookup order: $VRT_AUTOTUNE_CACHE (or ~/.cache/voxelrt_gb300/autotune.json),
then the table shipped in voxelrt_gb300/tuned.json (results measured on GB300).
"""
from __future__ import annotations

import itertools
import json
import os
from pathlib import Path

from .capi import BatchConfig

_FIELDS = ("tile_w", "tile_h", "morton", "warps_per_block", "blocks_per_sm", "refill_threshold", "chunk_tiles",
           "inner_iters")
SHIPPED = Path(__file__).resolve().parent / "tuned.json"


def user_cache() -> Path:
    p = os.environ.get("VRT_AUTOTUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "voxelrt_gb300" / "autotune.json"


def gpu_name() -> str:
    try:
        import torch
        return torch.cuda.get_device_name()
    except Exception:
        return "unknown"


def to_config(d: dict) -> BatchConfig:
    return BatchConfig(**{k: int(d.get(k, 0)) for k in _FIELDS})


def describe(cfg: BatchConfig | None) -> dict:
    if cfg is None:
        return {"default": True}
    return {k: int(getattr(cfg, k)) for k in _FIELDS}


def _load(p: Path) -> dict:
    try:
        return json.loads(p.read_text())
    except Exception:
        return {}


def lookup(workload: str, gpu: str | None = None):
    gpu = gpu or gpu_name()
    for src, table in (("cache", _load(user_cache())), ("shipped", _load(SHIPPED))):
        entry = table.get(gpu, {}).get(workload)
        if entry:
            return to_config(entry["config"]), f"{src}:{gpu}"
    return None, "library defaults"


def store(workload: str, cfg: dict, result: dict, path: Path | None = None, gpu: str | None = None) -> Path:
    path = path or user_cache()
    gpu = gpu or gpu_name()
    table = _load(path)
    table.setdefault(gpu, {})[workload] = {"config": cfg, **result}
    path.parent.mkdir(parents=True, exist_ok=True)
    path.write_text(json.dumps(table, indent=1, sort_keys=True))
    return path


def time_config(worlds, views, cfg: BatchConfig, hits, stream, launches: int = 4) -> float:
    """Milliseconds per graph launch of a batch built with cfg."""
    import torch

    from . import Batch
    b = Batch(worlds, views, cfg)
    b.launch(hits, stream, graph=True)
    b.launch(hits, stream, graph=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(launches):
        b.launch(hits, stream, graph=True)
    e1.record(stream)
    e1.synchronize()
    b.close()
    return e0.elapsed_time(e1) / launches


def tune(worlds, views, hits, stream, log=print, passes: int = 2) -> tuple[dict, float, list]:
    """Staged sweep (coordinate descent over the stages, `passes` times, so the tile shape
    and warps are chosen again under the refill and round length found after them);
    returns (best config dict, ms, trials)."""
    trials = []

    def run(d):
        ms = time_config(worlds, views, to_config(d), hits, stream)
        trials.append({**d, "ms": ms})
        log(f"  {d} -> {ms:.3f} ms")
        return ms

    best = {"tile_w": 8, "tile_h": 8, "morton": 0, "warps_per_block": 4, "blocks_per_sm": 0,
            "refill_threshold": 16, "chunk_tiles": 2, "inner_iters": 4}
    best_ms = run(best)
    # refill 1 with 128 steps per round is the "no compaction" end: a warp traces its 32
    # rays until all of them end (up to the iteration cap) before it takes new ones
    stages = [
        [dict(tile_w=tw, tile_h=th, morton=m, warps_per_block=wp)
         for (tw, th, m), wp in itertools.product([(8, 8, 0), (8, 8, 1), (16, 4, 0), (32, 1, 0)], [2, 4, 8])],
        [dict(refill_threshold=r, inner_iters=i)
         for r, i in itertools.product([1, 2, 4, 8, 12, 16, 20, 24, 28], [4, 8, 16, 32, 64, 128])],
        [dict(chunk_tiles=c) for c in (1, 2, 4, 8, 16, 32, 64)],
    ]
    tried = set()
    for _ in range(passes):
        for stage in stages:
            for delta in stage:
                d = {**best, **delta}
                key = tuple(sorted(d.items()))
                if d == best or key in tried:
                    continue
                tried.add(key)
                ms = run(d)
                if ms < best_ms:
                    best, best_ms = d, ms
    return best, best_ms, trials


def main(argv=None) -> None:
    """python -m voxelrt_gb300.autotune [--workload uneven_batch] [--out PATH]

    Tunes the batched launch on a workload of voxelrt_gb300.workloads and stores the
    winner under this GPU's name (default: the user cache)."""
    import argparse
    import json as _json

    import torch

    from . import World
    from . import workloads as W

    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="uneven_batch", choices=["uneven_batch", "large_world", "incoherent"])
    ap.add_argument("--out", default=None)
    ap.add_argument("--worlds", type=int, default=128)
    a = ap.parse_args(argv)
    if a.workload == "uneven_batch":
        wl = W.uneven_batch(n_worlds=a.worlds)
    elif a.workload == "large_world":
        wl = W.large_world()
    else:
        wl = W.incoherent()
    worlds = []
    for d in wl.worlds:
        w = World(d.sectors, brick_capacity=d.n_bricks + 64)
        w.upload(d)
        worlds.append(w)
    from . import Batch
    records = Batch(worlds, wl.views).total_records
    hits = torch.empty(records * 16, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    best, ms, trials = tune(worlds, wl.views, hits, stream)
    rays = wl.primary_rays
    path = store(wl.name, best, {"ms": ms, "primary_rays": rays, "trials": len(trials)},
                 path=Path(a.out) if a.out else None)
    print(_json.dumps({"workload": wl.name, "best": best, "ms": ms, "gpu": gpu_name(), "stored": str(path)}))


if __name__ == "__main__":
    main()
