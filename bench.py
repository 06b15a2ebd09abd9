#!/usr/bin/env python3
"""Benchmark of the brickmap traversal path (one JSON line on stdout).

Default workload: the uneven batch - 128 seeded worlds (edge 64..512 voxels) with
1-16 views each at 64^2..1280x720, every view's primary rays in ONE persistent
launch fed by the device tile queue and replayed from a CUDA graph.  The same line
reports the plain one-launch-per-view kernel on the same views (the comparison the
metric names), the end-to-end host-buffer call, the HBM roofline of the persistent
kernel, the CPU oracle timed on a bounded sample, the large-world (primary + shadow)
and incoherent (4 bounces + 2^26 random rays) workloads as sub-results, and the
request server under Poisson arrivals with edits, replayed against the oracle.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload uneven_batch|large_world|incoherent|single_view]

Multi-GPU: with --gpus N > 1 and no torchrun environment, bench.py starts itself
under torch.distributed.run with N ranks, one per GPU.  Every rank traverses its own
batch of the same shape (weak scaling, no collective on the data path); the time is
the max over ranks and the rays are the sum over ranks.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import socket
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# device bytes per brick slot: 512 payload + 512 voxel codes + 64 cell masks
SLOT_BYTES = 512 + 512 + 64
METRIC = "Grays/s batched vs per-view launch (bit-exact hits); p50/p99 request latency"
HIT_BYTES = 16
PACKED_BYTES = 12
BYTES_FORMULA = "8*step_calls + 12*occ_fetches + 1*hits + 16*records"


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="uneven_batch",
                    choices=["uneven_batch", "large_world", "incoherent", "single_view"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="bounded CPU-oracle sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-per-view", action="store_true")
    ap.add_argument("--no-serving", action="store_true", help="skip the request-server run")
    ap.add_argument("--no-sub", action="store_true",
                    help="uneven_batch: skip the large-world and incoherent sub-results")
    ap.add_argument("--sub-steps", type=int, default=5, help="timed launches of each sub-result")
    ap.add_argument("--no-stress", action="store_true", help="skip the 2^26 stress rays")
    ap.add_argument("--stress-rays", type=int, default=1 << 26, help="number of stress rays")
    ap.add_argument("--glsl", action="store_true",
                    help="trace every view in the GLSL mode (the GPU renderer's rayCast) instead of the CPU traversal")
    ap.add_argument("--aniso", action="store_true", help="the GLSL mode with anisotropic LODs (implies --glsl)")
    ap.add_argument("--serve-rates", default="50,200,1000,2000,8000,16000",
                    help="render requests per second to sweep (16000 puts the host link near its limit)")
    ap.add_argument("--serve-seconds", type=float, default=2.0, help="duration of each arrival-rate run, at least")
    ap.add_argument("--serve-min-requests", type=int, default=400,
                    help="renders per arrival rate, at least (longer runs at low rates)")
    ap.add_argument("--serve-worlds", type=int, default=32)
    ap.add_argument("--serve-max-edge", type=int, default=1024)
    ap.add_argument("--serve-check-worlds", type=int, default=8,
                    help="worlds (the largest and smallest among them) whose renders are replayed on the oracle")
    ap.add_argument("--serve-check-cap", type=int, default=200,
                    help="replayed renders per arrival rate and mode, at most")
    ap.add_argument("--l2-persist", action="store_true",
                    help="create the workload's worlds with VRT_WORLD_L2_PERSIST (an L2 access-policy window "
                         "over the brick table of a batch's single such world)")
    ap.add_argument("--worlds", type=int, default=128, help="uneven_batch: number of worlds")
    ap.add_argument("--max-views", type=int, default=16, help="uneven_batch: views per world, at most")
    ap.add_argument("--cameras", type=int, default=64, help="large_world: number of 1080p cameras")
    ap.add_argument("--renderer-path", action="store_true",
                    help="large_world: every view traces the GPU renderer's whole per-pixel path (primary, sun, "
                         "3 bounces, a sun ray after the first two) instead of primary + shadow")
    ap.add_argument("--scaling", default="weak", choices=["weak", "strong"],
                    help="N>1: every rank traces its own batch (weak) or a share, by world, of one batch (strong)")
    return ap.parse_args(argv)


# ---------------------------------------------------------------------------------------
# ranks

def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def relaunch_cmd(gpus: int, argv: list[str], port: int) -> list[str]:
    """The torchrun command that runs this script as `gpus` ranks on this node."""
    return [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={gpus}",
            "--master-addr", "127.0.0.1", "--master-port", str(port), str(Path(__file__).resolve()), *argv]


def rank_env():
    """(world size, rank, local rank) of this process (1, 0, 0 without torchrun)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def dist_setup(backend: str = "nccl"):
    """Process group of a torchrun job (None for one process).  nccl binds the rank's GPU;
    gloo (CPU) is what the multi-rank tests use."""
    ws, rank, local = rank_env()
    pg = None
    if ws > 1:
        import torch
        import torch.distributed as dist
        if backend == "nccl":
            torch.cuda.set_device(local)
            dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        else:
            dist.init_process_group(backend)
        pg = dist
    return ws, rank, local, pg


def barrier(pg):
    from voxelrt_gb300 import shard
    shard.barrier(pg)


def max_over_ranks(pg, x: float, device="cuda") -> float:
    from voxelrt_gb300 import shard
    return shard.max_over_ranks(pg, x, device)


def sum_over_ranks(pg, x: float, device="cuda") -> float:
    from voxelrt_gb300 import shard
    return shard.sum_over_ranks(pg, x, device)


# ---------------------------------------------------------------------------------------
# workloads

def build_workload(name: str, rank: int, args=None, world_size: int = 1):
    """The rank's workload: its own seeded batch (weak scaling) or its share, by world, of
    the one batch (strong scaling, uneven_batch only).  With --glsl every view traces in
    the GLSL mode (the GPU renderer's rayCast)."""
    wl = _build_workload(name, rank, args, world_size)
    if args is not None and (getattr(args, "glsl", False) or getattr(args, "aniso", False)):
        from voxelrt_gb300 import capi
        aniso = getattr(args, "aniso", False)
        for vw in wl.views:
            vw.flags |= capi.VIEW_GLSL | (capi.VIEW_GLSL_ANISO if aniso else 0)
        wl.description += ", GLSL traversal mode" + (" with anisotropic LODs" if aniso else "")
    return wl


def _build_workload(name: str, rank: int, args=None, world_size: int = 1):
    from voxelrt_gb300 import shard
    from voxelrt_gb300 import workloads as W
    if name == "uneven_batch":
        nw = args.worlds if args is not None else 128
        mv = args.max_views if args is not None else 16
        strong = args is not None and getattr(args, "scaling", "weak") == "strong" and world_size > 1
        wl = W.uneven_batch(n_worlds=nw, max_views=mv, seed=2 if strong else shard.rank_seed(2, rank))
        if strong:
            worlds, views, own = shard.shard_batch(wl.worlds, wl.views, rank, world_size)
            wl = W.Workload(wl.name, worlds, views, f"{wl.description}, worlds {own} of {world_size} ranks")
        return wl
    if name == "large_world":
        wl = W.large_world(n_cameras=args.cameras if args is not None else 64)
        if args is not None and getattr(args, "renderer_path", False):
            from voxelrt_gb300 import make_view
            sun = tuple(float(c) for c in wl.views[0].sun_dir)
            wl.views = [make_view(vw.cam, n_bounces=3, shadow_dir=sun) for vw in wl.views]
            wl.description = (f"2048x256x2048 terrain+caves, {len(wl.views)} cameras 1920x1080, the GPU renderer's "
                              "whole path (primary, sun, 3 bounces, a sun ray after the first two)")
            # no tuned entry: the library's defaults for views with bounces, not the camera-ray table entry
            wl.name = "large_world_renderer_path"
        return wl
    if name == "incoherent":
        return W.incoherent()
    return W.single_view()


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


# What bounds the persistent kernel on a workload, from the committed ncu summaries.
LIMITERS = {
    "uneven_batch": "instruction issue: 72.5 % of issue slots busy, wait (fixed-latency dependency) the first "
                    "stall (profiles/persistent_kernel_uneven_batch_medium.md)",
}


def traffic_from_profile(workload: str, args=None):
    """DRAM bytes per launch of the persistent kernel from a committed ncu summary, for
    the configuration that summary covers (the workload at its default sizes, default
    traversal); None for any other."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    if args is not None and (args.glsl or args.aniso or args.worlds != 128 or args.max_views != 16 or
                             getattr(args, "cameras", 64) != 64 or getattr(args, "renderer_path", False)):
        return None
    try:
        return json.loads(p.read_text()).get(workload)
    except Exception:
        return None


def host_cores() -> int:
    """CPUs this process may run on (the affinity set), not the machine's count."""
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


def traversal_name(args) -> str:
    return "glsl_aniso" if args.aniso else "glsl" if args.glsl else "cpu"


def view_is_glsl(vw) -> bool:
    from voxelrt_gb300 import capi
    return bool(vw.flags & capi.VIEW_GLSL)


def view_is_aniso(vw) -> bool:
    from voxelrt_gb300 import capi
    return bool(vw.flags & capi.VIEW_GLSL_ANISO)


def oracle_view(o, vw):
    """Every record of a view from the oracle, shaped (kinds, width*height)."""
    glsl, aniso = view_is_glsl(vw), view_is_aniso(vw)
    if vw.flags & 1 and vw.n_bounces:
        return o.render_view_path(vw.cam, np.array(vw.sun_dir[:], np.float32), vw.n_bounces, vw.max_iters,
                                  glsl=glsl, aniso=aniso)
    if vw.flags & 1:
        return np.stack(o.render_view_shadow(vw.cam, np.array(vw.sun_dir[:], np.float32), vw.max_iters,
                                             glsl=glsl, aniso=aniso))
    if vw.n_bounces:
        return o.render_view_bounces(vw.cam, vw.n_bounces, vw.max_iters, glsl=glsl, aniso=aniso)
    return o.render_view(vw.cam, vw.max_iters, glsl=glsl, aniso=aniso)[None]


def cpu_oracle_sample(wl, seconds: float, threads: int = 0):
    """Time the CPU oracle on whole views of the workload until `seconds` of work."""
    from oracle.oracle import OracleWorld
    order = np.argsort([vw.cam.width * vw.cam.height for vw in wl.views], kind="stable")
    cache = {}
    rays, elapsed, nviews = 0, 0.0, 0
    for i in order:
        vw = wl.views[int(i)]
        if vw.world not in cache:
            cache.clear()
            o = OracleWorld(wl.worlds[vw.world].sectors)
            o.upload(wl.worlds[vw.world])
            cache[vw.world] = o
        o = cache[vw.world]
        glsl, aniso = view_is_glsl(vw), view_is_aniso(vw)
        t0 = time.perf_counter()
        if vw.flags & 1 and vw.n_bounces:
            o.render_view_path(vw.cam, np.array(vw.sun_dir[:], np.float32), vw.n_bounces, vw.max_iters, threads,
                               glsl=glsl, aniso=aniso)
        elif vw.flags & 1:
            o.render_view_shadow(vw.cam, np.array(vw.sun_dir[:], np.float32), vw.max_iters, threads, glsl=glsl,
                                 aniso=aniso)
        elif vw.n_bounces:
            o.render_view_bounces(vw.cam, vw.n_bounces, vw.max_iters, threads, glsl=glsl, aniso=aniso)
        else:
            o.render_view(vw.cam, vw.max_iters, threads, glsl=glsl, aniso=aniso)
        elapsed += time.perf_counter() - t0
        rays += o.last_stats["rays"]
        nviews += 1
        if elapsed >= seconds:
            break
    return rays, elapsed, nviews


def run_reference(args):
    """Reference arm: the CPU restatement of the reference traversal on all host cores.
    Loads the oracle and the host-only input generators, never the product library."""
    ws, rank, _ = rank_env()
    if rank != 0:
        return
    from voxelrt_gb300 import build
    build.build_oracle()
    build.build_synth()
    wl = build_workload(args.workload, 0, args)
    cores = host_cores()
    per_step = max(2.0, min(20.0, args.cpu_seconds))
    for _ in range(args.warmup):
        cpu_oracle_sample(wl, 0.5, cores)
    tot_rays, tot_t = 0, 0.0
    nv = 0
    for _ in range(args.steps):
        r, t, nv = cpu_oracle_sample(wl, per_step, cores)
        tot_rays += r
        tot_t += t
    value = tot_rays / tot_t / 1e9
    algo = ("VoxelTraversal.glsl rayCast" + (" with anisotropic LODs" if args.aniso else "")
            if args.glsl or args.aniso else "CpuRenderer.cpp RayCast")
    sample = (f"{nv} smallest views of the {wl.name} workload per step ({tot_rays // max(args.steps, 1)} rays), "
              f"scalar C++ restatement of {algo}, all {cores} host threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Grays/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": wl.name, "description": wl.description,
                   "traversal": traversal_name(args)},
        "cpu_baseline": {"value": value, "unit": "Grays/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "Grays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------
# our arm: an engine measures one rank; run_ours reduces over ranks and prints the line

class GpuEngine:
    """One rank's measurement on its GPU: the persistent batch (CUDA graph), the per-view
    launches, the end-to-end host-buffer call, and on rank 0 the parity sample, the CPU
    baseline, the sub-results and the serving run."""

    def __init__(self, args, rank: int, world_size: int, local: int):
        import torch

        import voxelrt_gb300 as v
        from voxelrt_gb300 import autotune
        self.args, self.rank, self.dev = args, rank, local
        self.torch, self.v = torch, v
        torch.cuda.set_device(local)
        self.wl = build_workload(args.workload, rank, args, world_size)
        self.worlds = []
        flags = 1 if getattr(args, "l2_persist", False) else 0  # VRT_WORLD_L2_PERSIST
        for d in self.wl.worlds:
            w = v.World(d.sectors, brick_capacity=d.n_bricks + 64, device=local, flags=flags)
            w.upload(d)
            self.worlds.append(w)
        self.cfg, self.cfg_src = autotune.lookup(self.wl.name)
        self.batch = v.Batch(self.worlds, self.wl.views, self.cfg)
        self.n_rec = self.batch.total_records
        self.stream = torch.cuda.Stream()
        self.hits = torch.empty(self.n_rec * HIT_BYTES, dtype=torch.uint8, device=f"cuda:{local}")
        self.parity = parity_sample(self.wl, self.batch, self.hits, self.stream) if rank == 0 else None
        # counting launch (untimed): algorithmic bytes of one launch
        self.meas = self.batch.measure(self.hits, self.stream)
        self.rays_per_step = self.meas["rays_cast"]
        m = self.meas
        self.alg_bytes = 8 * m["step_calls"] + 12 * m["occ_fetches"] + 1 * m["hits"] + HIT_BYTES * self.n_rec
        self.h2d_bytes = 128 * len(self.wl.views)
        # end to end the records arrive as vrt_hit_packed (12 bytes: the per-ray output
        # without the 16-byte record's tag, which a record's position already gives)
        self.d2h_bytes = self.n_rec * PACKED_BYTES
        self.ms = None

    def time_batched(self, sync):
        """ms per persistent launch (graph replay) over `steps`, and the clocks meanwhile."""
        torch, s = self.torch, self.stream
        with torch.cuda.stream(s):
            for _ in range(max(3, self.args.warmup)):
                self.batch.launch(self.hits, s, graph=True)
        s.synchronize()
        sync()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(self.dev) as clk:
            torch.cuda.synchronize()
            sync()
            ev0.record(s)
            for _ in range(self.args.steps):
                self.batch.launch(self.hits, s, graph=True)
            ev1.record(s)
            ev1.synchronize()
            torch.cuda.synchronize()
        sync()
        self.ms = ev0.elapsed_time(ev1) / self.args.steps
        self.ms_l2_flushed = self._time_l2_flushed()
        return self.ms, clk.summary()

    def _time_l2_flushed(self, flush_bytes=512 << 20):
        """ms per launch with L2 flushed before each one (a 512 MiB write, four times L2, not
        timed): the bricks a batch touches fit in L2 across launches, so this shows what the
        first touch of every line costs."""
        torch, s = self.torch, self.stream
        flush = torch.empty(flush_bytes, dtype=torch.uint8, device=self.hits.device)
        evs = []
        with torch.cuda.stream(s):
            for i in range(self.args.steps):
                flush.fill_(i & 0xFF)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(s)
                self.batch.launch(self.hits, s, graph=True)
                e1.record(s)
                evs.append((e0, e1))
        s.synchronize()
        del flush
        return sum(a.elapsed_time(b) for a, b in evs) / len(evs)

    def time_per_view(self):
        """ms per pass of one plain launch per view over the same views."""
        torch, s = self.torch, self.stream
        with torch.cuda.stream(s):
            for _ in range(2):
                self.batch.launch_per_view(self.hits, s)
        s.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        k = max(1, min(self.args.steps, 5))
        e0.record(s)
        for _ in range(k):
            self.batch.launch_per_view(self.hits, s)
        e1.record(s)
        e1.synchronize()
        return e0.elapsed_time(e1) / k, k

    def _time_run(self, sync, run, host):
        """Seconds per call of update_cameras + `run` into `host`, and each call's ms."""
        cams = [vw.cam for vw in self.wl.views]
        self.batch.update_cameras(cams, self.stream)
        run(host.array, self.stream)
        ke = max(1, 2 * self.args.steps)  # calls of about 23-31 ms: twice the timed launches
        sync()
        calls = []  # each call returns once its records are in host memory
        # Python's collector stays off while the calls are timed, as timeit does: a full
        # collection over this process's objects is a pause of the harness, not of the call
        gc.collect()
        gc.disable()
        try:
            t0 = time.perf_counter()
            for _ in range(ke):
                t1 = time.perf_counter()
                self.batch.update_cameras(cams, self.stream)
                run(host.array, self.stream)
                calls.append((time.perf_counter() - t1) * 1e3)
            total = time.perf_counter() - t0
        finally:
            gc.enable()
        return total / ke, calls

    def time_e2e(self, sync):
        """Seconds per end-to-end call through the host-buffer API: new cameras in (H2D), all
        records out to pinned host memory from vrt_host_alloc (the copies of finished parts
        overlap the traversal of later ones), as 12-byte records (vrt_batch_run_packed).  The
        16-byte records (vrt_batch_run) are timed beside them, and every packed record is
        checked against its 16-byte record."""
        v = self.v
        full = v.PinnedHits(self.n_rec)
        self.e2e_full = self._time_run(sync, self.batch.run, full)
        packed = v.PinnedHits(self.n_rec, dtype=v.PACKED_DTYPE)
        sec, self.e2e_calls_ms = self._time_run(sync, self.batch.run_packed, packed)
        f = full.array.view(np.uint32).reshape(-1, 4)
        g = packed.array.view(np.uint32).reshape(-1, 3)
        no_ray = f[:, 3] == v.NO_RAY
        word1 = np.where(no_ray, (f[:, 1] & 0xFFFF00FF) | (v.PACKED_NO_RAY << 8), f[:, 1])
        self.e2e_packed_exact = bool(np.array_equal(f[:, 0], g[:, 0]) and np.array_equal(word1, g[:, 1])
                                     and np.array_equal(f[:, 2], g[:, 2]))
        del f, g, no_ray, word1
        full.close()
        packed.close()
        return sec

    def d2h_link_gbs(self):
        return d2h_link_gbs(self.torch, self.stream)

    def config(self):
        from voxelrt_gb300 import autotune
        wl = self.wl
        return {"workload": wl.name, "description": wl.description, "worlds": len(wl.worlds),
                "views": len(wl.views), "rays_per_step": self.rays_per_step, "records_per_step": self.n_rec,
                "world_bytes": int(sum(d.n_bricks for d in wl.worlds) * SLOT_BYTES),
                "l2": "inputs larger than L2 (brick pools of all worlds); l2_flushed: the same launches, each after an L2 flush",
                "batch_config": autotune.describe(self.cfg), "batch_config_source": self.cfg_src,
                "launch": "persistent kernel + queue reset, CUDA graph replay",
                "traversal": traversal_name(self.args),
                "l2_persist": bool(getattr(self.args, "l2_persist", False))}

    def extras(self):
        """Rank 0's further results (parity, roofline inputs, CPU baseline, sub-results,
        serving); frees the batch's device memory first where a later part needs it."""
        args, v = self.args, self.v
        out = {"parity_sample": self.parity,
               "traversal": {"step_calls": self.meas["step_calls"], "occ_fetches": self.meas["occ_fetches"],
                             "hits": self.meas["hits"],
                             "mean_steps_per_ray": self.meas["step_calls"] / max(self.rays_per_step, 1)}}
        peak, peak_src = peak_hbm()
        achieved = self.alg_bytes / (self.ms * 1e-3) / 1e9
        traffic = traffic_from_profile(self.wl.name, args)
        out["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                           "traffic": traffic, "peak_source": peak_src,
                           "algorithmic_bytes_per_launch": self.alg_bytes, "bytes_formula": BYTES_FORMULA}
        if traffic:
            # what DRAM actually moved per launch, against the same peak: the brick data stays in
            # L2/L1, so this fraction is far below the algorithmic one
            out["roofline"]["dram_frac"] = traffic / (self.ms * 1e-3) / 1e9 / peak
            out["roofline"]["limiter"] = LIMITERS.get(self.wl.name)
        cpu = None
        if not args.no_cpu:
            cores = host_cores()
            r, t, nv = cpu_oracle_sample(self.wl, args.cpu_seconds, cores)
            cpu = {"value": r / t / 1e9, "unit": "Grays/s", "cores": cores, "kind": "port",
                   "sample": f"{nv} smallest views of the workload, {r} rays, CPU oracle (scalar restatement of "
                             f"CpuRenderer.cpp RayCast) on all host threads"}
        out["cpu_baseline"] = cpu
        if args.workload == "incoherent" and not args.no_stress:
            out["stress"] = run_stress(v, self.worlds[0], self.wl.worlds[0], args, self.stream, n=args.stress_rays)
        self.close()
        if args.workload == "uneven_batch" and not args.no_sub:
            out["sub_results"] = run_sub_results(args, self.dev)
        if args.workload == "uneven_batch" and not args.no_serving:
            out["serving"] = run_serving(args, self.dev)
        return out

    def close(self):
        if self.batch is not None:
            self.batch.close()
            self.batch = None
            self.hits = None
            for w in self.worlds:
                w.close()
            self.worlds = []
            self.torch.cuda.synchronize()
            self.torch.cuda.empty_cache()


def run_ours(args, engine_cls=None, backend: str = "nccl", device: str = "cuda"):
    """Measure on every rank with `engine_cls` (GpuEngine by default), reduce over ranks
    (time: max, rays and bytes: sum) and print rank 0's JSON line."""
    ws, rank, local, pg = dist_setup(backend)
    eng = (engine_cls or GpuEngine)(args, rank, ws, local)
    sync = lambda: barrier(pg)  # noqa: E731
    ms_rank, clocks = eng.time_batched(sync)
    ms = max_over_ranks(pg, ms_rank, device)
    job_rays = sum_over_ranks(pg, eng.rays_per_step, device)
    value = job_rays / (ms * 1e-3) / 1e9

    per_view = None
    if not args.no_per_view:
        pms_rank, k = eng.time_per_view()
        pms = max_over_ranks(pg, pms_rank, device)
        per_view = {"value": job_rays / (pms * 1e-3) / 1e9, "unit": "Grays/s", "ms_per_step": pms,
                    "launches_per_step": int(sum_over_ranks(pg, len(eng.wl.views), device)), "steps": k,
                    "kernel": "view_path_kernel, 8x8 blocks, thread per pixel"}

    link_before = eng.d2h_link_gbs()
    e2e_s = max_over_ranks(pg, eng.time_e2e(sync), device)
    d2h = sum_over_ranks(pg, eng.d2h_bytes, device)
    e2e = {"value": job_rays / e2e_s / 1e9, "unit": "Grays/s", "ms_per_step": e2e_s * 1e3,
           "h2d_bytes_per_step": int(sum_over_ranks(pg, eng.h2d_bytes, device)), "d2h_bytes_per_step": int(d2h),
           "api": "vrt_batch_update_cameras + vrt_batch_run_packed (12-byte records into pinned host memory)"}
    full = getattr(eng, "e2e_full", None)
    if full:  # the same calls delivering 16-byte records (with tags), this rank's time
        e2e["full_records"] = {"value": eng.rays_per_step / full[0] / 1e9, "unit": "Grays/s",
                               "ms_per_step": full[0] * 1e3, "d2h_bytes_per_step": eng.n_rec * HIT_BYTES,
                               "api": "vrt_batch_update_cameras + vrt_batch_run (16-byte records)",
                               "calls_ms": [round(c, 3) for c in full[1]]}
    if hasattr(eng, "e2e_packed_exact"):
        e2e["packed_equal_full"] = eng.e2e_packed_exact
    link = eng.d2h_link_gbs()
    e2e["d2h_link_gbs"] = link
    e2e["d2h_link_gbs_before"] = link_before
    e2e["d2h_link_frac"] = eng.d2h_bytes / (e2e_s * 1e9) / max(link, link_before)
    calls = getattr(eng, "e2e_calls_ms", None)
    if calls:  # this rank's calls: a slow mean from a few stalled calls shows here
        e2e["calls_ms"] = {"n": len(calls), "min": min(calls), "median": sorted(calls)[len(calls) // 2],
                           "max": max(calls), "each": [round(c, 3) for c in calls]}
    barrier(pg)

    if rank == 0:
        extra = eng.extras()
        line = {
            "metric": METRIC, "value": value, "unit": "Grays/s", "n_gpus": ws, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True, "scaling": args.scaling,
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": eng.config(),
            "roofline": extra.pop("roofline"), "cpu_baseline": extra.pop("cpu_baseline"), "e2e": e2e,
            "gpu_launches": args.steps, "clocks": clocks, "per_view": per_view,
            "batched_over_per_view": (value / per_view["value"]) if per_view else None,
            "job_rays_per_step": job_rays,
        }
        fl = getattr(eng, "ms_l2_flushed", None)
        if fl:  # this rank's launches, each after a 512 MiB write that evicts L2
            line["l2_flushed"] = {"ms_per_step": fl, "value": eng.rays_per_step / (fl * 1e-3) / 1e9,
                                  "unit": "Grays/s", "flush_bytes": 512 << 20}
        line.update(extra)
        print(json.dumps(line), flush=True)
    else:
        eng.close()
    barrier(pg)
    if pg is not None:
        pg.destroy_process_group()


# ---------------------------------------------------------------------------------------
# sub-results: the large world (config 1) and the incoherent workload (config 3)

def measure_workload(v, wl, dev, steps, stream, check_views=2, stress=None, hook=None):
    """Persistent-launch throughput of one workload (CUDA graph replay, inputs resident),
    its roofline and an oracle check of `check_views` whole views.  hook(v, worlds, wl,
    stream) -> dict adds further measurements on the same resident worlds."""
    import torch

    from voxelrt_gb300 import autotune
    worlds = []
    for d in wl.worlds:
        w = v.World(d.sectors, brick_capacity=d.n_bricks + 64, device=dev)
        w.upload(d)
        worlds.append(w)
    cfg, src = autotune.lookup(wl.name)
    batch = v.Batch(worlds, wl.views, cfg)
    n_rec = batch.total_records
    hits = torch.empty(n_rec * HIT_BYTES, dtype=torch.uint8, device=f"cuda:{dev}")
    parity = parity_sample(wl, batch, hits, stream, max_views=check_views, pick="largest")
    meas = batch.measure(hits, stream)
    alg = 8 * meas["step_calls"] + 12 * meas["occ_fetches"] + meas["hits"] + HIT_BYTES * n_rec
    with torch.cuda.stream(stream):
        for _ in range(3):
            batch.launch(hits, stream, graph=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        batch.launch(hits, stream, graph=True)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    # the plain one-launch-per-view kernel on the same views
    for _ in range(2):
        batch.launch_per_view(hits, stream)
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    for _ in range(steps):
        batch.launch_per_view(hits, stream)
    p1.record(stream)
    p1.synchronize()
    pms = p0.elapsed_time(p1) / steps
    peak, peak_src = peak_hbm()
    out = {"workload": wl.name, "description": wl.description, "value": meas["rays_cast"] / (ms * 1e-3) / 1e9,
           "per_view": {"value": meas["rays_cast"] / (pms * 1e-3) / 1e9, "ms_per_step": pms,
                        "launches_per_step": len(wl.views)},
           "batched_over_per_view": pms / ms,
           "unit": "Grays/s", "ms_per_step": ms, "steps": steps, "rays_per_step": meas["rays_cast"],
           "records_per_step": n_rec, "mean_steps_per_ray": meas["step_calls"] / max(meas["rays_cast"], 1),
           "roofline": {"achieved": alg / (ms * 1e-3) / 1e9, "peak": peak, "frac": alg / (ms * 1e-3) / 1e9 / peak,
                        "peak_source": peak_src, "algorithmic_bytes_per_launch": alg},
           "batch_config": autotune.describe(cfg), "batch_config_source": src,
           "world_bytes": int(sum(d.n_bricks for d in wl.worlds) * SLOT_BYTES), "parity_sample": parity}
    del hits
    batch.close()
    if stress is not None:
        out["stress"] = run_stress(v, worlds[0], wl.worlds[0], stress, stream, n=stress.stress_rays)
    if hook is not None:
        out.update(hook(v, worlds, wl, stream))
    for w in worlds:
        w.close()
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return out


def run_sub_results(args, dev):
    """Configs 1 and 3 at their full sizes, each with its own persistent launch."""
    import torch

    import voxelrt_gb300 as v
    from voxelrt_gb300 import workloads as W
    stream = torch.cuda.Stream()
    out = {}
    for name, make in (("large_world", W.large_world), ("incoherent", W.incoherent)):
        wl = make()
        if args.glsl or args.aniso:
            for vw in wl.views:
                vw.flags |= v.VIEW_GLSL | (v.capi.VIEW_GLSL_ANISO if args.aniso else 0)
        stress = args if (name == "incoherent" and not args.no_stress) else None
        hook = None
        if not (args.glsl or args.aniso):
            hook = renderer_rows if name == "large_world" else cvox_round_trip
        out[name] = measure_workload(v, wl, dev, args.sub_steps, stream, stress=stress, hook=hook)
    return out


def _projection(aspect, near=0.1, far=4000.0, fov=90.0):
    """A perspective matrix, column-major (glm layout), for the G-buffer's projected depth."""
    f = 1.0 / np.tan(np.radians(fov) / 2)
    p = np.zeros((4, 4))
    p[0, 0], p[1, 1] = f / aspect, f
    p[2, 2], p[2, 3] = (far + near) / (near - far), 2 * far * near / (near - far)
    p[3, 2] = -1.0
    return p.T.astype(np.float32).reshape(16)


def _time_ms(stream, fn, reps=5):
    import torch
    with torch.cuda.stream(stream):
        fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def renderer_rows(v, worlds, wl, stream):
    """On the large world: the G-buffer of a 1080p view (vrt_render_gbuffer_device) and the GPU
    renderer's whole per-pixel path (primary, sun, 3 bounces with a sun ray after the first two)
    over 8 1080p views in one persistent launch.  Each is checked against the oracle on a
    320x180 view of the same camera."""
    import torch

    from oracle.oracle import OracleWorld
    w, d = worlds[0], wl.worlds[0]
    cams = [vw.cam for vw in wl.views[:8]]
    rng = np.random.default_rng(5)
    pal = rng.integers(0, 1 << 16, 256, dtype=np.uint32) | rng.integers(0, 1 << 16, 256, dtype=np.uint32) << 16
    pal[0] = 0
    proj = _projection(16 / 9)
    # G-buffer, device buffers, primary records included
    view = v.make_view(cams[0])
    n = cams[0].width * cams[0].height
    d_tex = torch.empty(n, dtype=torch.int32, device="cuda")
    d_depth = torch.empty(n, dtype=torch.float32, device="cuda")
    d_hits = torch.empty(n * HIT_BYTES, dtype=torch.uint8, device="cuda")
    ss = stream.cuda_stream

    def gbuf():
        v.check(v.lib().vrt_render_gbuffer_device(w.handle, v.capi.C.byref(view), pal.ctypes.data, proj.ctypes.data,
                                                  d_tex.data_ptr(), d_depth.data_ptr(), d_hits.data_ptr(), ss))
    g_ms = _time_ms(stream, gbuf)
    del d_tex, d_depth, d_hits
    # the renderer's whole path, 8 views in one batch
    sun = tuple(float(c) for c in wl.views[0].sun_dir)
    pviews = [v.make_view(c, n_bounces=3, shadow_dir=sun) for c in cams]
    b = v.Batch(worlds, pviews)
    ph = torch.empty(b.total_records * HIT_BYTES, dtype=torch.uint8, device="cuda")
    p_ms = _time_ms(stream, lambda: b.launch(ph, stream, graph=True))
    st = b.measure(ph, stream)
    del ph
    b.close()
    # oracle checks on a 320x180 view of the first camera
    o = OracleWorld(d.sectors)
    o.upload(d)
    sc = _scaled_camera(v, cams[0], 320, 180)
    tex, depth = v.render_gbuffer(w, v.make_view(sc), pal, proj)
    want_tex, want_depth, _ = o.render_gbuffer(sc, pal, proj)
    g_ok = bool(np.array_equal(tex, want_tex) and np.array_equal(depth.view(np.uint32), want_depth.view(np.uint32)))
    sb = v.Batch(worlds, [v.make_view(sc, n_bounces=3, shadow_dir=sun)])
    got = sb.view_hits(sb.run(), 0)
    sb.close()
    want = o.render_view_path(sc, np.array(sun, np.float32), 3)
    p_ok = bool(got.shape == want.shape and all(hits_match(got[k], want[k]) for k in range(got.shape[0])))
    o.close()
    return {"gbuffer": {"api": "vrt_render_gbuffer_device", "view": "1920x1080", "ms": g_ms,
                        "mpix_s": n / (g_ms * 1e-3) / 1e6, "checked": "320x180 view of the same camera",
                        "bit_exact": g_ok},
            "renderer_path": {"api": "vrt_batch (persistent launch, graph replay)", "views": "8 x 1920x1080",
                              "path": "primary, sun, 3 bounces, a sun ray after the first two", "ms": p_ms,
                              "rays": st["rays_cast"], "value": st["rays_cast"] / (p_ms * 1e-3) / 1e9,
                              "unit": "Grays/s", "checked": "320x180 view of the first camera", "bit_exact": p_ok}}


def _scaled_camera(v, cam, width, height):
    """The camera `cam` at another resolution: the same eye and image plane (d0 is the plane's
    corner, du and dv one pixel's step), so the same field of view."""
    c = v.Camera()
    C = v.capi.C
    C.memmove(C.byref(c), C.byref(cam), C.sizeof(c))
    sx, sy = cam.width / width, cam.height / height
    for i in range(3):
        c.du[i] = cam.du[i] * sx
        c.dv[i] = cam.dv[i] * sy
    c.width, c.height = width, height
    return c


def cvox_round_trip(v, worlds, wl, stream):
    """On the 1024^3 world: save to a cvox v4 file (vrt_world_save_cvox) and load it into a new
    world (vrt_world_load_cvox); the loaded world must cast 64 Ki random rays exactly as the
    original."""
    import tempfile
    import time as _t

    w, d = worlds[0], wl.worlds[0]
    with tempfile.TemporaryDirectory() as tmp:
        path = Path(tmp) / "world.cvox"
        t0 = _t.perf_counter()
        w.save_cvox(path)
        t_save = _t.perf_counter() - t0
        size = path.stat().st_size
        w2 = v.World(d.sectors, brick_capacity=d.n_bricks + 64)
        t0 = _t.perf_counter()
        w2.load_cvox(path)
        v.check(v.lib().vrt_world_wait(w2.handle))
        t_load = _t.perf_counter() - t0
    rays = v.random_rays([c * 32 for c in d.sectors], seed=11, n=1 << 16)
    same = bool(np.array_equal(w.cast(rays).view(np.uint8), w2.cast(rays).view(np.uint8)))
    w2.close()
    bricks_mb = d.n_bricks * 512 / 1e6
    return {"cvox": {"api": "vrt_world_save_cvox / vrt_world_load_cvox", "file_mb": size / 1e6,
                     "brick_mb": bricks_mb, "save_s": t_save, "load_s": t_load,
                     "save_mb_s": bricks_mb / t_save, "load_mb_s": bricks_mb / t_load,
                     "check": "64 Ki random rays cast on the loaded world equal the original's", "bit_exact": same}}


# ---------------------------------------------------------------------------------------
# serving

def surface_points(w, edge, n, seed):
    """Random surface voxels: rays cast straight down from the top of random columns."""
    import voxelrt_gb300 as v
    rng = np.random.default_rng(seed)
    org = np.stack([rng.uniform(0, edge, n), np.full(n, edge - 0.5), rng.uniform(0, edge, n)], 1)
    d = np.tile(np.array([[1e-4, -1.0, 1e-4]], np.float32), (n, 1))
    rays = np.zeros(n, v.RAY_DTYPE)
    rays["origin"], rays["dir"] = org.astype(np.float32), d
    h = w.cast(rays, max_iters=1000)
    vox = v.unpack_voxel(h["voxel"][h["voxel"] != v.MISS_VOXEL])
    return vox if len(vox) else np.array([[edge // 2, edge // 2, edge // 2]])


def load_serving_worlds(v, datas, dev):
    """Resident worlds with a quarter of their bricks (and at least 4096 slots) of pool room for
    the edits, which relocate the sectors they grow."""
    worlds, edges, surf = [], [], []
    for i, d in enumerate(datas):
        w = v.World(d.sectors, brick_capacity=d.n_bricks + max(4096, d.n_bricks // 4), device=dev)
        w.upload(d)
        worlds.append(w)
        edges.append(d.sectors[0] * 32)
        surf.append(surface_points(w, edges[-1], 256, seed=i))
    return worlds, edges, surf


def check_worlds(edges, n) -> list[int]:
    """Worlds whose renders the oracle replays: the largest, the smallest, and the rest
    drawn evenly from the others by edge."""
    order = sorted(range(len(edges)), key=lambda i: (edges[i], i))
    n = min(n, len(order))
    if n >= len(order):
        return order
    picks = {order[-1], order[0]}
    k = 1
    while len(picks) < n:
        picks.add(order[(k * (len(order) - 1)) // (n - 1)])
        k += 1
    return sorted(picks)


def run_serving(args, dev):
    """Poisson render arrivals (+100 edits/s) against the request server, per arrival rate,
    in both scheduling modes, each on freshly uploaded worlds: the default, one resident
    launch taking requests while it runs (top-level rates), and a launch per batch of
    queued requests ("launches")."""
    import voxelrt_gb300 as v
    from voxelrt_gb300 import workloads as W
    datas = W.serving_worlds(n_worlds=args.serve_worlds, max_edge=args.serve_max_edge)
    modes = {}
    reserve = SampleReserve(v, args.serve_check_cap)
    for name, resident in (("launches", False), ("resident", True)):
        worlds, edges, surf = load_serving_worlds(v, datas, dev)
        modes[name] = serve_sweep(args, v, datas, worlds, edges, surf, resident, reserve)
        if name != "resident":
            for w in worlds:
                w.close()
    reserve.close()
    edit_lat = edit_latency(v, worlds, edges, surf)
    for w in worlds:
        w.close()
    return {"worlds": len(datas), "max_edge": max(edges), "world_bytes": int(sum(d.n_bricks for d in datas) * SLOT_BYTES),
            "edit_latency": edit_lat, "resolutions": "256^2 / 1280x720 / 1920x1080 at p 0.5 / 0.3 / 0.2",
            "edits_per_s": 100,
            "seconds_per_rate": f"max({args.serve_seconds}, {args.serve_min_requests} / rate): at least "
                                f"{args.serve_min_requests} renders per rate for the p99",
            "mode": "resident", "rates": modes["resident"]["rates"],
            "oracle_replay": modes["resident"]["oracle_replay"], "launches": modes["launches"],
            "pool_compactions": modes["resident"]["pool_compactions"],
            "latency": "submit to records in pinned host memory, server clock"}


def d2h_link_gbs(torch, stream, nbytes=1 << 30, reps=3):
    """Device-to-host copy bandwidth into pinned memory (GB/s): the bound of the end-to-end
    leg, whose records all cross this link."""
    dev = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    host = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    with torch.cuda.stream(stream):
        host.copy_(dev, non_blocking=True)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            host.copy_(dev, non_blocking=True)
        b.record(stream)
    b.synchronize()
    return reps * nbytes / (a.elapsed_time(b) * 1e-3) / 1e9


class SampleReserve:
    """Pinned record buffers (1080p each) that stand in for the rotation buffers of renders
    kept for the oracle replay, so keeping a render's records costs the request loop no copy."""

    def __init__(self, v, n, max_rec=1920 * 1080):
        self.free = [v.PinnedHits(max_rec) for _ in range(n)]
        self.all = list(self.free)

    def take(self):
        return self.free.pop() if self.free else None

    def give(self, buf):
        self.free.append(buf)

    def close(self):
        for b in self.all:
            b.close()


def serve_sweep(args, v, datas, worlds, edges, surf, resident, reserve):
    """One scheduling mode over every arrival rate.  Every render of the checked worlds is
    kept (up to --serve-check-cap per rate) and, after each rate, replayed on oracle copies
    of those worlds that apply every edit of the log in submission order."""
    import collections

    from oracle.oracle import OracleWorld
    from voxelrt_gb300 import workloads as W
    srv = v.Server(worlds, max_inflight=3, resident=resident)
    max_rec = 1920 * 1080
    bufs = [v.PinnedHits(max_rec) for _ in range(24)]
    out = []
    checked = check_worlds(edges, args.serve_check_worlds)
    oracles = {}
    for wi in checked:
        o = OracleWorld(datas[wi].sectors)
        o.upload(datas[wi])
        oracles[wi] = o
    replay = {"renders": 0, "bit_exact": True, "worlds": checked, "world_edges": [edges[i] for i in checked],
              "by_rate": [], "renders_1080p": 0, "records": 0}
    for ri, lam in enumerate(float(x) for x in args.serve_rates.split(",")):
        seconds = max(args.serve_seconds, args.serve_min_requests / lam)
        sched = W.serving_schedule(lam, seconds, len(worlds), edges, seed=100 + ri)
        srv.stats(reset=True)
        free = list(range(len(bufs)))
        inflight = collections.deque()
        infos, log = [], []
        kept = 0
        # keep every `stride`-th render of the checked worlds, so the kept ones span the run
        expect = sum(1 for e in sched if e[1] == "render" and e[2] in oracles)
        stride = max(1, expect // max(1, args.serve_check_cap))
        seen = 0

        def retire():
            t, b, res, sample = inflight.popleft()
            info = srv.wait(t, timeout_ms=60000)
            info["res"] = res
            infos.append(info)
            if sample is None:
                free.append(b)

        t0 = time.perf_counter()
        for (t, kind, wi, payload) in sched:
            while True:
                now = time.perf_counter() - t0
                if now >= t:
                    break
                time.sleep(min(t - now, 2e-4))
            if kind == "render":
                n = v.view_records(payload)
                sample = None
                keep = wi in oracles and seen % stride == 0 and kept < args.serve_check_cap
                seen += int(wi in oracles)
                if keep:
                    rb = reserve.take()
                    if rb is not None:
                        sample = {"view": payload, "n": n, "buf": rb}
                        kept += 1
                if sample is not None:
                    target = sample["buf"].array[:n]
                    b = None
                else:
                    while not free:
                        retire()
                    b = free.pop()
                    target = bufs[b].array[:n]
                tk = srv.submit_render(payload, target)
                inflight.append((tk, b, (payload.cam.width, payload.cam.height), sample))
                log.append(("render", wi, sample))
            else:
                radius, material, pick = payload
                c = surf[wi][pick % len(surf[wi])]
                e = np.zeros(1, v.EDIT_DTYPE)
                e["center"], e["radius"], e["material"] = c, radius, material
                srv.submit_edit(wi, e)
                log.append(("edit", wi, e))
        while inflight:
            retire()
        srv.drain()
        wall = time.perf_counter() - t0
        st = srv.stats()
        lat = np.array([i["done_us"] - i["submit_us"] for i in infos]) / 1e3
        hd = np.array([i["done_us"] - i["submit_us"] for i in infos if i["res"] == (1920, 1080)]) / 1e3
        rays = sum(i["rays"] for i in infos)
        out.append({"rate_req_s": lam, "renders": len(infos), "edits": st["edits_done"], "launches": st["launches"],
                    "grays_s": rays / wall / 1e9, "p50_ms": float(np.percentile(lat, 50)),
                    "p99_ms": float(np.percentile(lat, 99)), "p999_ms": float(np.percentile(lat, 99.9)),
                    "p99_1080p_ms": float(np.percentile(hd, 99)) if len(hd) else None,
                    "mean_batch": float(np.mean([i["batch_size"] for i in infos])), "busy_s": st["busy_seconds"],
                    "wall_s": wall})
        # replay the log of the checked worlds on the oracle: edits in submission order
        n_ok, n_1080 = 0, 0
        for kind, wi, item in log:
            if wi not in oracles:
                continue
            o = oracles[wi]
            if kind == "edit":
                o.edit(item)
            elif item is not None:
                vw = item["view"]
                want = o.render_view(vw.cam, vw.max_iters)
                got = item["buf"].array[:item["n"]]
                ok = hits_match(got, want)
                replay["bit_exact"] &= ok
                n_ok += int(ok)
                n_1080 += int((vw.cam.width, vw.cam.height) == (1920, 1080))
                replay["records"] += item["n"]
                reserve.give(item["buf"])
        replay["by_rate"].append({"rate_req_s": lam, "renders": kept, "bit_exact": n_ok == kept, "renders_1080p": n_1080})
        replay["renders"] += kept
        replay["renders_1080p"] += n_1080
    srv.close()
    for o in oracles.values():
        o.close()
    for b in bufs:
        b.close()
    return {"rates": out, "oracle_replay": replay, "launches": sum(r["launches"] for r in out),
            "pool_compactions": int(sum(w.stats()["compactions"] for w in worlds))}


def edit_latency(v, worlds, edges, surf):
    """Sphere edits (radius 4..32, carve or fill at surface points) applied one at a time to
    the largest resident world: the host call of vrt_world_edit (the work is queued on the
    device, allocation included) and the time to completion (vrt_world_wait after it); then
    one vrt_world_defrag of the pool the edits fragmented."""
    big = int(np.argmax(edges))
    w = worlds[big]
    rng = np.random.default_rng(77)
    call_ms, done_ms = [], []
    for k in range(200):
        e = np.zeros(1, v.EDIT_DTYPE)
        e["center"] = surf[big][int(rng.integers(0, len(surf[big])))]
        e["radius"] = int(rng.integers(4, 33))
        e["material"] = 0 if k % 2 else int(rng.integers(1, 256))
        t0 = time.perf_counter()
        w.edit(e, wait=False)
        t1 = time.perf_counter()
        v.check(v.lib().vrt_world_wait(w.handle))
        t2 = time.perf_counter()
        call_ms.append((t1 - t0) * 1e3)
        done_ms.append((t2 - t0) * 1e3)
    before = w.stats()
    t0 = time.perf_counter()
    w.defrag()
    defrag_ms = (time.perf_counter() - t0) * 1e3
    after = w.stats()
    return {"edits": len(call_ms), "world_edge": edges[big],
            "p50_ms": float(np.percentile(done_ms, 50)), "p99_ms": float(np.percentile(done_ms, 99)),
            "call_p50_ms": float(np.percentile(call_ms, 50)), "call_p99_ms": float(np.percentile(call_ms, 99)),
            "api": "vrt_world_edit (device allocation, no host sync) + vrt_world_wait; p50/p99 to completion",
            "defrag": {"ms": defrag_ms, "live_bricks": after["allocated_bricks"],
                       "free_ranges_before": before["free_ranges"], "free_ranges_after": after["free_ranges"],
                       "capacity": after["brick_capacity"]}}


def hits_match(got, want) -> bool:
    """Integer fields bit-exact, t within 1e-6 relative (the parity bar)."""
    ok = True
    for f in ("voxel", "face", "material", "steps", "tag"):
        ok &= bool(np.array_equal(got[f], want[f]))
    fin = np.isfinite(want["t"])
    ok &= bool(np.array_equal(np.isfinite(got["t"]), fin))
    ok &= bool(np.allclose(got["t"][fin], want["t"][fin], rtol=1e-6, atol=0))
    return ok


def run_stress(v, world, data, args, stream, n=1 << 26, steps=3):
    """The incoherent workload's stress set: 2^26 rays with origins uniform in the world box and
    directions uniform on the sphere, cast with vrt_cast_device from device memory; 64 Ki
    of them are checked against the CPU oracle."""
    import torch

    from oracle.oracle import OracleWorld
    size = [c * 32 for c in data.sectors]
    rays = v.random_rays(size, seed=9, n=n)
    d_rays = torch.from_numpy(rays.view(np.uint8)).cuda()
    d_hits = torch.empty(n * HIT_BYTES, dtype=torch.uint8, device="cuda")
    with torch.cuda.stream(stream):
        world.cast_device(d_rays, n, d_hits, stream=stream)
        world.cast_device(d_rays, n, d_hits, stream=stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            world.cast_device(d_rays, n, d_hits, stream=stream)
        e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    sub = rays[: 1 << 16]
    got = d_hits[: sub.size * HIT_BYTES].cpu().numpy().view(v.HIT_DTYPE)
    o = OracleWorld(data.sectors)
    o.upload(data)
    ok = hits_match(got, o.cast(sub))
    o.close()
    return {"rays": n, "ms": ms, "value": n / (ms * 1e-3) / 1e9, "unit": "Grays/s",
            "api": "vrt_cast_device, rays and records in device memory", "checked_rays": int(sub.size),
            "bit_exact": ok}


def parity_sample(wl, batch, hits, stream, max_views=48, pick="spread"):
    """Compare whole views of one batch launch with the CPU oracle: `max_views` views spread
    evenly over the batch in its order (every world size, resolution and path kind of the
    workload is drawn), or its largest views (pick="largest")."""
    import voxelrt_gb300 as v
    from oracle.oracle import OracleWorld
    batch.launch(hits, stream)
    stream.synchronize()
    n = len(wl.views)
    if pick == "largest":
        sizes = [vw.cam.width * vw.cam.height for vw in wl.views]
        order = sorted(np.argsort(sizes, kind="stable")[::-1][:max_views].tolist())
    else:
        order = sorted({(k * n) // max_views for k in range(min(max_views, n))})
    rays, ok, bad = 0, True, []
    cache = {}
    for i in order:
        vw = wl.views[i]
        if vw.world not in cache:
            for o in cache.values():
                o.close()
            cache = {vw.world: OracleWorld(wl.worlds[vw.world].sectors)}
            cache[vw.world].upload(wl.worlds[vw.world])
        want = oracle_view(cache[vw.world], vw)
        a, b = int(batch.offsets[i]), int(batch.offsets[i + 1])
        got = hits[a * HIT_BYTES:b * HIT_BYTES].cpu().numpy().view(v.HIT_DTYPE).reshape(want.shape)
        match = hits_match(got, want)
        ok &= match
        if not match:
            bad.append(i)
        rays += want.size
    for o in cache.values():
        o.close()
    return {"views": len(order), "of_views": n, "pick": pick, "records": rays, "bit_exact": ok,
            "mismatched_views": bad[:8]}


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    args = parse(argv)
    ws_env = os.environ.get("WORLD_SIZE")
    if ws_env is None and args.gpus > 1:
        # one process per GPU: run this script again under torchrun
        return subprocess.call(relaunch_cmd(args.gpus, argv, free_port()))
    ws = int(ws_env or 1)
    if ws != args.gpus:
        print(f"bench.py: WORLD_SIZE={ws} disagrees with --gpus {args.gpus}", file=sys.stderr)
        return 2
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)
    return 0


if __name__ == "__main__":
    sys.exit(main())
