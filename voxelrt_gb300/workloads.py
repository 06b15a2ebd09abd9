"""Seeded synthetic workloads for the five benchmark configurations.

No public dataset exists for this path; every world and camera is drawn from the
seeded generators of libvrt (include/vrt_synth.h) so that runs on any host build the
same voxels and rays.

* single_view   - 256^3 heightfield (base 96, amplitude 48, seed 1), one 640x360 view
* large_world   - 2048x256x2048 heightfield (base 128, amplitude 96, seed 2) minus caves
                  (3-octave 3D fbm at scale 64 > 0.35, seed 3); 64 cameras at 1920x1080
                  placed 20-60 voxels above the terrain, primary + shadow rays
* uneven_batch  - 128 worlds of edge log-uniform in [64, 512] (multiples of 32) mixing
                  terrain, spheres and random voxels; 1-16 views each at
                  {64^2, 256^2, 640x360, 1280x720}
* incoherent    - 1024^3 terrain (base 128, amplitude 96) + caves (seed 4), a 1280x720 view from (512,300,0)
                  toward (512,100,512) with 4 diffuse bounces; plus 2^26 random rays
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import look_at, make_view, synth_mix, synth_terrain, terrain_height

SUN_DIR = tuple(float(c) for c in np.array([0.3, 0.8, 0.5]) / math.sqrt(0.3 ** 2 + 0.8 ** 2 + 0.5 ** 2))


@dataclass
class Workload:
    name: str
    worlds: list = field(default_factory=list)   # SectorData per world
    views: list = field(default_factory=list)    # vrt_view structs
    description: str = ""

    @property
    def primary_rays(self) -> int:
        return sum(vw.cam.width * vw.cam.height for vw in self.views)


def single_view(width=640, height=360) -> Workload:
    d = synth_terrain((256, 256, 256), base=96, amplitude=48, seed=1)
    cam = look_at((128, 200, -40), (128, 80, 128), 90.0, width, height)
    return Workload("single_view", [d], [make_view(cam)],
                    f"256^3 heightfield seed 1, one {width}x{height} primary view")


LARGE_TERRAIN = dict(size=(2048, 256, 2048), base=128, amplitude=96, seed=2, cave_octaves=3, cave_scale=64.0,
                     cave_threshold=0.35, cave_seed=3)


def large_world(n_cameras=64, width=1920, height=1080, threads=0) -> Workload:
    d = synth_terrain(**LARGE_TERRAIN, threads=threads)
    rng = np.random.default_rng(1)
    views = []
    for _ in range(n_cameras):
        x, z = rng.uniform(64, 2048 - 64, 2)
        h = terrain_height(x, z, LARGE_TERRAIN["size"], LARGE_TERRAIN["base"], LARGE_TERRAIN["amplitude"],
                           LARGE_TERRAIN["seed"])
        y = min(h + rng.uniform(20, 60), 250.0)
        yaw = rng.uniform(0, 2 * math.pi)
        pitch = math.radians(rng.uniform(-30, 10))
        d_ = (math.cos(pitch) * math.cos(yaw), math.sin(pitch), math.cos(pitch) * math.sin(yaw))
        cam = look_at((x, y, z), (x + d_[0], y + d_[1], z + d_[2]), 90.0, width, height)
        views.append(make_view(cam, world=0, shadow_dir=SUN_DIR))
    return Workload("large_world", [d], views,
                    f"2048x256x2048 terrain+caves, {n_cameras} cameras {width}x{height}, primary + shadow")


BATCH_RESOLUTIONS = [(64, 64), (256, 256), (640, 360), (1280, 720)]


def uneven_batch(n_worlds=128, max_views=16, seed=2, threads=0) -> Workload:
    rng = np.random.default_rng(seed)
    worlds, views = [], []
    for i in range(n_worlds):
        edge = int(round(math.exp(rng.uniform(math.log(64), math.log(512))) / 32.0)) * 32
        edge = min(512, max(64, edge))
        worlds.append(synth_mix(edge, seed=seed * 100003 + i, threads=threads))
        for _ in range(int(rng.integers(1, max_views + 1))):
            w, h = BATCH_RESOLUTIONS[int(rng.integers(0, len(BATCH_RESOLUTIONS)))]
            pos = rng.uniform(0, edge, 3)
            tgt = rng.uniform(0, edge, 3)
            if np.linalg.norm(tgt - pos) < 1.0:
                tgt = pos + np.array([1.0, 0.0, 0.0])
            cam = look_at(pos, tgt, float(rng.uniform(60, 90)), w, h)
            views.append(make_view(cam, world=i))
    return Workload("uneven_batch", worlds, views,
                    f"{n_worlds} mixed worlds (edge 64..512), {len(views)} views at 64^2..1280x720")


INCOHERENT_TERRAIN = dict(size=(1024, 1024, 1024), base=128, amplitude=96, seed=4, cave_octaves=3, cave_scale=64.0,
                          cave_threshold=0.35, cave_seed=5)


def incoherent(n_bounces=4, threads=0) -> Workload:
    d = synth_terrain(**INCOHERENT_TERRAIN, threads=threads)
    cam = look_at((512, 300, 0), (512, 100, 512), 90.0, 1280, 720)
    return Workload("incoherent", [d], [make_view(cam, world=0, n_bounces=n_bounces)],
                    f"1024^3 terrain+caves seed 4, 1280x720 primary + {n_bounces} diffuse bounces")


SERVING_RESOLUTIONS = [(256, 256), (1280, 720), (1920, 1080)]
SERVING_RES_P = [0.5, 0.3, 0.2]


def serving_worlds(n_worlds=32, max_edge=1024, seed=4, threads=0) -> list:
    """Resident worlds of the serving workload: mixed worlds, edge log-uniform in [64, max_edge]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_worlds):
        edge = int(round(math.exp(rng.uniform(math.log(64), math.log(max_edge))) / 32.0)) * 32
        out.append(synth_mix(min(max_edge, max(64, edge)), seed=seed * 100019 + i, threads=threads))
    return out


def serving_schedule(rate: float, seconds: float, n_worlds: int, edges, seed: int = 0, edit_rate: float = 100.0):
    """Poisson arrivals of render requests (rate per second) and sphere edits (edit_rate per
    second): list of (time, kind, world, payload) sorted by time.  Render payload is a
    vrt_view; edit payload is (radius, material) for a surface point chosen at run time."""
    rng = np.random.default_rng(seed)
    events = []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            break
        wi = int(rng.integers(0, n_worlds))
        edge = edges[wi]
        w, h = SERVING_RESOLUTIONS[int(rng.choice(3, p=SERVING_RES_P))]
        pos = rng.uniform(0, edge, 3)
        tgt = rng.uniform(0, edge, 3)
        if np.linalg.norm(tgt - pos) < 1.0:
            tgt = pos + np.array([1.0, 0.0, 0.0])
        cam = look_at(pos, tgt, float(rng.uniform(60, 90)), w, h)
        events.append((t, "render", wi, make_view(cam, world=wi)))
    t = 0.0
    while edit_rate > 0:
        t += rng.exponential(1.0 / edit_rate)
        if t >= seconds:
            break
        wi = int(rng.integers(0, n_worlds))
        events.append((t, "edit", wi, (int(rng.integers(4, 33)), 0 if rng.random() < 0.5 else int(rng.integers(1, 256)),
                                       int(rng.integers(0, 1 << 30)))))
    events.sort(key=lambda e: e[0])
    return events
