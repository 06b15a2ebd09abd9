#!/usr/bin/env python3
"""Generate the golden vectors that pin the CPU oracle to the reference itself.

Runs the reference's own RayCast (src/VoxelRT/CpuRenderer.cpp:172-224) over its own
FlatVoxelStorage filled through VoxelMap + SyncBuffers (CpuRenderer.cpp:20-84),
compiled in place by oracle/ref_pin/build_ref.sh (x86-64 AVX-512 only), on seeded
worlds from libvrt's generators and seeded rays, and stores rays + reference
outputs in tests/golden/refcast.npz.  The worlds are rebuilt from their recipe at
test time (the generators are deterministic across hosts), so only rays and results
are stored.

The reference's FlatVoxelStorage spans a fixed 2048x512x2048 view (64x16x64
sectors, CpuRenderer.cpp:13-16) and has no entry clip, so rays start inside it and
the oracle is run on a world of that extent.

Usage: python tests/golden/make_golden.py <reference checkout> (or $VRT_REFERENCE_DIR)
"""
from __future__ import annotations

import ctypes as C
import subprocess
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import voxelrt_gb300 as v  # noqa: E402

OUT = Path(__file__).resolve().parent / "refcast.npz"
OUT_PICK = Path(__file__).resolve().parent / "refpick.npz"

# world recipes: (name, kind, params)
WORLDS = {
    "terrain256": ("terrain", dict(size=(256, 256, 256), base=96, amplitude=48, seed=1)),
    "mix128": ("mix", dict(edge=128, seed=7)),
    "mix64": ("mix", dict(edge=64, seed=3)),
}


def build_world(name: str) -> v.SectorData:
    kind, p = WORLDS[name]
    if kind == "terrain":
        return v.synth_terrain(**p)
    return v.synth_mix(p["edge"], p["seed"])


def cases():
    """(case name, world name, origins, dirs, world origin)."""
    out = []
    rng = np.random.default_rng(20240601)
    for world, edge, n in (("terrain256", 256, 6000), ("mix128", 128, 4000), ("mix64", 64, 3000)):
        rays = v.random_rays((edge, edge, edge), seed=int(rng.integers(1 << 30)), n=n)
        org = np.clip(rays["origin"], 1.0, edge - 1.0).astype(np.float32)
        d = rays["dir"].copy()
        # some exact-zero and negative-zero components (NaN side distances)
        z = rng.random(d.shape) < 0.06
        d[z] = np.where(rng.random(z.sum()) < 0.5, 0.0, -0.0).astype(np.float32)
        d[(d == 0).all(1)] = np.float32([0.0, -1.0, 0.0])
        # some origins on voxel boundaries
        k = rng.random(n) < 0.1
        org[k] = np.floor(org[k])
        out.append((f"{world}_random", world, org, d, (0, 0, 0)))
    # camera rays inside the terrain world, in the camera frame (world origin = floor(pos))
    cam = v.look_at((128.3, 200.7, 20.2), (128.0, 80.0, 128.0), 90.0, 96, 54)
    from oracle.oracle import camera_rays
    rays = camera_rays(cam)
    out.append(("terrain256_camera", "terrain256", rays["origin"].copy(), rays["dir"].copy(),
                tuple(int(c) for c in cam.world_origin)))
    return out


def main(ref: str) -> None:
    subprocess.run([str(ROOT / "oracle" / "ref_pin" / "build_ref.sh"), ref], check=True)
    L = C.CDLL(str(ROOT / "oracle" / "_ref" / "libvrt_ref.so"))
    L.ref_world_create.restype = C.c_void_p
    L.ref_world_destroy.argtypes = [C.c_void_p]
    L.ref_world_load.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
    L.ref_raycast.argtypes = [C.c_void_p, C.c_uint64] + [C.c_void_p] * 8
    view = (C.c_uint32 * 3)()
    L.ref_view_sectors(view)
    arrays = {"view_sectors": np.array(view[:], np.int32), "lanes": np.array([L.ref_lanes()], np.int32)}
    names = []
    worlds = {}
    for case, world, org, d, wo in cases():
        if world not in worlds:
            data = build_world(world)
            h = L.ref_world_create()
            L.ref_world_load(h, len(data.sector_idx), data.sector_idx.ctypes.data, data.alloc_mask.ctypes.data,
                             data.bricks.ctypes.data)
            worlds[world] = h
        h = worlds[world]
        n = len(org)
        org = np.ascontiguousarray(org, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        hit = np.zeros(n, np.uint8)
        pos = np.zeros((n, 3), np.float32)
        nrm = np.zeros((n, 3), np.float32)
        dist = np.zeros(n, np.float32)
        mat = np.zeros(n, np.int32)
        wo_c = (C.c_int32 * 3)(*wo)
        L.ref_raycast(h, n, org.ctypes.data, d.ctypes.data, wo_c, hit.ctypes.data, pos.ctypes.data,
                      nrm.ctypes.data, dist.ctypes.data, mat.ctypes.data)
        names.append(case)
        arrays[f"{case}/world"] = np.array(world)
        arrays[f"{case}/world_origin"] = np.array(wo, np.int32)
        arrays[f"{case}/origin"] = org
        arrays[f"{case}/dir"] = d
        arrays[f"{case}/hit"] = hit
        arrays[f"{case}/pos"] = pos
        arrays[f"{case}/normal"] = nrm.astype(np.int8)
        arrays[f"{case}/dist"] = dist
        arrays[f"{case}/material"] = (mat & 0xFFFF).astype(np.uint16)
        print(f"{case}: {n} rays, {int(hit.sum())} hits")
    arrays["cases"] = np.array(names)
    np.savez_compressed(OUT, **arrays)
    print(OUT, OUT.stat().st_size, "bytes")

    # picking: VoxelMap::RayCast (VoxelMap.cpp:140-170) over the same maps, double precision
    L.ref_pick.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint32] + [C.c_void_p] * 4
    pick = {}
    rng = np.random.default_rng(77)
    for world, edge in (("terrain256", 256), ("mix128", 128), ("mix64", 64)):
        n = 1500
        o = rng.uniform(-0.25 * edge, 1.25 * edge, (n, 3))
        tgt = rng.uniform(0, edge, (n, 3))
        d = tgt - o
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        d[: n // 10, rng.integers(0, 3)] = 0.0  # some zero components
        rays = np.ascontiguousarray(np.concatenate([o, d], 1), np.float64)
        dist = np.zeros(n, np.float64)
        nrm = np.zeros((n, 3), np.float32)
        uv = np.zeros((n, 2), np.float32)
        vox = np.zeros((n, 3), np.int32)
        L.ref_pick(worlds[world], n, rays.ctypes.data, 1024, dist.ctypes.data, nrm.ctypes.data, uv.ctypes.data,
                   vox.ctypes.data)
        pick[f"{world}/rays"] = rays
        pick[f"{world}/distance"] = dist
        pick[f"{world}/normal"] = nrm
        pick[f"{world}/uv"] = uv
        pick[f"{world}/voxel"] = vox
        print(f"pick {world}: {n} rays, {int((dist > 0).sum())} hits")
    pick["worlds"] = np.array(["terrain256", "mix128", "mix64"])
    pick["view_sectors"] = arrays["view_sectors"]
    np.savez_compressed(OUT_PICK, **pick)
    print(OUT_PICK, OUT_PICK.stat().st_size, "bytes")
    for h in worlds.values():
        L.ref_world_destroy(h)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VRT_REFERENCE_DIR")
    if not ref:
        sys.exit("usage: give the reference checkout as the argument or in $VRT_REFERENCE_DIR")
    main(ref)
