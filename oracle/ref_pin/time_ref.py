#!/usr/bin/env python3
"""Times the reference's own AVX-512 RayCast (src/VoxelRT/CpuRenderer.cpp:172-224, built
in place by oracle/ref_pin/build_ref.sh) on the camera rays of the uneven batch, beside
the scalar oracle on the same rays, on this host's cores.  TEST INFRASTRUCTURE: a CPU
baseline recipe, x86-64 with AVX-512 only (the reference's SIMD layer runs nowhere else).

Views are taken in batch order (seed 2, the benchmark's batch) until --seconds of
reference work; each view's world is loaded into the reference's VoxelMap and
FlatVoxelStorage (SyncBuffers), its camera rays (the vrt_camera contract) are split into
one slice per thread, and RenderFrame's row parallelism (CpuRenderer.cpp:455-462) is
stood in for by that many threads each calling RayCast over its slice in 16-ray groups.
The reference has no entry clip and bounds its grid by its fixed 2048x512x2048 view
(CpuRenderer.cpp:13-16), so rays leaving a smaller world walk on through empty sectors:
its work per ray is at least the oracle's.

Usage: python oracle/ref_pin/time_ref.py [--seconds 20] [--threads N] [--reference DIR]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import platform
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))


def load_ref():
    L = C.CDLL(str(ROOT / "oracle" / "_ref" / "libvrt_ref.so"))
    L.ref_world_create.restype = C.c_void_p
    L.ref_world_destroy.argtypes = [C.c_void_p]
    L.ref_world_load.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
    L.ref_raycast.argtypes = [C.c_void_p, C.c_uint64] + [C.c_void_p] * 8
    L.ref_lanes.restype = C.c_uint32
    return L


def ref_cast(L, h, org, d, wo, threads):
    """RayCast over the rays in `threads` slices at once; returns seconds."""
    n = len(org)
    hit = np.zeros(n, np.uint8)
    pos = np.zeros((n, 3), np.float32)
    nrm = np.zeros((n, 3), np.float32)
    dist = np.zeros(n, np.float32)
    mat = np.zeros(n, np.int32)
    wo_c = (C.c_int32 * 3)(*wo)
    cuts = np.linspace(0, n, threads + 1).astype(np.int64)

    def run(a, b):
        L.ref_raycast(h, int(b - a), org[a:].ctypes.data, d[a:].ctypes.data, wo_c, hit[a:].ctypes.data,
                      pos[a:].ctypes.data, nrm[a:].ctypes.data, dist[a:].ctypes.data, mat[a:].ctypes.data)

    ths = [threading.Thread(target=run, args=(int(cuts[k]), int(cuts[k + 1]))) for k in range(threads)]
    t0 = time.perf_counter()
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    return time.perf_counter() - t0


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--seconds", type=float, default=20.0)
    ap.add_argument("--threads", type=int, default=len(os.sched_getaffinity(0)))
    ap.add_argument("--reference", default=os.environ.get("VRT_REFERENCE_DIR"))
    a = ap.parse_args()
    if a.reference:
        subprocess.run(["sh", str(ROOT / "oracle" / "ref_pin" / "build_ref.sh"), a.reference], check=True,
                       stdout=subprocess.DEVNULL)
    from oracle.oracle import OracleWorld, camera_rays
    from voxelrt_gb300 import workloads as W
    L = load_ref()
    wl = W.uneven_batch(n_worlds=128, max_views=16, seed=2)
    ref_s, ora_s, rays, views = 0.0, 0.0, 0, 0
    cur, h, o = None, None, None
    for vw in wl.views:
        if ref_s >= a.seconds:
            break
        if vw.world != cur:
            if h:
                L.ref_world_destroy(h)
                o.close()
            d = wl.worlds[vw.world]
            h = L.ref_world_create()
            L.ref_world_load(h, len(d.sector_idx), d.sector_idx.ctypes.data, d.alloc_mask.ctypes.data,
                             d.bricks.ctypes.data)
            o = OracleWorld(d.sectors)
            o.upload(d)
            cur = vw.world
        r = camera_rays(vw.cam)
        org = np.ascontiguousarray(r["origin"], np.float32)
        dr = np.ascontiguousarray(r["dir"], np.float32)
        wo = tuple(int(c) for c in vw.cam.world_origin)
        ref_s += ref_cast(L, h, org, dr, wo, a.threads)
        t0 = time.perf_counter()
        o.cast(r, world_origin=wo, threads=a.threads)
        ora_s += time.perf_counter() - t0
        rays += len(r)
        views += 1
    if h:
        L.ref_world_destroy(h)
        o.close()
    cpu = platform.processor() or platform.machine()
    try:
        for ln in Path("/proc/cpuinfo").read_text().splitlines():
            if ln.startswith("model name"):
                cpu = ln.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    print(json.dumps({
        "sample": f"first {views} views of the uneven batch in batch order, {rays} primary rays",
        "threads": a.threads, "cpu": cpu, "lanes": int(L.ref_lanes()),
        "reference_avx512": {"seconds": ref_s, "grays_s": rays / ref_s / 1e9},
        "oracle_port": {"seconds": ora_s, "grays_s": rays / ora_s / 1e9},
    }))


if __name__ == "__main__":
    main()
