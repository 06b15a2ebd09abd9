#!/usr/bin/env python3
"""Generate the golden world state that pins the oracle's sphere edits to the reference's
own region dispatch and brick GC.

Loads a seeded world into the reference's VoxelMap and applies seeded sphere edits through
VoxelMap::RegionDispatchSIMD + its empty-brick GC (src/VoxelRT/VoxelMap.h:222-263), called as
BrushSession::Dispatch calls it (Brush.cpp:10-31) with the library's exact integer sphere in
place of the brush's capsule SDF (ref_world_edit_spheres in oracle/ref_pin/ref_driver.cpp,
compiled in place by oracle/ref_pin/build_ref.sh).  Stores the edits and every resulting
sector (index, allocation mask, bricks) in tests/golden/refedit.npz.  The world is rebuilt
from its recipe at test time.

Usage: python tests/golden/make_golden_edit.py <reference checkout> (or $VRT_REFERENCE_DIR)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import voxelrt_gb300 as v  # noqa: E402

OUT = Path(__file__).resolve().parent / "refedit.npz"
REF_LIB = ROOT / "oracle" / "_ref" / "libvrt_ref.so"
EDGE, SEED = 128, 41  # world recipe: world()
GOLDEN_WORLD_EDGE = EDGE
N_EDITS = 240


def world() -> v.SectorData:
    """A 128^3 heightfield: solid below about y = 48, empty bricks and sectors above it, so fills
    create bricks and sectors and carves free them."""
    return v.synth_terrain(size=(EDGE, EDGE, EDGE), base=48, amplitude=24, seed=SEED)


def brick_positions(sector_idx, masks) -> np.ndarray:
    """(x, y, z) brick positions of the allocated bricks, sector by sector in mask-bit order
    (WorldSectorIndexer packing: x in bits 0-11, z in 12-23, y in 24-31, non-negative here)."""
    out = []
    for idx, m in zip(sector_idx, masks):
        sx, sz, sy = int(idx) & 4095, (int(idx) >> 12) & 4095, (int(idx) >> 24) & 255
        for b in range(64):
            if (int(m) >> b) & 1:
                out.append((sx * 4 + (b & 3), sy * 4 + (b >> 4), sz * 4 + ((b >> 2) & 3)))
    return np.array(out, np.int32).reshape(-1, 3)


def edits(rng) -> np.ndarray:
    """Sphere edits inside the world: fills, carves (material 0) and replaces."""
    e = np.zeros(N_EDITS, v.EDIT_DTYPE)
    for i in range(N_EDITS):
        r = int(rng.integers(1, 21))
        e[i]["center"] = rng.integers(r, EDGE - r, 3)
        e[i]["radius"] = r
        kind = rng.random()
        e[i]["material"] = 0 if kind < 0.35 else int(rng.integers(1, 256))
        e[i]["mode"] = v.capi.EDIT_REPLACE if kind > 0.8 else 0
    return e


def main(argv):
    ref = argv[1] if len(argv) > 1 else os.environ.get("VRT_REFERENCE_DIR")
    if not ref:
        sys.exit("usage: make_golden_edit.py <reference checkout> (or set VRT_REFERENCE_DIR)")
    subprocess.run(["sh", str(ROOT / "oracle" / "ref_pin" / "build_ref.sh"), ref], check=True)
    L = C.CDLL(str(REF_LIB))
    L.ref_world_create.restype = C.c_void_p
    L.ref_world_destroy.argtypes = [C.c_void_p]
    L.ref_world_load.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
    L.ref_world_edit_spheres.argtypes = [C.c_void_p, C.c_uint32] + [C.c_void_p] * 4
    L.ref_world_sector_count.restype = C.c_uint32
    L.ref_world_sector_count.argtypes = [C.c_void_p, C.c_void_p]
    L.ref_world_export.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.ref_world_occupancy.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
    d = world()
    e = edits(np.random.default_rng(20261205))
    w = L.ref_world_create()
    L.ref_world_load(w, len(d.sector_idx), d.sector_idx.ctypes.data, d.alloc_mask.ctypes.data, d.bricks.ctypes.data)
    centers = np.ascontiguousarray(e["center"], np.int32)
    radii = np.ascontiguousarray(e["radius"], np.uint32)
    mats = np.ascontiguousarray(e["material"], np.uint8)
    modes = np.ascontiguousarray(e["mode"], np.uint8)
    L.ref_world_edit_spheres(w, len(e), centers.ctypes.data, radii.ctypes.data, mats.ctypes.data, modes.ctypes.data)
    nb = C.c_uint64(0)
    ns = L.ref_world_sector_count(w, C.byref(nb))
    idx = np.zeros(ns, np.int32)
    masks = np.zeros(ns, np.uint64)
    bricks = np.zeros((nb.value, 512), np.uint8)
    L.ref_world_export(w, idx.ctypes.data, masks.ctypes.data, bricks.ctypes.data)
    pos = brick_positions(idx, masks)
    occ = np.zeros((len(pos), 8), np.uint64)
    L.ref_world_occupancy(w, len(pos), np.ascontiguousarray(pos, np.int32).ctypes.data, occ.ctypes.data)
    L.ref_world_destroy(w)
    np.savez_compressed(OUT, edge=np.array([EDGE, SEED], np.int32), edits=e, sector_idx=idx, alloc_mask=masks,
                        bricks=bricks, occupancy=occ)
    print(f"{len(e)} edits -> {ns} sectors, {nb.value} bricks (before: {len(d.sector_idx)} sectors, "
          f"{d.n_bricks} bricks): {OUT}")


if __name__ == "__main__":
    main(sys.argv)
