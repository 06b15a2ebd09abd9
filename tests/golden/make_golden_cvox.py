#!/usr/bin/env python3
"""Generate the world-file fixtures that pin the cvox v4 reader and writer to the
reference's own serializer.

The reference's VoxelMap::Serialize / Deserialize (src/VoxelRT/VoxelMap.cpp:211-273)
with its zstd framing (src/LibGlimpsw/Common/BinaryIO.cpp:8-64) are compiled in place
by oracle/ref_pin/build_ref.sh against the system's libzstd (x86-64 only).  On a
seeded world from libvrt's generators this script

  * loads the world into the reference's VoxelMap and has Serialize write
    tests/golden/refworld.cvox - a file with zstd-compressed packs and checksums,
    exactly as the reference writes them;
  * writes the same world with vrt_cvox_write, has the reference's Deserialize read
    that file, and stores what it read (sector indices, masks, bricks) and the SHA-256
    of the file in tests/golden/refcvox.npz.

The world is rebuilt from its recipe at test time (the generators are deterministic
across hosts), so tests compare what each side read with it.

Usage: python tests/golden/make_golden_cvox.py <reference checkout> (or $VRT_REFERENCE_DIR)
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import voxelrt_gb300 as v  # noqa: E402

HERE = Path(__file__).resolve().parent
OUT_FILE = HERE / "refworld.cvox"
OUT_NPZ = HERE / "refcvox.npz"

# the seeded world of the fixtures: mixed world of edge 96, seed 61
WORLD = dict(edge=96, seed=61)


def build_world() -> v.SectorData:
    return v.synth_mix(WORLD["edge"], WORLD["seed"])


def main(ref: str) -> None:
    subprocess.run(["sh", str(ROOT / "oracle" / "ref_pin" / "build_ref.sh"), ref], check=True)
    L = C.CDLL(str(ROOT / "oracle" / "_ref" / "libvrt_ref.so"))
    L.ref_world_create.restype = C.c_void_p
    L.ref_world_destroy.argtypes = [C.c_void_p]
    L.ref_world_load.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]
    L.ref_serialize.argtypes = [C.c_void_p, C.c_char_p]
    L.ref_world_from_file.restype = C.c_void_p
    L.ref_world_from_file.argtypes = [C.c_char_p]
    L.ref_world_sector_count.restype = C.c_uint32
    L.ref_world_sector_count.argtypes = [C.c_void_p, C.POINTER(C.c_uint64)]
    L.ref_world_export.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]

    data = build_world()
    # 1. the reference writes the world
    w = L.ref_world_create()
    L.ref_world_load(w, len(data.sector_idx), data.sector_idx.ctypes.data, data.alloc_mask.ctypes.data,
                     data.bricks.ctypes.data)
    if L.ref_serialize(w, str(OUT_FILE).encode()) != 0:
        sys.exit("the reference's Serialize failed (libzstd missing?)")
    L.ref_world_destroy(w)
    print(OUT_FILE, OUT_FILE.stat().st_size, "bytes")

    # 2. the reference reads a file this library wrote
    with tempfile.TemporaryDirectory() as td:
        ours = Path(td) / "ours.cvox"
        v.cvox_write(ours, data)
        sha = hashlib.sha256(ours.read_bytes()).hexdigest()
        r = L.ref_world_from_file(str(ours).encode())
        if not r:
            sys.exit("the reference's Deserialize refused this library's file")
    nb = C.c_uint64()
    n = L.ref_world_sector_count(r, C.byref(nb))
    idx = np.zeros(n, np.int32)
    masks = np.zeros(n, np.uint64)
    bricks = np.zeros((nb.value, 512), np.uint8)
    L.ref_world_export(r, idx.ctypes.data, masks.ctypes.data, bricks.ctypes.data)
    L.ref_world_destroy(r)
    np.savez_compressed(OUT_NPZ, sector_idx=idx, alloc_mask=masks, bricks=bricks, ours_sha256=np.array(sha),
                        world=np.array([WORLD["edge"], WORLD["seed"]]))
    print(OUT_NPZ, OUT_NPZ.stat().st_size, "bytes;", n, "sectors,", nb.value, "bricks read by the reference")


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VRT_REFERENCE_DIR")
    if not ref:
        sys.exit("usage: give the reference checkout as the argument or in $VRT_REFERENCE_DIR")
    main(ref)
