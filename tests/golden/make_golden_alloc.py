#!/usr/bin/env python3
"""Generate the golden slot placements that pin the host free list to the reference's own
brick-slot allocator.

Runs the reference's BrickSlotAllocator / FreeList (src/VoxelRT/BrickSlotAllocator.cpp:5-94),
compiled in place by oracle/ref_pin/build_ref.sh, over seeded runs of sector edits: each
op adds a random set of bricks to one sector and then drops another set.  After every op
the sector's base slot and allocation mask are stored, and at the end the free ranges, in
tests/golden/refalloc.npz.  The reference throws when no free range fits a growing sector
(after freeing its old range), so a run stops before such an op; the stored op count says
where.

Usage: python tests/golden/make_golden_alloc.py <reference checkout> (or $VRT_REFERENCE_DIR)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
OUT = Path(__file__).resolve().parent / "refalloc.npz"
REF_LIB = ROOT / "oracle" / "_ref" / "libvrt_ref.so"

# (name, bounds_xz, bounds_y, ops, bricks added per op at most, chance of a removal)
RUNS = [
    ("small", 2, 2, 600, 24, 0.5),      # 512 slots, 8 sectors: fills up, fragments
    ("medium", 4, 2, 2500, 40, 0.45),   # 2048 slots, 32 sectors
    ("large", 4, 4, 4000, 64, 0.4),     # 4096 slots, 64 sectors, whole-sector adds
]


def random_masks(rng, n, max_bits):
    """n 64-bit masks with 0..max_bits random bricks each."""
    out = np.zeros(n, np.uint64)
    for i in range(n):
        k = int(rng.integers(0, max_bits + 1))
        bits = rng.choice(64, size=k, replace=False)
        out[i] = np.bitwise_or.reduce((np.uint64(1) << bits.astype(np.uint64)), initial=np.uint64(0))
    return out


def main(argv):
    ref = argv[1] if len(argv) > 1 else os.environ.get("VRT_REFERENCE_DIR")
    if not ref:
        sys.exit("usage: make_golden_alloc.py <reference checkout> (or set VRT_REFERENCE_DIR)")
    subprocess.run(["sh", str(ROOT / "oracle" / "ref_pin" / "build_ref.sh"), ref], check=True)
    lib = C.CDLL(str(REF_LIB))
    fn = lib.ref_alloc_run
    fn.restype = C.c_uint32
    fn.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32] + [C.c_void_p] * 6 + [C.c_uint32, C.c_void_p]
    rng = np.random.default_rng(20261204)
    data = {}
    for name, bxz, by, n, max_bits, p_remove in RUNS:
        n_sectors = bxz * bxz * by
        sector = rng.integers(0, n_sectors, n).astype(np.uint32)
        add = random_masks(rng, n, max_bits)
        remove = np.where(rng.random(n) < p_remove, random_masks(rng, n, 64), np.uint64(0)).astype(np.uint64)
        base = np.zeros(n, np.uint32)
        mask = np.zeros(n, np.uint64)
        ranges = np.zeros(2 * 4096, np.uint32)
        nr = C.c_uint32(0)
        ran = fn(bxz, by, n, sector.ctypes.data, add.ctypes.data, remove.ctypes.data, base.ctypes.data,
                 mask.ctypes.data, ranges.ctypes.data, 4096, C.byref(nr))
        print(f"{name}: {ran} of {n} ops, {nr.value} free ranges at the end")
        data[f"{name}_bounds"] = np.array([bxz, by], np.uint32)
        data[f"{name}_sector"] = sector[:ran]
        data[f"{name}_add"] = add[:ran]
        data[f"{name}_remove"] = remove[:ran]
        data[f"{name}_base"] = base[:ran]
        data[f"{name}_mask"] = mask[:ran]
        data[f"{name}_ranges"] = ranges[: 2 * nr.value].reshape(-1, 2)
    np.savez_compressed(OUT, **data)
    print(OUT)


if __name__ == "__main__":
    main(sys.argv)
