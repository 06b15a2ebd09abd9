"""The oracle's sphere edits pinned to the reference's own region dispatch and brick GC (no GPU).

tests/golden/refedit.npz holds 240 seeded sphere edits (fills, carves, replaces) and the world
they leave in the reference's VoxelMap: RegionDispatchSIMD + empty-brick GC
(src/VoxelRT/VoxelMap.h:222-263), called as the brush calls it (Brush.cpp:10-31) with the
library's exact integer sphere, compiled in place by tests/golden/make_golden_edit.py.  The
oracle applies the same edits to the same world; every sector's allocation mask and every
brick must be the reference's.  The GPU tests compare the device's edits with the oracle
(tests/test_edit_gpu.py), which closes the chain to the reference.
"""
from pathlib import Path

import numpy as np

from oracle.oracle import OracleWorld
from tests.golden.make_golden_edit import GOLDEN_WORLD_EDGE, world

GOLDEN = Path(__file__).resolve().parent / "golden" / "refedit.npz"


def sector_index(x: int, y: int, z: int) -> int:
    """WorldSectorIndexer packing (VoxelMap.h:60-102) for non-negative coordinates."""
    return x | z << 12 | y << 24


def test_oracle_edits_match_the_reference():
    g = np.load(GOLDEN)
    assert int(g["edge"][0]) == GOLDEN_WORLD_EDGE
    d = world()
    o = OracleWorld(d.sectors)
    o.upload(d)
    o.edit(g["edits"])
    want = {}
    off = 0
    for idx, mask in zip(g["sector_idx"], g["alloc_mask"]):
        n = bin(int(mask)).count("1")
        want[int(idx)] = (int(mask), g["bricks"][off:off + n])
        off += n
    assert off == len(g["bricks"])
    sx, sy, sz = d.sectors
    seen = 0
    for y in range(sy):
        for z in range(sz):
            for x in range(sx):
                idx = sector_index(x, y, z)
                mask, bricks = o.read_sector(idx)
                wmask, wbricks = want.get(idx, (0, np.zeros((0, 512), np.uint8)))
                assert mask == wmask, (x, y, z)
                assert np.array_equal(bricks, wbricks), (x, y, z)
                seen += idx in want
    assert seen == len(want)  # every sector the reference holds lies in the world
    o.close()


def test_the_edits_create_and_free_bricks():
    """The seeded world is a heightfield with empty sectors above it, so the edits both create
    bricks and sectors (fills in the air) and free them (carves)."""
    g = np.load(GOLDEN)
    d = world()
    before = {int(i): int(m) for i, m in zip(d.sector_idx, d.alloc_mask)}
    after = {int(i): int(m) for i, m in zip(g["sector_idx"], g["alloc_mask"])}
    assert set(after) - set(before), "no sector was created"
    created = sum(bin(after.get(i, 0) & ~before.get(i, 0)).count("1") for i in set(before) | set(after))
    freed = sum(bin(before.get(i, 0) & ~after.get(i, 0)).count("1") for i in set(before) | set(after))
    assert created > 100 and freed > 20, (created, freed)
    modes = g["edits"]["mode"]
    mats = g["edits"]["material"]
    assert (mats == 0).sum() > 40 and (modes == 1).sum() > 20 and ((mats != 0) & (modes == 0)).sum() > 80


def test_cell_masks_match_the_reference():
    """The 4^3-cell occupancy masks of every brick of the edited world equal those the
    reference's FlatVoxelStorage::UpdateOccupancy (CpuRenderer.cpp:63-83) derived for it."""
    from tests.golden.make_golden_edit import brick_positions
    g = np.load(GOLDEN)
    d = world()
    o = OracleWorld(d.sectors)
    o.upload(d)
    o.edit(g["edits"])
    pos = brick_positions(g["sector_idx"], g["alloc_mask"])
    want = g["occupancy"]
    assert len(pos) == len(want) == len(g["bricks"])
    got = np.stack([o.brick_occupancy(int(x), int(y), int(z)) for x, y, z in pos])
    assert np.array_equal(got, want)
    full = np.uint64(0xFFFFFFFFFFFFFFFF)
    assert (want == 0).any() and (want == full).any() and ((want != 0) & (want != full)).mean() > 0.1
    o.close()
