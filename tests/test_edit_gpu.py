"""Edit and sync paths on the device vs the oracle.

After every batch of edits or dirty-brick syncs, every sector's allocation mask and
brick bytes must equal the oracle's, the allocator must hold exactly the non-empty
bricks, and a re-trace (which reads the re-derived cell masks) must be bit-exact.
"""
import numpy as np
import pytest

import voxelrt_gb300 as v
from oracle.oracle import OracleWorld
from tests.helpers import assert_hits_equal, both_worlds, cfg0_camera, dense_to_stream

pytestmark = pytest.mark.gpu


def assert_worlds_equal(w: v.World, o: OracleWorld):
    sx, sy, sz = w.sectors
    total = 0
    for y in range(sy):
        for z in range(sz):
            for x in range(sx):
                idx = v.sector_index(x, y, z)
                mg, bg = w.read_sector(idx)
                mo, bo = o.read_sector(idx)
                assert mg == mo, f"sector {(x, y, z)} mask {mg:#x} != {mo:#x}"
                assert np.array_equal(bg, bo), f"sector {(x, y, z)} bricks differ"
                total += bin(mg).count("1")
    assert w.stats()["allocated_bricks"] == total == o.allocated_bricks()


def random_edits(rng, n, size, rmax=24):
    e = np.zeros(n, v.EDIT_DTYPE)
    e["center"] = rng.integers(-16, np.array(size) + 16, (n, 3))
    e["radius"] = rng.integers(0, rmax, n)
    kind = rng.integers(0, 4, n)
    e["material"] = np.where(kind == 0, 0, rng.integers(1, 256, n))
    e["mode"] = np.where(kind == 3, v.capi.EDIT_REPLACE, v.capi.EDIT_FILL)
    return e


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_edit_batches_match_oracle(gpu, seed):
    rng = np.random.default_rng(seed)
    data = v.synth_mix(96, seed=40 + seed)
    w, o = both_worlds(data)
    cam = v.look_at((48, 80, -30), (48, 40, 48), 80.0, 96, 64)
    for batch in range(4):
        edits = random_edits(rng, int(rng.integers(1, 12)), (96, 96, 96))
        w.edit(edits)
        o.edit(edits)
        assert_worlds_equal(w, o)
        assert_hits_equal(w.render_view(cam), o.render_view(cam))
    w.close()


def test_carve_to_empty_and_refill(gpu):
    vol = np.zeros((64, 64, 64), np.uint8)
    vol[:16] = 5
    w, o = both_worlds(dense_to_stream(vol))
    carve = np.zeros(1, v.EDIT_DTYPE)
    carve["center"] = (32, 0, 32)
    carve["radius"] = 200
    w.edit(carve)
    o.edit(carve)
    assert_worlds_equal(w, o)
    assert w.stats()["allocated_bricks"] == 0
    fill = np.zeros(3, v.EDIT_DTYPE)
    fill["center"] = [(10, 10, 10), (50, 40, 20), (0, 0, 0)]
    fill["radius"] = [9, 12, 0]
    fill["material"] = [7, 8, 9]
    w.edit(fill)
    o.edit(fill)
    assert_worlds_equal(w, o)
    rays = v.random_rays((64, 64, 64), seed=4, n=20_000)
    assert_hits_equal(w.cast(rays), o.cast(rays))
    w.close()


def test_dirty_sync_moves_and_zero_fill(gpu):
    rng = np.random.default_rng(7)
    vol = ((rng.random((64, 96, 64)) < 0.03) * rng.integers(1, 256, (64, 96, 64))).astype(np.uint8)
    vol[40:] = 0
    data = dense_to_stream(vol)
    w, o = both_worlds(data)
    for step in range(6):
        k = int(rng.integers(1, len(data.sector_idx) + 1))
        pick = rng.choice(len(data.sector_idx), k, replace=False)
        idx = data.sector_idx[pick]
        masks = np.array([int(o.sector_mask(int(i))) for i in idx], np.uint64)
        new_masks = masks.copy()
        dirty = np.zeros(k, np.uint64)
        bricks = []
        for j in range(k):
            m = int(masks[j])
            add = int(rng.integers(0, 1 << 63)) & ~m & int(rng.integers(0, 1 << 63))
            drop = m & int(rng.integers(0, 1 << 63))
            nm = (m & ~drop) | add
            if step == 5 and j == 0:
                nm = 0  # delete a sector
            d = nm & int(rng.integers(0, 1 << 63))
            new_masks[j] = nm
            dirty[j] = d
            for _ in range(bin(d).count("1")):
                bricks.append(rng.integers(0, 256, 512, dtype=np.uint8) * (rng.random(512) < 0.1))
        b = np.stack(bricks).astype(np.uint8) if bricks else None
        w.sync_sectors(idx, new_masks, b, dirty)
        o.sync_sectors(idx, new_masks, b, dirty)
        assert_worlds_equal(w, o)
    rays = v.random_rays((64, 64, 96), seed=5, n=50_000)
    assert_hits_equal(w.cast(rays), o.cast(rays))
    w.close()


def test_pool_growth_keeps_content(gpu):
    data = v.synth_terrain((256, 256, 256), base=96, amplitude=48, seed=1)
    w = v.World(data.sectors, brick_capacity=64)
    half = len(data.sector_idx) // 2
    nb = int(sum(bin(int(m)).count("1") for m in data.alloc_mask[:half]))
    w.sync_sectors(data.sector_idx[:half], data.alloc_mask[:half], data.bricks[:nb])
    w.sync_sectors(data.sector_idx[half:], data.alloc_mask[half:], data.bricks[nb:])
    assert w.stats()["brick_capacity"] >= data.n_bricks
    o = OracleWorld(data.sectors)
    o.upload(data)
    cam = cfg0_camera(320, 180)
    assert_hits_equal(w.render_view(cam), o.render_view(cam))
    w.close()


def test_invalid_arguments(gpu):
    w = v.World((1, 1, 1))
    with pytest.raises(v.VrtError):
        bad = np.zeros(1, v.EDIT_DTYPE)
        bad["radius"] = 5000
        w.edit(bad)
    with pytest.raises(v.VrtError):
        v.World((65, 1, 1))
    with pytest.raises(v.VrtError):
        w.sync_sectors([0], [1], None)  # brick data missing
    w.close()


def test_world_cvox_save_load(gpu, tmp_path):
    data = v.synth_mix(96, seed=21)
    w, o = both_worlds(data)
    e = np.zeros(2, v.EDIT_DTYPE)
    e["center"] = [(40, 40, 40), (10, 80, 10)]
    e["radius"] = [15, 9]
    e["material"] = [0, 99]
    w.edit(e)
    o.edit(e)
    p = tmp_path / "world.cvox"
    w.save_cvox(p)
    w2 = v.World(data.sectors)
    w2.load_cvox(p)
    assert_worlds_equal(w2, o)
    w.close()
    w2.close()


def test_world_loads_the_reference_file(gpu):
    """A device world loads the file the reference's own Serialize wrote
    (tests/golden/refworld.cvox) into the seeded world's content, and traces like the oracle."""
    from tests.golden.make_golden_cvox import OUT_FILE, build_world
    data = build_world()
    w = v.World(data.sectors)
    try:
        w.load_cvox(OUT_FILE)
    except v.VrtError as e:
        w.close()
        if "libzstd" in str(e):
            pytest.skip("compressed packs need the system libzstd.so.1")
        raise
    o = OracleWorld(data.sectors)
    o.upload(data)
    assert_worlds_equal(w, o)
    rays = v.random_rays(w.size, seed=8, n=20_000)
    assert_hits_equal(w.cast(rays), o.cast(rays))
    w.close()
