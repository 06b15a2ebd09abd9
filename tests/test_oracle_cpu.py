"""Known-answer tests of the CPU oracle (no GPU).

The reference ships no tests or fixtures, so these pin the oracle's restatement of
src/VoxelRT/CpuRenderer.cpp:20-224 with hand-derived answers, an independent numpy
occupancy model, and the golden vectors produced by the reference's own RayCast
(tests/golden/, see tests/golden/make_golden.py).
"""
import numpy as np
import pytest

import voxelrt_gb300 as v
from oracle.oracle import OracleWorld
from tests.helpers import cfg0_camera, cfg0_world, dense_to_stream, make_rays, single_voxel_world


def occupancy_numpy(brick: np.ndarray) -> np.ndarray:
    """8 cell masks of a (512,) brick: cell cx|cz<<1|cy<<2, bit vx + vz*4 + vy*16."""
    b = brick.reshape(8, 8, 8) != 0  # (y, z, x)
    out = np.zeros(8, np.uint64)
    for cy in range(2):
        for cz in range(2):
            for cx in range(2):
                m = 0
                for vy in range(4):
                    for vz in range(4):
                        for vx in range(4):
                            if b[cy * 4 + vy, cz * 4 + vz, cx * 4 + vx]:
                                m |= 1 << (vx + vz * 4 + vy * 16)
                out[cx | cz << 1 | cy << 2] = m
    return out


def test_occupancy_matches_numpy_model():
    rng = np.random.default_rng(0)
    vol = np.zeros((32, 32, 32), np.uint8)
    for density in (0.01, 0.1, 0.5):
        vol[:] = (rng.random(vol.shape) < density) * rng.integers(1, 256, vol.shape)
        data = dense_to_stream(vol)
        o = OracleWorld(data.sectors)
        o.upload(data)
        k = 0
        for b in range(64):
            bx, bz, by = b & 3, (b >> 2) & 3, b >> 4
            want = occupancy_numpy(vol[by * 8:by * 8 + 8, bz * 8:bz * 8 + 8, bx * 8:bx * 8 + 8].reshape(-1))
            assert np.array_equal(o.brick_occupancy(bx, by, bz), want)
            k += 1


def test_single_voxel_known_answers():
    data = single_voxel_world((37, 21, 45), material=9)
    o = OracleWorld(data.sectors)
    o.upload(data)
    # slightly tilted axis rays (unit main component, so t is exact): t is the
    # distance to the voxel face the ray enters through
    rays = make_rays([[37.5, 21.5, 25.5], [37.5, 21.5, 60.5], [60.5, 21.5, 45.5], [37.5, 0.5, 45.5]],
                     [[1e-3, 1e-3, 1], [1e-3, 1e-3, -1], [-1, 1e-3, 1e-3], [1e-3, 1, 1e-3]])
    h = o.cast(rays)
    assert (h["voxel"] == (37 | 21 << 11 | 45 << 21)).all()
    assert (h["material"] == 9).all()
    assert h["face"].tolist() == [4, 5, 1, 2]
    assert h["t"].tolist() == [19.5, 14.5, 22.5, 20.5]
    # a ray that passes beside the voxel misses and leaves the 64^3 grid
    miss = o.cast(make_rays([[36.5, 21.5, 0.5]], [[1e-3, 1e-3, 1]]))
    assert miss["voxel"][0] == v.MISS_VOXEL and miss["face"][0] == 0xFF and np.isinf(miss["t"][0])


def test_zero_direction_components_follow_minps():
    # With dir.y = dir.z = 0 the side distances of y and z are NaN (-inf + inf);
    # minps returns its second operand on NaN, so tmin is NaN, floor2i gives
    # INT32_MIN and the ray leaves the grid on iteration 1 (CpuRenderer.cpp:200,
    # SIMD_AVX512.h:109,123).  The ray of the previous test, exactly axis-aligned:
    data = single_voxel_world((37, 21, 45), material=9)
    o = OracleWorld(data.sectors)
    o.upload(data)
    h = o.cast(make_rays([[60.5, 21.5, 45.5]], [[-1, 0, 0]]))
    assert h["voxel"][0] == v.MISS_VOXEL and h["steps"][0] == 1
    # one zero component in x: min(NaN, sy) = sy, so the ray still traverses
    h = o.cast(make_rays([[37.5, 0.5, 45.5]], [[0, 1, 1e-3]]))
    assert h["voxel"][0] == (37 | 21 << 11 | 45 << 21)


def test_empty_space_skipping_step_counts():
    # a ray through an empty 64^3 world: each iteration steps a whole 32-voxel sector
    data = v.SectorData((2, 2, 2), np.zeros(0, np.int32), np.zeros(0, np.uint64), np.zeros((0, 512), np.uint8))
    o = OracleWorld(data.sectors)
    o.upload(data)
    h = o.cast(make_rays([[0.5, 10.5, 10.5]], [[1, 1e-3, 1e-3]]))
    assert h["steps"][0] == 2 and h["voxel"][0] == v.MISS_VOXEL
    assert o.last_stats["step_calls"] == 2 and o.last_stats["occ_fetches"] == 0


def test_iteration_cap_is_a_miss():
    data = cfg0_world()
    o = OracleWorld(data.sectors)
    o.upload(data)
    cam = cfg0_camera(64, 36)
    full = o.render_view(cam, 1000)
    capped = o.render_view(cam, 2)
    long_rays = full["steps"] >= 2
    assert long_rays.any()
    assert (capped["voxel"][long_rays] == v.MISS_VOXEL).all()
    assert (capped["steps"][long_rays] == 2).all()
    short = ~long_rays
    assert np.array_equal(capped[short], full[short])


def test_clip_keeps_parametric_t():
    # a ray from outside the grid enters through the clip; t stays measured from the
    # original origin (tStart uses the unclipped origin, VoxelTraversal.glsl:163-167)
    data = single_voxel_world((10, 10, 10))
    o = OracleWorld(data.sectors)
    o.upload(data)
    h = o.cast(make_rays([[10.5, 10.5, -100.0]], [[1e-4, 1e-4, 1]]))
    assert h["t"][0] == 110.0 and h["face"][0] == 4


def test_hits_are_solid_and_first_along_ray():
    data = cfg0_world()
    dense = data.dense()
    o = OracleWorld(data.sectors)
    o.upload(data)
    cam = cfg0_camera(320, 180)
    h = o.render_view(cam)
    hit = h["voxel"] != v.MISS_VOXEL
    vox = v.unpack_voxel(h["voxel"][hit])
    assert (dense[vox[:, 1], vox[:, 2], vox[:, 0]] == h["material"][hit]).all()
    # the origin of the camera is outside the world; the voxel just before the hit
    # along the ray (t - 0.5) must be empty for most rays (grazing hits excepted)
    from oracle.oracle import camera_rays
    rays = camera_rays(cam)[hit]
    p = rays["origin"] + cam_world_origin(cam) + rays["dir"] * (h["t"][hit][:, None] - 0.5)
    pi = np.floor(p).astype(int)
    inb = (pi >= 0).all(1) & (pi < 256).all(1)
    before = dense[pi[inb, 1], pi[inb, 2], pi[inb, 0]]
    assert (before == 0).mean() > 0.95


def cam_world_origin(cam):
    return np.array(list(cam.world_origin), np.float32)


def test_sync_dirty_semantics():
    rng = np.random.default_rng(3)
    vol = (rng.random((64, 64, 64)) < 0.05) * rng.integers(1, 256, (64, 64, 64))
    vol[16:] = 0  # bricks with by >= 2 stay empty
    data = dense_to_stream(vol.astype(np.uint8))
    o = OracleWorld(data.sectors)
    o.upload(data)
    idx = int(data.sector_idx[0])
    m, bricks = o.read_sector(idx)
    assert m == int(data.alloc_mask[0])
    # drop the lowest brick, add brick 63 without data (zero-filled), keep the rest
    low = m & -m
    new_mask = (m & ~low) | (1 << 63)
    o.sync_sectors([idx], [new_mask], None, dirty_mask=[0])
    m2, b2 = o.read_sector(idx)
    assert m2 == new_mask
    assert not (m >> 63) & 1
    assert np.array_equal(b2[:-1], bricks[1:])
    assert not b2[-1].any()
    # delete the sector
    o.sync_sectors([idx], [0])
    assert o.sector_mask(idx) == 0


def sphere_model(vol, center, r, material, replace=False):
    Y, Z, X = vol.shape
    y, z, x = np.ogrid[:Y, :Z, :X]
    inside = (x - center[0]) ** 2 + (y - center[1]) ** 2 + (z - center[2]) ** 2 <= r * r
    if replace:
        inside &= vol != 0
    vol[inside] = material


@pytest.mark.parametrize("seed", [0, 1])
def test_edit_semantics_vs_dense_model(seed):
    rng = np.random.default_rng(seed)
    vol = np.zeros((64, 96, 64), np.uint8)
    vol[:20] = 3
    data = dense_to_stream(vol)
    o = OracleWorld(data.sectors)
    o.upload(data)
    edits = np.zeros(12, v.EDIT_DTYPE)
    for k in range(len(edits)):
        edits[k]["center"] = rng.integers(-10, 100, 3)
        edits[k]["radius"] = rng.integers(0, 20)
        edits[k]["material"] = 0 if k % 3 == 0 else rng.integers(1, 256)
        edits[k]["mode"] = 1 if k % 4 == 3 else 0
    o.edit(edits)
    for e in edits:
        sphere_model(vol, e["center"], int(e["radius"]), int(e["material"]), e["mode"] == 1)
    want = dense_to_stream(vol)
    # every sector matches the dense model and holds no empty bricks
    got_masks = {int(i): o.sector_mask(int(i)) for i in want.sector_idx}
    assert got_masks == {int(i): int(m) for i, m in zip(want.sector_idx, want.alloc_mask)}
    assert o.allocated_bricks() == want.n_bricks
    for x in range(0, 64, 7):
        for y in range(0, 64, 5):
            for z in range(0, 96, 3):
                assert o.voxel(x, y, z) == vol[y, z, x]
