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
from tests.helpers import cell_corner_world, cfg0_camera, cfg0_world, dense_to_stream, make_rays, single_voxel_world


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


# ---- GLSL mode (VoxelTraversal.glsl rayCast); parity unpinned, so known answers and
# properties against the default mode

def _empty_world(sectors):
    data = v.SectorData(sectors, np.zeros(0, np.int32), np.zeros(0, np.uint64), np.zeros((0, 512), np.uint8))
    o = OracleWorld(data.sectors)
    o.upload(data)
    return o


def test_glsl_mode_group_level_known_answer():
    # empty 256^3 world = 2x2x2 groups of 4^3 sectors, all empty: iteration 0 leaves the
    # start voxel (100 -> 101), getStepPos skips to the 128-voxel group cell's end (127),
    # iteration 1 enters x = 128 and skips to 255, iteration 2 leaves the grid
    o = _empty_world((8, 8, 8))
    r = make_rays([[100.5, 100.5, 100.5]], [[1, 1e-4, 1e-4]])
    h = o.cast(r, glsl=True)
    assert h["steps"][0] == 2 and h["voxel"][0] == v.MISS_VOXEL
    assert o.last_stats["step_calls"] == 2 and o.last_stats["occ_fetches"] == 0
    # the default mode steps sector by sector: 101 -> 127 | 128 -> 159 | ... | 224 -> 255
    h = o.cast(r)
    assert h["steps"][0] == 5


def test_glsl_mode_single_voxel_hit():
    data = single_voxel_world((40, 20, 50), material=9, sectors=(8, 2, 8))
    o = OracleWorld(data.sectors)
    o.upload(data)
    h = o.cast(make_rays([[40.5, 20.5, 200.25]], [[1e-4, 1e-4, -1]]), glsl=True)
    assert h["voxel"][0] == 40 | 20 << 11 | 50 << 21 and h["material"][0] == 9
    assert h["face"][0] == 5  # z axis, moving in -z
    # t is the biased tmin of the hit step: the +z face at 51 is 149.25 away, plus 5 ulp
    t = np.float32(149.25).view(np.uint32) + 5
    assert h["t"][0].view(np.uint32) == t


def test_glsl_mode_finds_the_same_first_voxel_in_sparse_worlds():
    # the 4th level must never skip a non-empty sector: in a sparse world rays from empty
    # space hit the same voxel as the default mode, except where the two biases (+5 ulp
    # vs +0.001) enter a different voxel at an edge.  Rays start as camera rays do: in the
    # frame of worldOrigin = floor(eye), origin = the fractional part (GBuffer.h:79); the
    # 5-ulp bias of rayCast only moves the position off a cell boundary when positions
    # scale with t like that, and rays in far-from-origin frames stall until the cap.
    rng = np.random.default_rng(3)
    vol = np.zeros((128, 256, 256), np.uint8)
    for _ in range(150):
        y, z, x = rng.integers(0, (128, 256, 256))
        vol[max(0, y - 6):y + 6, max(0, z - 6):z + 6, max(0, x - 6):x + 6] = rng.integers(1, 256)
    data = dense_to_stream(vol)
    o = OracleWorld(data.sectors)
    o.upload(data)
    dense = data.dense()
    same = hits = steps_a = steps_b = 0
    for k in range(60):
        eye = rng.uniform((0, 0, 0), (256, 128, 256))
        if dense[int(eye[1]), int(eye[2]), int(eye[0])]:
            continue
        wo = np.floor(eye).astype(np.int32)
        d = rng.normal(size=(500, 3)).astype(np.float32)
        r = make_rays(np.tile((eye - wo).astype(np.float32), (500, 1)), d)
        a, b = o.cast(r, world_origin=tuple(wo)), o.cast(r, world_origin=tuple(wo), glsl=True)
        both = (a["voxel"] != v.MISS_VOXEL) & (b["voxel"] != v.MISS_VOXEL)
        hits += both.sum()
        same += (a["voxel"][both] == b["voxel"][both]).sum()
        steps_a += a["steps"].astype(np.int64).sum()
        steps_b += b["steps"].astype(np.int64).sum()
    assert hits > 2000
    assert same / hits > 0.99
    # and it takes fewer iterations through the empty space
    assert steps_b < steps_a


def test_glsl_mode_iteration_cap_default_256():
    o = _empty_world((64, 1, 64))
    r = make_rays([[0.5, 16.5, 0.5]], [[1, 0, 1e-3]])  # zero y component: x86 min leaves NaN sides out
    h = o.cast(r, glsl=True, max_iters=3)
    assert h["steps"][0] <= 3


def test_glsl_coarse_rays_stop_at_the_first_solid_voxel_of_a_cell():
    """rayCastCoarse (VoxelTraversal.glsl:206-240): in a world with one solid voxel at
    offset (3,3,3) of every 4^3 cell, a ray along +x near y = z = 0 steps two voxels
    per iteration (its 2^3 blocks are empty) and lands on x = 2 + 2i; from iteration
    31 (x = 64) the non-empty cell ends it at that cell's solid voxel (67, 3, 3).
    rayCast, with no coarse steps, runs to the edge of the world."""
    data = cell_corner_world()
    o = OracleWorld(data.sectors)
    o.upload(data)
    d = np.array([1.0, 1e-3, 1e-3], np.float32)
    rays = make_rays([[1.5, 0.5, 0.5]], [d / np.linalg.norm(d)])
    h = o.cast(rays, glsl=True, coarse=True)[0]
    assert int(h["steps"]) == 31
    assert tuple(v.unpack_voxel(np.array([h["voxel"]]))[0]) == (67, 3, 3)
    assert int(h["material"]) == 7
    assert 62.5 < float(h["t"]) < 62.51  # the biased tmin of the step onto x = 64 from x = 1.5
    plain = o.cast(rays, glsl=True)[0]
    assert int(plain["voxel"]) == v.MISS_VOXEL
    # before iteration 31 a coarse ray is a rayCast ray with the CPU bias: capped at 20
    # iterations it misses where it stood
    capped = o.cast(rays, glsl=True, coarse=True, max_iters=20)[0]
    assert int(capped["voxel"]) == v.MISS_VOXEL and int(capped["steps"]) == 20


def test_ray_cell_lut_is_the_forward_box():
    """GenerateRayCellInteractionMaskLUT (GpuRenderer.cpp:193-210): entry idx + octant*64
    holds the cells of the 4^3 block at or ahead of cell idx on every axis, ahead meaning
    +1 where the octant's bit is set (x bit 0, y bit 1, z bit 2) and -1 elsewhere."""
    from oracle.oracle import ray_cell_lut
    lut = ray_cell_lut()
    for oct_ in range(8):
        sgn = [1 if oct_ >> a & 1 else -1 for a in range(3)]  # x, y, z
        for idx in range(64):
            o = (idx & 3, idx >> 4, (idx >> 2) & 3)
            want = 0
            for x in range(4):
                for y in range(4):
                    for z in range(4):
                        if all((p - q) * s >= 0 for p, q, s in zip((x, y, z), o, sgn)):
                            want |= 1 << (x | z << 2 | y << 4)
            assert int(lut[idx + oct_ * 64]) == want


def test_anisotropic_lods_find_the_same_voxels_in_fewer_steps():
    """Masking the occupancy behind the ray (u_UseAnisotropicLods) only widens the empty
    cells ahead of it: the first solid voxel along each ray is the same, with no more
    iterations, and fewer over many rays in a cluttered world (rays without a zero
    direction component; see the GPU test for those)."""
    rng = np.random.default_rng(3)
    vol = (rng.random((64, 64, 64)) < 0.02).astype(np.uint8) * 5
    data = dense_to_stream(vol)
    o = OracleWorld(data.sectors)
    o.upload(data)
    eye = np.array([20.3, 30.7, 11.2], np.float32)
    d = rng.normal(size=(20_000, 3)).astype(np.float32)
    rays = make_rays(np.tile(eye - np.floor(eye), (len(d), 1)), d)
    wo = tuple(int(c) for c in np.floor(eye))
    iso = o.cast(rays, world_origin=wo, glsl=True)
    ani = o.cast(rays, world_origin=wo, glsl=True, aniso=True)
    hit = iso["voxel"] != v.MISS_VOXEL
    assert hit.mean() > 0.5
    assert np.array_equal(iso["voxel"], ani["voxel"]) and np.array_equal(iso["material"], ani["material"])
    assert (ani["steps"] <= iso["steps"]).all()
    assert ani["steps"].astype(np.int64).sum() < 0.9 * iso["steps"].astype(np.int64).sum()


@pytest.mark.parametrize("glsl", [False, True])
def test_renderer_path_decomposes_into_shadow_and_bounce_paths(glsl):
    """The GPU renderer's whole path (VoxelRender.comp:51-86) interleaves sun rays with the
    bounce chain without changing it: its primary and bounce planes equal the bounce-only
    path, its first sun plane the shadow path, and a sun ray is cast exactly after the
    primary and the first two bounce hits."""
    data = cfg0_world()
    o = OracleWorld(data.sectors)
    o.upload(data)
    cam = cfg0_camera(96, 54)
    sun = np.array([0.3, 0.9, -0.28], np.float32) / np.float32(np.linalg.norm([0.3, 0.9, -0.28]))
    n = 4
    full = o.render_view_path(cam, sun, n, glsl=glsl)
    assert full.shape == (2 + n + 2, 96 * 54)
    bounces = o.render_view_bounces(cam, n, glsl=glsl)
    prim, shad = o.render_view_shadow(cam, sun, glsl=glsl)
    planes_of_bounce = [0, 2, 4, 6, 7]  # primary, bounce 1..4
    for k, p in enumerate(planes_of_bounce):
        assert np.array_equal(full[p], bounces[k])
    assert np.array_equal(full[0], prim) and np.array_equal(full[1], shad)
    for sun_plane, after in ((1, 0), (3, 2), (5, 4)):
        cast = full[sun_plane]["tag"] != 0xFFFFFFFF
        assert np.array_equal(cast, full[after]["voxel"] != 0xFFFFFFFF)
    o.close()


def test_gbuffer_texels_follow_the_material_and_normal():
    """G-buffer of the oracle on a world of one material: every hit texel carries the squared
    RGB565 color rounded to 8 bits and a single-axis normal opposite the ray's direction."""
    vol = np.zeros((64, 64, 64), np.uint8)
    vol[:20] = 5
    data = dense_to_stream(vol)
    o = OracleWorld(data.sectors)
    o.upload(data)
    cam = v.look_at((32.0, 50.0, 32.0), (32.0, 0.0, 33.0), 60.0, 32, 32)
    pal = np.zeros(256, np.uint32)
    pal[5] = (20 << 11) | (40 << 5) | 10
    proj = np.eye(4, dtype=np.float32).reshape(16)
    tex, depth, hits = o.render_gbuffer(cam, pal, proj)
    hit = hits["voxel"] != 0xFFFFFFFF
    assert hit.all()
    rgb = [round((20 / 31) ** 2 * 255), round((40 / 63) ** 2 * 255), round((10 / 31) ** 2 * 255)]
    assert np.all(tex & 0xFFFFFF == rgb[0] | rgb[1] << 8 | rgb[2] << 16)
    # the CPU traversal's normal has the one axis of the record's face, opposite the ray:
    # field 2 where dir < 0 (face odd), 0 where dir >= 0, the other fields 1
    axis, neg = hits["face"] >> 1, hits["face"] & 1
    want_a = np.zeros(len(hits), np.uint32)
    for c in range(3):
        want_a |= np.where(axis == c, np.where(neg == 1, 2, 0), 1).astype(np.uint32) << (2 * c)
    assert np.array_equal(tex >> 24, want_a)
    assert np.any(axis == 1)
    # identity projection: depth = z of hitPos / 16, hitPos in the ray frame (relative to the
    # camera's world origin), within the hit voxel's z extent
    zrel = (hits["voxel"] >> 21).astype(np.float64) - cam.world_origin[2]
    assert np.all((depth >= (zrel - 1e-3) / 16) & (depth <= (zrel + 1 + 1e-3) / 16))
    o.close()
