"""The GLSL traversal mode on the device against the oracle's restatement of the GPU
renderer's rayCast (VoxelTraversal.glsl:100-204): casts, single-view paths, batches,
edits that change the 4th-level group masks.  The oracle's restatement is itself
pinned to the reference's shader source compiled as C++ (tests/test_glsl_pin.py)."""
import numpy as np
import pytest

import voxelrt_gb300 as v
from oracle.oracle import OracleWorld
from tests.helpers import assert_hits_equal, both_worlds, cell_corner_world, cfg0_camera, cfg0_world, dense_to_stream, \
    make_rays, oracle_view

pytestmark = pytest.mark.gpu

SUN = (0.3, 0.8, 0.5)


def sparse_world(seed, shape=(128, 320, 288), blobs=60):
    """(Y, Z, X) sector extents not multiples of 4, solid boxes far apart: long empty runs."""
    rng = np.random.default_rng(seed)
    vol = np.zeros(shape, np.uint8)
    for _ in range(blobs):
        y, z, x = rng.integers(0, shape)
        vol[max(0, y - 5):y + 5, max(0, z - 5):z + 5, max(0, x - 5):x + 5] = rng.integers(1, 256)
    return dense_to_stream(vol)


def camera_frame_rays(rng, size, n, zero_frac=0.02):
    eye = rng.uniform((0, 0, 0), size)
    wo = tuple(int(c) for c in np.floor(eye))
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d[rng.random(d.shape) < zero_frac] = 0.0
    return make_rays(np.tile((eye - np.floor(eye)).astype(np.float32), (n, 1)), d), wo


@pytest.mark.parametrize("seed", [1, 2])
def test_glsl_cast_matches_oracle(gpu, seed):
    rng = np.random.default_rng(seed)
    for data in (sparse_world(seed), v.synth_mix(96, seed=seed), cfg0_world()):
        size = [s * 32 for s in data.sectors]
        w, o = both_worlds(data)
        for _ in range(3):
            rays, wo = camera_frame_rays(rng, size, 40_000)
            assert_hits_equal(w.cast(rays, world_origin=wo, glsl=True),
                              o.cast(rays, world_origin=wo, glsl=True))
        # world-frame rays, where the 5-ulp bias can stall a ray until the cap
        rays = v.random_rays(size, seed=seed, n=30_000)
        assert_hits_equal(w.cast(rays, max_iters=96, glsl=True), o.cast(rays, max_iters=96, glsl=True))
        w.close()


def test_glsl_mode_takes_fewer_steps_in_sparse_worlds(gpu):
    data = sparse_world(7, shape=(256, 512, 512), blobs=30)
    w, o = both_worlds(data)
    rays, wo = camera_frame_rays(np.random.default_rng(7), [512, 256, 512], 50_000, zero_frac=0.0)
    a = w.cast(rays, world_origin=wo)
    b = w.cast(rays, world_origin=wo, glsl=True)
    assert_hits_equal(b, o.cast(rays, world_origin=wo, glsl=True))
    assert b["steps"].astype(np.int64).sum() < 0.8 * a["steps"].astype(np.int64).sum()
    w.close()


def test_glsl_render_paths_match_oracle(gpu):
    data = cfg0_world()
    w, o = both_worlds(data)
    cam = cfg0_camera(160, 90)
    for view in (v.make_view(cam, glsl=True), v.make_view(cam, shadow_dir=SUN, glsl=True),
                 v.make_view(cam, n_bounces=3, max_iters=200, glsl=True)):
        got = v.render_path(w, view)
        want = oracle_view(o, view)
        for k in range(want.shape[0]):
            assert_hits_equal(got[k], want[k])
    w.close()


def test_glsl_batch_matches_oracle_and_per_view(gpu):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    worlds, oracles, views = [], [], []
    for i in range(5):
        data = sparse_world(20 + i, shape=(96, 160, 128), blobs=20) if i % 2 else v.synth_mix(96, seed=30 + i)
        w, o = both_worlds(data)
        worlds.append(w)
        oracles.append(o)
        size = [s * 32 for s in data.sectors]
        for k in range(3):
            cam = v.look_at(rng.uniform(0, size), rng.uniform(0, size), 70.0, *[(64, 48), (33, 65), (80, 40)][k])
            views.append(v.make_view(cam, world=i, glsl=True, **[{}, {"shadow_dir": SUN}, {"n_bounces": 2}][k]))
    for cfg in (None, v.BatchConfig(8, 8, 1, 2, 0, 8, 4, 16), v.BatchConfig(32, 1, 0, 4, 0, 28, 1, 2)):
        b = v.Batch(worlds, views, cfg)
        hits = b.run()
        for i, vw in enumerate(views):
            got, want = b.view_hits(hits, i), oracle_view(oracles[vw.world], vw)
            for k in range(want.shape[0]):
                assert_hits_equal(got[k], want[k])
        n = b.total_records
        a = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
        c = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
        b.launch(a, graph=True)
        b.launch_per_view(c)
        torch.cuda.synchronize()
        assert torch.equal(a, c)
        b.close()
    # one traversal mode per launch
    with pytest.raises(v.VrtError):
        v.Batch(worlds, views[:2] + [v.make_view(views[0].cam, world=0)])
    for w in worlds:
        w.close()


def test_glsl_group_masks_follow_edits(gpu):
    # carving whole sectors empty and filling empty ones changes the 4th-level masks
    data = v.synth_mix(128, seed=9)
    w, o = both_worlds(data)
    rng = np.random.default_rng(9)
    cam = v.look_at((64, 120, -20), (64, 40, 64), 80.0, 96, 64)
    for step in range(3):
        e = np.zeros(3, v.EDIT_DTYPE)
        e["center"] = rng.integers(0, 128, (3, 3))
        e["radius"] = [40, 25, 12]
        e["material"] = [0, 7 + step, 0] if step != 1 else [5, 0, 9]
        w.edit(e)
        o.edit(e)
        view = v.make_view(cam, glsl=True)
        got = v.render_path(w, view)
        assert_hits_equal(got[0], oracle_view(o, view)[0])
        rays, wo = camera_frame_rays(rng, [128, 128, 128], 20_000)
        assert_hits_equal(w.cast(rays, world_origin=wo, glsl=True), o.cast(rays, world_origin=wo, glsl=True))
    w.close()


def test_glsl_coarse_casts_match_oracle(gpu):
    """rayCastCoarse (VRT_CAST_GLSL_COARSE): 0.001 bias, coarse hits from iteration 31,
    cap 96; through the thread-per-ray kernel and, from 2^18 rays, the persistent one."""
    rng = np.random.default_rng(13)
    for data in (sparse_world(13), v.synth_mix(96, seed=13), cell_corner_world()):
        size = [s * 32 for s in data.sectors]
        w, o = both_worlds(data)
        for n in (30_000, (1 << 18) + 5):
            rays, wo = camera_frame_rays(rng, size, n)
            got = w.cast(rays, world_origin=wo, glsl=True, coarse=True)
            assert_hits_equal(got, o.cast(rays, world_origin=wo, glsl=True, coarse=True))
            assert int(got["steps"].max()) <= 96
        w.close()
    # the known answer: the coarse step at iteration 31 stops on the cell's solid voxel
    data = cell_corner_world()
    w, _ = both_worlds(data)
    d = np.array([1.0, 1e-3, 1e-3], np.float32)
    h = w.cast(make_rays([[1.5, 0.5, 0.5]], [d / np.linalg.norm(d)]), glsl=True, coarse=True)[0]
    assert int(h["steps"]) == 31 and tuple(v.unpack_voxel(np.array([h["voxel"]]))[0]) == (67, 3, 3)
    with pytest.raises(v.VrtError):  # coarse without the GLSL mode
        p = v.capi.CastParams((v.C.c_int32 * 3)(0, 0, 0), 0, v.capi.CAST_GLSL_COARSE)
        v.check(v.lib().vrt_cast(w.handle, None, 0, v.C.byref(p), None, None))
    w.close()


def test_glsl_aniso_casts_match_oracle(gpu):
    """Anisotropic LODs (VRT_CAST_GLSL_ANISO, u_UseAnisotropicLods): the raw cell,
    sector and group masks restricted to the 4x4x4 box ahead of the ray; alone and with
    rayCastCoarse, through both cast kernels.  Same voxels as the isotropic mode where
    neither is capped and no direction component is zero, in no more steps."""
    rng = np.random.default_rng(17)
    for data in (sparse_world(17), v.synth_mix(96, seed=17), cell_corner_world()):
        size = [s * 32 for s in data.sectors]
        w, o = both_worlds(data)
        for n in (30_000, (1 << 18) + 3):
            rays, wo = camera_frame_rays(rng, size, n)
            got = w.cast(rays, world_origin=wo, aniso=True)
            assert_hits_equal(got, o.cast(rays, world_origin=wo, glsl=True, aniso=True))
            iso = w.cast(rays, world_origin=wo, glsl=True)
            # a zero direction component makes a side distance NaN (0 * inf) wherever the
            # stepped-to voxel is not above the origin on that axis, and the shader's min then
            # drops a side: such rays may part ways between the two modes
            nz = (rays["dir"] != 0).all(axis=1)
            both = (got["steps"] < 256) & (iso["steps"] < 256) & nz
            assert np.array_equal(got["voxel"][both], iso["voxel"][both])
            assert (got["steps"][both] <= iso["steps"][both]).all()
            assert got["steps"].astype(np.int64).sum() < iso["steps"].astype(np.int64).sum()
            c = w.cast(rays, world_origin=wo, coarse=True, aniso=True)
            assert_hits_equal(c, o.cast(rays, world_origin=wo, glsl=True, coarse=True, aniso=True))
        w.close()
    with pytest.raises(v.VrtError):  # anisotropic LODs without the GLSL mode
        w, _ = both_worlds(cell_corner_world())
        p = v.capi.CastParams((v.C.c_int32 * 3)(0, 0, 0), 0, v.capi.CAST_GLSL_ANISO)
        try:
            v.check(v.lib().vrt_cast(w.handle, None, 0, v.C.byref(p), None, None))
        finally:
            w.close()


def test_glsl_aniso_paths_and_batch_match_oracle(gpu):
    rng = np.random.default_rng(19)
    worlds, oracles, views = [], [], []
    for i in range(4):
        data = sparse_world(40 + i, shape=(96, 160, 128), blobs=20) if i % 2 else v.synth_mix(96, seed=50 + i)
        w, o = both_worlds(data)
        worlds.append(w)
        oracles.append(o)
        size = [s * 32 for s in data.sectors]
        for k in range(3):
            cam = v.look_at(rng.uniform(0, size), rng.uniform(0, size), 70.0, *[(64, 48), (33, 65), (80, 40)][k])
            views.append(v.make_view(cam, world=i, aniso=True, **[{}, {"shadow_dir": SUN}, {"n_bounces": 2}][k]))
    for vw in views[:3]:
        got, want = v.render_path(worlds[vw.world], vw), oracle_view(oracles[vw.world], vw)
        for k in range(want.shape[0]):
            assert_hits_equal(got[k], want[k])
    for cfg in (None, v.BatchConfig(32, 1, 0, 4, 0, 28, 1, 2)):
        b = v.Batch(worlds, views, cfg)
        hits = b.run()
        for i, vw in enumerate(views):
            got, want = b.view_hits(hits, i), oracle_view(oracles[vw.world], vw)
            for k in range(want.shape[0]):
                assert_hits_equal(got[k], want[k])
        b.close()
    # one traversal mode per launch: GLSL and GLSL with anisotropic LODs do not mix
    with pytest.raises(v.VrtError):
        v.Batch(worlds, views[:2] + [v.make_view(views[0].cam, world=0, glsl=True)])
    bad = v.make_view(views[0].cam, world=0)
    bad.flags |= v.capi.VIEW_GLSL_ANISO  # without the GLSL mode
    with pytest.raises(v.VrtError):
        v.Batch(worlds, [bad])
    # edits re-derive the cell masks the anisotropic LODs read
    e = np.zeros(2, v.EDIT_DTYPE)
    e["center"] = [[40, 40, 40], [60, 30, 50]]
    e["radius"] = [20, 9]
    e["material"] = [0, 33]
    worlds[0].edit(e)
    oracles[0].edit(e)
    rays, wo = camera_frame_rays(rng, [96, 96, 96], 40_000)
    assert_hits_equal(worlds[0].cast(rays, world_origin=wo, aniso=True),
                      oracles[0].cast(rays, world_origin=wo, glsl=True, aniso=True))
    for w in worlds:
        w.close()


def test_edits_rederive_only_their_sector_groups(gpu):
    """A world of 3 x 1 x 3 sector groups: each edit changes one or two groups, whose
    brick-table entries alone are re-derived (the rest keep theirs).  Filling empty
    sectors and carving whole blobs away flips sector emptiness, so the group masks the
    GLSL and anisotropic entries read change; casts in all three modes match the oracle."""
    data = sparse_world(5)
    assert data.sectors == (9, 4, 10)
    w, o = both_worlds(data)
    rng = np.random.default_rng(5)
    size = [s * 32 for s in data.sectors]
    edits = [((40, 60, 40), 20, 9), ((250, 100, 280), 30, 0), ((150, 20, 150), 12, 33), ((260, 64, 40), 24, 0),
             ((30, 110, 300), 16, 77)]
    for center, radius, material in edits:
        e = np.zeros(1, v.EDIT_DTYPE)
        e["center"], e["radius"], e["material"] = center, radius, material
        w.edit(e)
        o.edit(e)
        rays, wo = camera_frame_rays(rng, size, 20_000, zero_frac=0.0)
        assert_hits_equal(w.cast(rays, world_origin=wo), o.cast(rays, world_origin=wo))
        assert_hits_equal(w.cast(rays, world_origin=wo, glsl=True), o.cast(rays, world_origin=wo, glsl=True))
        assert_hits_equal(w.cast(rays, world_origin=wo, aniso=True),
                          o.cast(rays, world_origin=wo, glsl=True, aniso=True))
    w.close()
