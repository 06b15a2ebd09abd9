"""Device traversal vs the CPU oracle, bit-exact on every ray (t within 1e-6 relative).

Cases follow the edge cases a brickmap DDA has: empty space, single voxels,
axis-aligned and +-0 direction components (NaN side distances), rays starting
inside solid voxels or outside the grid, non-zero world origins, iteration caps.
"""
import numpy as np
import pytest

import voxelrt_gb300 as v
from oracle.oracle import OracleWorld
from tests.helpers import (assert_hits_equal, both_worlds, cfg0_camera, cfg0_world, dense_to_stream, make_rays,
                           single_voxel_world)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cfg0(gpu):
    data = cfg0_world()
    w, o = both_worlds(data)
    yield data, w, o
    w.close()


def test_cfg0_primary_view_bit_exact(cfg0):
    _, w, o = cfg0
    cam = cfg0_camera()
    got = w.render_view(cam)
    want = o.render_view(cam)
    assert (want["voxel"] != v.MISS_VOXEL).mean() > 0.2  # the view sees terrain
    assert_hits_equal(got, want)


@pytest.mark.parametrize("max_iters", [1, 7, 32, 128, 1000])
def test_cfg0_iteration_caps(cfg0, max_iters):
    _, w, o = cfg0
    cam = cfg0_camera(160, 90)
    assert_hits_equal(w.render_view(cam, max_iters), o.render_view(cam, max_iters))


def test_cfg0_random_rays(cfg0):
    _, w, o = cfg0
    rays = v.random_rays((256, 256, 256), seed=11, n=200_000)
    assert_hits_equal(w.cast(rays), o.cast(rays))


def test_cfg0_rays_from_outside(cfg0):
    _, w, o = cfg0
    rng = np.random.default_rng(5)
    n = 50_000
    orig = rng.uniform(-300, 560, (n, 3)).astype(np.float32)
    tgt = rng.uniform(0, 256, (n, 3))
    d = tgt - orig
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    rays = make_rays(orig, d)
    assert_hits_equal(w.cast(rays), o.cast(rays))


@pytest.mark.parametrize("wo", [(0, 0, 0), (100, 50, -20), (-7, 3, 300)])
def test_world_origin_frames(cfg0, wo):
    _, w, o = cfg0
    rays = v.random_rays((256, 256, 256), seed=3, n=30_000)
    rays["origin"] -= np.asarray(wo, np.float32)
    assert_hits_equal(w.cast(rays, world_origin=wo), o.cast(rays, world_origin=wo))


def test_single_voxel_axis_rays(gpu):
    data = single_voxel_world((37, 21, 45))
    w, o = both_worlds(data)
    origins, dirs = [], []
    for axis in range(3):
        for s in (-1.0, 1.0):
            p = [37.5, 21.5, 45.5]
            p[axis] -= s * 20.0
            for eps in (0.0, -0.0, 1e-3, -1e-3):
                d = [eps, eps, eps]
                d[axis] = s
                origins.append(p)
                dirs.append(d)
            p3 = list(p)
            p3[(axis + 1) % 3] = float(int(p3[(axis + 1) % 3]))  # exactly on a voxel boundary
            d = [1e-3, 1e-3, 1e-3]
            d[axis] = s
            origins.append(p3)
            dirs.append(d)
    rays = make_rays(origins, dirs)
    got, want = w.cast(rays), o.cast(rays)
    assert_hits_equal(got, want)
    hit = want["voxel"] != v.MISS_VOXEL
    assert hit.sum() >= 12
    assert (v.unpack_voxel(want["voxel"][hit]) == [37, 21, 45]).all()
    assert (want["material"][hit] == 7).all()


def test_rays_starting_inside_solid(cfg0):
    data, w, o = cfg0
    dense = data.dense()
    ys, zs, xs = np.nonzero(dense[:80])
    pick = np.random.default_rng(1).choice(len(xs), 5000, replace=False)
    orig = np.stack([xs[pick], ys[pick], zs[pick]], 1).astype(np.float32) + 0.25
    dirs = v.random_rays((256, 256, 256), seed=9, n=5000)["dir"]
    rays = make_rays(orig, dirs)
    got, want = w.cast(rays), o.cast(rays)
    assert_hits_equal(got, want)
    assert (want["steps"][want["voxel"] != v.MISS_VOXEL] == 0).mean() > 0.9


def test_empty_world_and_empty_batch(gpu):
    data = v.SectorData((2, 1, 3), np.zeros(0, np.int32), np.zeros(0, np.uint64), np.zeros((0, 512), np.uint8))
    w, o = both_worlds(data)
    rays = v.random_rays((64, 32, 96), seed=2, n=1000)
    got, want = w.cast(rays), o.cast(rays)
    assert_hits_equal(got, want)
    assert (got["voxel"] == v.MISS_VOXEL).all()
    assert len(w.cast(rays[:0])) == 0


def test_non_power_of_two_extent(gpu):
    rng = np.random.default_rng(4)
    vol = (rng.random((64, 96, 160)) < 0.02).astype(np.uint8) * rng.integers(1, 255, (64, 96, 160), dtype=np.uint8)
    data = dense_to_stream(vol)
    w, o = both_worlds(data)
    rays = v.random_rays((160, 64, 96), seed=8, n=100_000)
    assert_hits_equal(w.cast(rays), o.cast(rays))


def test_degenerate_directions(cfg0):
    _, w, o = cfg0
    rng = np.random.default_rng(6)
    n = 20_000
    orig = rng.uniform(0, 256, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    zero = rng.random((n, 3)) < 0.3
    d[zero] = np.where(rng.random(zero.sum()) < 0.5, 0.0, -0.0)
    d[(d == 0).all(1)] = [0, -1, 0]
    orig[: n // 4] = np.floor(orig[: n // 4])  # origins on voxel corners
    rays = make_rays(orig, d)
    assert_hits_equal(w.cast(rays), o.cast(rays))


def test_rays_near_the_grid_corner_and_brick_edges(gpu):
    # dense random voxels; origins in the first cells of the grid and on brick edges,
    # where state carried from one step to the next must not leak between rays
    rng = np.random.default_rng(12)
    vol = ((rng.random((64, 64, 64)) < 0.08) * rng.integers(1, 256, (64, 64, 64))).astype(np.uint8)
    data = dense_to_stream(vol)
    w, o = both_worlds(data)
    n = 40_000
    orig = rng.uniform(0, 6, (n, 3)).astype(np.float32)
    orig[n // 2:] = (rng.integers(0, 8, (n - n // 2, 3)) * 8 + rng.choice([0.0, 0.25, 7.75], (n - n // 2, 3))).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    rays = make_rays(orig, d)
    assert_hits_equal(w.cast(rays), o.cast(rays))
    cam = v.look_at((0.5, 0.5, 0.5), (40, 30, 50), 80.0, 64, 48)
    assert_hits_equal(w.render_view(cam), o.render_view(cam))
    view = v.make_view(cam, n_bounces=3)
    got = v.render_path(w, view)
    want = o.render_view_bounces(cam, 3)
    for k in range(4):
        assert_hits_equal(got[k], want[k])


def sparse_voxels_world(voxels, sectors):
    """SectorData holding the given (x, y, z, material) voxels."""
    by_sector = {}
    for x, y, z, m in voxels:
        s = (x >> 5, y >> 5, z >> 5)
        b = ((x >> 3) & 3) | ((z >> 3) & 3) << 2 | ((y >> 3) & 3) << 4
        by_sector.setdefault(s, {}).setdefault(b, np.zeros(512, np.uint8))[(x & 7) | (z & 7) << 3 | (y & 7) << 6] = m
    idx, masks, bricks = [], [], []
    for (sx, sy, sz), bs in sorted(by_sector.items()):
        idx.append(v.sector_index(sx, sy, sz))
        masks.append(sum(1 << b for b in bs))
        bricks += [bs[b] for b in sorted(bs)]
    return v.SectorData(sectors, np.array(idx, np.int32), np.array(masks, np.uint64), np.stack(bricks))


@pytest.mark.parametrize("glsl", [False, True])
def test_maximum_world_extent(gpu, glsl):
    """64 x 32 x 64 sectors = 2048 x 1024 x 2048 voxels, the largest world the 11/10/11-bit
    hit packing allows, with voxels at both far corners and scattered between."""
    rng = np.random.default_rng(17)
    vox = [(2047, 1023, 2047, 200), (0, 0, 0, 3), (2047, 0, 0, 4), (0, 1023, 2047, 5)]
    vox += [tuple(int(c) for c in rng.integers(0, (2048, 1024, 2048))) + (int(rng.integers(1, 256)),)
            for _ in range(3000)]
    data = sparse_voxels_world(vox, (64, 32, 64))
    w, o = both_worlds(data)
    # rays at the far corner from inside the world, camera-like frame
    eye = np.array([2040.3, 1015.6, 2041.1])
    wo = tuple(int(c) for c in np.floor(eye))
    d = (np.array([2047.5, 1023.5, 2047.5]) - eye + rng.normal(0, 0.05, (2000, 3))).astype(np.float32)
    r = make_rays(np.tile((eye - np.floor(eye)).astype(np.float32), (2000, 1)), d)
    got = w.cast(r, world_origin=wo, glsl=glsl)
    assert_hits_equal(got, o.cast(r, world_origin=wo, glsl=glsl))
    assert (got["voxel"] == (2047 | 1023 << 11 | 2047 << 21)).mean() > 0.5
    rays = v.random_rays((2048, 1024, 2048), seed=17, n=60_000)
    assert_hits_equal(w.cast(rays, max_iters=400, glsl=glsl), o.cast(rays, max_iters=400, glsl=glsl))
    w.close()


@pytest.mark.parametrize("glsl", [False, True])
@pytest.mark.parametrize("max_iters", [0, 5])
def test_large_casts_take_the_persistent_kernel(cfg0, glsl, max_iters):
    """Casts of 2^18 rays and more run the persistent cast kernel (lanes refilled as rays
    end): a ragged count, random and degenerate directions, rays from inside solid, a
    non-zero world origin, iteration caps."""
    _, w, o = cfg0
    rng = np.random.default_rng(17 + glsl + max_iters)
    n = (1 << 18) + 37
    rays = v.random_rays((256, 256, 256), seed=21, n=n)
    d = rays["dir"].copy()
    zero = rng.random(d.shape) < 0.05
    d[zero] = np.where(rng.random(zero.sum()) < 0.5, 0.0, -0.0)
    d[(d == 0).all(1)] = [0, -1, 0]
    rays["dir"] = d
    rays["tag"] = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    for wo in ((0, 0, 0), (-40, 12, 300)):
        r = rays.copy()
        r["origin"] -= np.array(wo, np.float32)
        assert_hits_equal(w.cast(r, world_origin=wo, max_iters=max_iters, glsl=glsl),
                          o.cast(r, world_origin=wo, max_iters=max_iters, glsl=glsl))


def test_concurrent_large_casts_on_two_streams(cfg0):
    """The persistent cast kernel keeps no device queue: two large casts on one world, on
    two streams at once, give the records of the same casts run one after the other."""
    torch = pytest.importorskip("torch")
    _, w, o = cfg0
    n = 1 << 19
    rays = [v.random_rays((256, 256, 256), seed=s, n=n) for s in (31, 32)]
    d_rays = [torch.from_numpy(r.view(np.uint8)).cuda() for r in rays]
    alone = [torch.empty(n * 16, dtype=torch.uint8, device="cuda") for _ in rays]
    for r, h in zip(d_rays, alone):
        w.cast_device(r, n, h)
    torch.cuda.synchronize()
    streams = [torch.cuda.Stream() for _ in rays]
    mixed = [torch.empty(n * 16, dtype=torch.uint8, device="cuda") for _ in rays]
    for _ in range(3):
        for r, h, s in zip(d_rays, mixed, streams):
            w.cast_device(r, n, h, stream=s)
        torch.cuda.synchronize()
        for a, b in zip(alone, mixed):
            assert torch.equal(a, b)
    sub = rays[1][:1 << 16]
    assert_hits_equal(mixed[1][:sub.size * 16].cpu().numpy().view(v.HIT_DTYPE), o.cast(sub))


def test_l2_persisting_world_matches_oracle(gpu):
    """A VRT_WORLD_L2_PERSIST world: casts, views, paths and a single-world batch on a
    non-default stream carry the L2 window over its brick table and give the oracle's
    records; the stream's own (empty) window is restored after each launch."""
    torch = pytest.importorskip("torch")
    data = cfg0_world()
    w = v.World(data.sectors, flags=v.capi.WORLD_L2_PERSIST)
    w.upload(data)
    o = OracleWorld(data.sectors)
    o.upload(data)
    stream = torch.cuda.Stream()
    cam = cfg0_camera(160, 90)
    assert_hits_equal(w.render_view(cam, stream=stream), o.render_view(cam))
    rays = v.random_rays((256, 256, 256), seed=12, n=300_000)  # above the persistent-cast size
    assert_hits_equal(w.cast(rays, stream=stream), o.cast(rays))
    view = v.make_view(cam, shadow_dir=(0.3, 0.8, 0.5))
    got = v.render_path(w, view, stream=stream)
    want = np.stack(o.render_view_shadow(cam, np.array([0.3, 0.8, 0.5], np.float32)))
    for k in range(2):
        assert_hits_equal(got[k], want[k])
    b = v.Batch([w], [view, v.make_view(cam, n_bounces=2)])
    rec = b.run(stream=stream)
    assert_hits_equal(b.view_hits(rec, 0), want)
    assert_hits_equal(b.view_hits(rec, 1), o.render_view_bounces(cam, 2))
    hits = torch.empty(b.total_records * 16, dtype=torch.uint8, device="cuda")
    b.launch(hits, stream, graph=True)
    stream.synchronize()
    assert np.array_equal(hits.cpu().numpy().view(v.HIT_DTYPE), rec)
    b.close()
    with pytest.raises(v.VrtError):
        v.World((1, 1, 1), flags=2)  # unknown flag
    w.close()
    o.close()
