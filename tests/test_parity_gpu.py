"""Device traversal vs the CPU oracle, bit-exact on every ray (t within 1e-6 relative).

Cases follow the edge cases a brickmap DDA has: empty space, single voxels,
axis-aligned and +-0 direction components (NaN side distances), rays starting
inside solid voxels or outside the grid, non-zero world origins, iteration caps.
"""
import numpy as np
import pytest

import voxelrt_gb300 as v
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
