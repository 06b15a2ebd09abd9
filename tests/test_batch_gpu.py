"""Paths (shadow rays, diffuse bounces) and the batched persistent kernel vs the oracle.

Every record of every view is compared bit-exactly (t within 1e-6 relative) with
the CPU oracle, for the plain per-view launch, the persistent launch under each
tile shape / refill setting, and the CUDA-graph replay.
"""
import numpy as np
import pytest

import voxelrt_gb300 as v
from oracle.oracle import OracleWorld
from tests.helpers import assert_hits_equal, both_worlds, cfg0_camera, cfg0_world, oracle_view

pytestmark = pytest.mark.gpu

SUN = np.array([0.3, 0.8, 0.5]) / np.linalg.norm([0.3, 0.8, 0.5])


def torch_or_skip():
    return pytest.importorskip("torch")


@pytest.fixture(scope="module")
def cfg0(gpu):
    data = cfg0_world()
    w, o = both_worlds(data)
    yield data, w, o
    w.close()


def test_shadow_path_matches_oracle(cfg0):
    _, w, o = cfg0
    cam = cfg0_camera(320, 180)
    view = v.make_view(cam, shadow_dir=SUN.astype(np.float32))
    got = v.render_path(w, view)
    prim, shad = o.render_view_shadow(cam, SUN.astype(np.float32))
    assert_hits_equal(got[0], prim)
    assert_hits_equal(got[1], shad)
    assert (shad["tag"] != v.NO_RAY).sum() == (prim["voxel"] != v.MISS_VOXEL).sum()


@pytest.mark.parametrize("n_bounces", [1, 4])
def test_bounce_path_matches_oracle(cfg0, n_bounces):
    _, w, o = cfg0
    cam = cfg0_camera(200, 120)
    view = v.make_view(cam, n_bounces=n_bounces)
    got = v.render_path(w, view)
    want = o.render_view_bounces(cam, n_bounces)
    for k in range(n_bounces + 1):
        assert_hits_equal(got[k], want[k])
    assert (want[n_bounces]["tag"] != v.NO_RAY).any()


def mix_batch_setup(n_worlds=5, seed=0):
    rng = np.random.default_rng(seed)
    datas, worlds, oracles, views = [], [], [], []
    for i in range(n_worlds):
        edge = int(rng.choice([64, 96, 128]))
        d = v.synth_mix(edge, seed=100 + i)
        datas.append(d)
        w, o = both_worlds(d)
        worlds.append(w)
        oracles.append(o)
        for _ in range(int(rng.integers(1, 4))):
            res = [(64, 64), (70, 37), (96, 54), (33, 65)][int(rng.integers(0, 4))]
            pos = rng.uniform(0, edge, 3)
            tgt = rng.uniform(0, edge, 3)
            cam = v.look_at(pos, tgt, float(rng.uniform(50, 90)), *res)
            kind = int(rng.integers(0, 3))
            if kind == 0:
                views.append(v.make_view(cam, world=i))
            elif kind == 1:
                views.append(v.make_view(cam, world=i, shadow_dir=SUN))
            else:
                views.append(v.make_view(cam, world=i, n_bounces=2, max_iters=64))
    return worlds, oracles, views


@pytest.fixture(scope="module")
def mix(gpu):
    worlds, oracles, views = mix_batch_setup()
    want = [oracle_view(oracles[vw.world], vw) for vw in views]
    yield worlds, views, want
    for w in worlds:
        w.close()


CONFIGS = [
    dict(),
    dict(tile_w=8, tile_h=8, morton=1, refill_threshold=32, inner_iters=1),
    dict(tile_w=16, tile_h=4, refill_threshold=1, inner_iters=8, chunk_tiles=1),
    dict(tile_w=32, tile_h=1, warps_per_block=8, refill_threshold=24, chunk_tiles=5, blocks_per_sm=1),
    # the GB300 table's camera-workload shapes: rounds long enough to trace every ray to its end
    dict(refill_threshold=28, chunk_tiles=16, inner_iters=128),
    dict(warps_per_block=2, refill_threshold=1, chunk_tiles=4, inner_iters=128),
    # chunk size picked per launch, for a grid of one block per SM
    dict(blocks_per_sm=1, inner_iters=64),
]


@pytest.mark.parametrize("cfg", CONFIGS)
def test_batch_matches_oracle(mix, cfg):
    worlds, views, want = mix
    bc = v.BatchConfig(**{k: cfg.get(k, 0) for k in ("tile_w", "tile_h", "morton", "warps_per_block",
                                                       "blocks_per_sm", "refill_threshold", "chunk_tiles",
                                                       "inner_iters")})
    b = v.Batch(worlds, views, bc)
    hits = b.run()
    for i in range(len(views)):
        got = b.view_hits(hits, i)
        assert got.shape == want[i].shape
        for k in range(got.shape[0]):
            assert_hits_equal(got[k], want[i][k])
    cast = sum(int((w["tag"] != v.NO_RAY).sum()) for w in want)
    assert b.stats()["rays_cast"] == cast
    b.close()


def test_batch_launch_modes_agree(mix):
    torch = torch_or_skip()
    worlds, views, want = mix
    b = v.Batch(worlds, views)
    n = b.total_records
    outs = []
    for mode in ("launch", "graph", "graph", "per_view"):
        t = torch.zeros(n * 16, dtype=torch.uint8, device="cuda")
        if mode == "per_view":
            b.launch_per_view(t)
        else:
            b.launch(t, graph=(mode == "graph"))
        torch.cuda.synchronize()
        outs.append(t.cpu().numpy().view(v.HIT_DTYPE))
    for o in outs[1:]:
        assert np.array_equal(o.view(np.uint8), outs[0].view(np.uint8))
    st = b.measure(torch.zeros(n * 16, dtype=torch.uint8, device="cuda"))
    assert st["rays_cast"] == b.stats()["rays_cast"]
    assert st["step_calls"] > 0 and st["hits"] <= st["rays_cast"]
    b.close()


def test_batch_rejects_bad_input(mix):
    worlds, views, _ = mix
    bad = v.make_view(cfg0_camera(8, 8), world=len(worlds))
    with pytest.raises(v.VrtError):
        v.Batch(worlds, [bad])
    with pytest.raises(v.VrtError):
        v.Batch(worlds, views, v.BatchConfig(tile_w=4, tile_h=4))
    too_many = v.make_view(cfg0_camera(8, 8), n_bounces=16, shadow_dir=SUN)
    with pytest.raises(v.VrtError):
        v.Batch(worlds, [too_many])
    # camera updates keep each view's resolution and a world origin within +-2^30
    b = v.Batch(worlds, views)
    cams = [v.Camera.from_buffer_copy(vw.cam) for vw in views]
    cams[0].width += 1
    with pytest.raises(v.VrtError):
        b.update_cameras(cams)
    cams = [v.Camera.from_buffer_copy(vw.cam) for vw in views]
    cams[-1].world_origin[1] = (1 << 30) + 1
    with pytest.raises(v.VrtError):
        b.update_cameras(cams)
    b.close()


def test_run_into_pinned_buffers_matches_pageable(mix):
    """vrt_batch_run copies the records of each finished part of the batch while later
    parts trace; into vrt_host_alloc memory (also at an offset inside a larger
    allocation) or pageable memory, the records are the same."""
    worlds, views, want = mix
    b = v.Batch(worlds, views)
    n = b.total_records
    pageable = b.run()
    whole = v.PinnedHits(n)
    whole.array[:] = np.frombuffer(b"\xab" * (n * 16), v.HIT_DTYPE)
    got_whole = b.run(whole.array).copy()
    bigger = v.PinnedHits(n + 100)
    got_inner = b.run(bigger.array[37:37 + n]).copy()
    for got in (got_whole, got_inner):
        assert np.array_equal(got.view(np.uint8), pageable.view(np.uint8))
    for i in range(len(views)):
        g = b.view_hits(got_whole, i)
        for k in range(g.shape[0]):
            assert_hits_equal(g[k], want[i][k])
    b.close()
    whole.close()
    bigger.close()


def test_run_packed_is_run_without_tags(mix):
    """vrt_batch_run_packed delivers every record of vrt_batch_run without its tag (12 bytes),
    with the records of rays never cast marked PACKED_NO_RAY; into pageable memory, and into
    vrt_host_alloc memory at an offset that is not 16-byte aligned."""
    worlds, views, want = mix
    b = v.Batch(worlds, views)
    n = b.total_records
    full = b.run()
    assert (full["tag"] == v.NO_RAY).any() and (full["tag"] != v.NO_RAY).any()
    expect = v.pack_hits(full)
    pageable = b.run_packed()
    pinned = v.PinnedHits(n + 5, dtype=v.PACKED_DTYPE)
    pinned.array[:] = np.frombuffer(b"\xcd" * ((n + 5) * 12), v.PACKED_DTYPE)
    got_pinned = b.run_packed(pinned.array[3:3 + n]).copy()
    assert np.array_equal(pinned.array[:3].view(np.uint8), np.full(36, 0xCD, np.uint8))
    for got in (pageable, got_pinned):
        assert np.array_equal(got.view(np.uint8), expect.view(np.uint8))
    # against the oracle: a record's position in its view gives the pixel its tag named
    for i in range(len(views)):
        a, e = int(b.offsets[i]), int(b.offsets[i + 1])
        g = pageable[a:e]
        w = v.pack_hits(want[i].reshape(-1))
        for f in ("voxel", "face", "material", "steps"):
            assert np.array_equal(g[f], w[f]), f"view {i}: {f} differs"
        tg, tw = g["t"].astype(np.float64), w["t"].astype(np.float64)
        fin = np.isfinite(tw)
        assert np.array_equal(np.isfinite(tg), fin)
        assert np.all(np.abs(tg[fin] - tw[fin]) <= 1e-6 * np.abs(tw[fin]))
    pinned.close()
    b.close()
