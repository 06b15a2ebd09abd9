"""The device-side brick allocator: edits that allocate and free bricks on the device,
pool compaction (vrt_world_defrag) and growth, against the oracle.

Slot placement is the library's own business (BrickSlotAllocator.cpp:5-94 places
them on the host); what must hold is the reference's logical state - every sector's
mask and bricks - and bit-exact traversal, before and after the pool is compacted.
"""
import numpy as np
import pytest

import voxelrt_gb300 as v
from oracle.oracle import OracleWorld
from tests.helpers import assert_hits_equal
from tests.test_edit_gpu import assert_worlds_equal

pytestmark = pytest.mark.gpu


def surface_edits(rng, w, n, rmax=20):
    """Sphere fills and carves centred on surface voxels found by straight-down casts."""
    edge = w.size[0]
    org = np.stack([rng.uniform(0, edge, 256), np.full(256, w.size[1] - 0.5), rng.uniform(0, edge, 256)], 1)
    rays = np.zeros(256, v.RAY_DTYPE)
    rays["origin"] = org.astype(np.float32)
    rays["dir"] = np.array([1e-4, -1.0, 1e-4], np.float32)
    h = w.cast(rays, max_iters=1000)
    pts = v.unpack_voxel(h["voxel"][h["voxel"] != v.MISS_VOXEL])
    e = np.zeros(n, v.EDIT_DTYPE)
    e["center"] = pts[rng.integers(0, len(pts), n)]
    e["radius"] = rng.integers(2, rmax, n)
    e["material"] = np.where(rng.random(n) < 0.5, 0, rng.integers(1, 256, n))
    return e


def trace_check(w, o, seed):
    rays = v.random_rays(w.size, seed=seed, n=40_000)
    assert_hits_equal(w.cast(rays), o.cast(rays))
    cam = v.look_at((w.size[0] / 2, w.size[1] * 0.9, -20), (w.size[0] / 2, w.size[1] / 3, w.size[2] / 2), 75.0, 160, 90)
    assert_hits_equal(w.render_view(cam), o.render_view(cam))


def test_edits_fragment_then_defrag(gpu):
    rng = np.random.default_rng(3)
    data = v.synth_mix(128, seed=77)
    w = v.World(data.sectors, brick_capacity=data.n_bricks + 8192)
    w.upload(data)
    o = OracleWorld(data.sectors)
    o.upload(data)
    for k in range(60):
        e = surface_edits(rng, w, 1)
        w.edit(e, wait=False)  # queued: no host wait between edits
        o.edit(e)
    frag = w.stats()
    assert_worlds_equal(w, o)
    trace_check(w, o, seed=1)
    # relocated sectors leave gaps behind: more than the one free range at the tail
    assert frag["free_ranges"] > 1
    w.defrag()
    packed = w.stats()
    assert packed["allocated_bricks"] == frag["allocated_bricks"] == o.allocated_bricks()
    assert packed["free_ranges"] == 1 and packed["brick_capacity"] == frag["brick_capacity"]
    assert_worlds_equal(w, o)
    trace_check(w, o, seed=2)
    # and edits keep working on the packed pool
    for k in range(10):
        e = surface_edits(rng, w, 3)
        w.edit(e)
        o.edit(e)
    assert_worlds_equal(w, o)
    trace_check(w, o, seed=3)
    w.close()
    o.close()


def test_full_pool_compacts_and_grows(gpu):
    """A pool with almost no headroom: fills make the edit path compact the pool and then
    grow it, with every result still the oracle's."""
    rng = np.random.default_rng(5)
    data = v.synth_mix(96, seed=12)
    w = v.World(data.sectors, brick_capacity=data.n_bricks + 16)
    w.upload(data)
    o = OracleWorld(data.sectors)
    o.upload(data)
    cap0 = w.stats()["brick_capacity"]
    for k in range(25):
        e = np.zeros(2, v.EDIT_DTYPE)
        e["center"] = rng.integers(0, 96, (2, 3))
        e["radius"] = rng.integers(6, 24, 2)
        e["material"] = [int(rng.integers(1, 256)), 0 if k % 3 == 0 else int(rng.integers(1, 256))]
        w.edit(e)
        o.edit(e)
    assert w.stats()["brick_capacity"] > cap0
    assert_worlds_equal(w, o)
    trace_check(w, o, seed=4)
    w.close()
    o.close()


def test_edit_returns_before_the_device_runs_it(gpu):
    """vrt_world_edit only enqueues: behind a kernel that keeps the stream busy, the call
    returns while the stream is still busy, and the edit lands once the stream runs."""
    torch = pytest.importorskip("torch")
    data = v.synth_mix(64, seed=5)
    # room for every edit below: no compaction, so nothing makes the call wait
    w = v.World(data.sectors, brick_capacity=data.n_bricks + 65536)
    w.upload(data)
    o = OracleWorld(data.sectors)
    o.upload(data)
    rng = np.random.default_rng(9)
    edits = [surface_edits(rng, w, 2) for _ in range(3)]
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        torch.cuda._sleep(200_000_000)  # about 0.1 s of device time on this stream
    for e in edits:
        w.edit(e, stream=stream, wait=False)
    assert not stream.query()  # the edits are queued behind the sleep, not run
    v.check(v.lib().vrt_world_wait(w.handle))
    assert stream.query()
    for e in edits:
        o.edit(e)
    assert_worlds_equal(w, o)
    trace_check(w, o, seed=6)
    w.close()
    o.close()


def test_host_planned_sync_after_device_edits(gpu):
    """Device edits, then a host-planned dirty-brick sync, then more device edits: the host
    mirror is rebuilt from the device before the sync plans, the device's bump pointer
    restarts behind the sync, and the world stays the oracle's throughout."""
    rng = np.random.default_rng(17)
    data = v.synth_mix(96, seed=31)
    w = v.World(data.sectors, brick_capacity=data.n_bricks + 2048)
    w.upload(data)
    o = OracleWorld(data.sectors)
    o.upload(data)
    for _ in range(3):
        for _ in range(4):
            e = surface_edits(rng, w, 2)
            w.edit(e, wait=False)
            o.edit(e)
        # rewrite a few sectors from the host: new masks, some bricks dirty
        k = 5
        pick = rng.choice(len(data.sector_idx), k, replace=False)
        idx = data.sector_idx[pick]
        masks = np.array([int(o.sector_mask(int(i))) for i in idx], np.uint64)
        new_masks = masks.copy()
        dirty = np.zeros(k, np.uint64)
        bricks = []
        for j in range(k):
            m = int(masks[j])
            add = int(rng.integers(0, 1 << 63)) & ~m & int(rng.integers(0, 1 << 63))
            nm = (m & ~(m & int(rng.integers(0, 1 << 63)))) | add
            d = nm & int(rng.integers(0, 1 << 63)) | add
            new_masks[j], dirty[j] = nm, d
            for _ in range(bin(d).count("1")):
                bricks.append((rng.integers(1, 256, 512) * (rng.random(512) < 0.2)).astype(np.uint8))
        b = np.stack(bricks) if bricks else None
        w.sync_sectors(idx, new_masks, b, dirty)
        o.sync_sectors(idx, new_masks, b, dirty)
        assert_worlds_equal(w, o)
    trace_check(w, o, seed=8)
    w.close()
    o.close()


def test_save_after_edits_and_defrag(gpu, tmp_path):
    """A world edited on the device and compacted saves to cvox and loads back equal."""
    rng = np.random.default_rng(23)
    data = v.synth_mix(96, seed=41)
    w = v.World(data.sectors, brick_capacity=data.n_bricks + 1024)
    w.upload(data)
    o = OracleWorld(data.sectors)
    o.upload(data)
    for _ in range(12):
        e = surface_edits(rng, w, 2)
        w.edit(e, wait=False)
        o.edit(e)
    w.defrag(capacity=data.n_bricks * 2)
    st = w.stats()
    assert st["brick_capacity"] >= data.n_bricks * 2 and st["compactions"] >= 1 and st["free_ranges"] == 1
    p = tmp_path / "edited.cvox"
    w.save_cvox(p)
    w2 = v.World(data.sectors)
    w2.load_cvox(p)
    assert_worlds_equal(w2, o)
    trace_check(w2, o, seed=9)
    # an empty world compacts to nothing
    e = v.World((2, 2, 2))
    e.defrag()
    assert e.stats()["allocated_bricks"] == 0
    for x in (w, w2, e):
        x.close()
    o.close()
