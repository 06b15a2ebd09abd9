"""Parity at the full sizes of the benchmark workloads (GPU): every record of every view
(and every one of the 2^26 stress rays) against the CPU oracle.

On top of that, size-independent checks: the batched persistent launch and the
one-launch-per-view kernel give identical bytes, a second launch repeats them exactly,
and the record invariants hold (a secondary record is NO_RAY exactly where the path
ended before it, hits lie inside their world with a non-zero material and a finite t,
misses carry the sentinel, step counts respect the cap, primary tags are pixel indices).
"""
import numpy as np
import pytest

import voxelrt_gb300 as v
from oracle.oracle import OracleWorld
from tests.helpers import assert_hits_equal, oracle_view
from voxelrt_gb300 import autotune
from voxelrt_gb300 import workloads as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def eff_iters(m: int, glsl: bool = False) -> int:
    """The iteration cap a view runs with (0 = 128, or 256 in the GLSL mode; at most 65535)."""
    return (256 if glsl else 128) if m == 0 else min(m, 65535)


def load(wl):
    worlds = []
    for d in wl.worlds:
        w = v.World(d.sectors, brick_capacity=d.n_bricks + 64)
        w.upload(d)
        worlds.append(w)
    return worlds


def launch_both(wl, worlds):
    """Batched and per-view records (device tensors); asserts they are identical and repeat."""
    cfg, _ = autotune.lookup(wl.name)
    b = v.Batch(worlds, wl.views, cfg)
    n = b.total_records
    batched = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
    other = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
    b.launch(batched, graph=True)
    b.launch_per_view(other)
    torch.cuda.synchronize()
    assert torch.equal(batched, other), "persistent launch and per-view launches differ"
    b.launch(other, graph=True)
    torch.cuda.synchronize()
    assert torch.equal(batched, other), "a second launch differs from the first"
    del other
    return b, batched


def check_invariants(b, rec, wl):
    r = rec.view(torch.int32).view(-1, 4)
    voxel, w1, t, tag = r[:, 0], r[:, 1], r[:, 2].view(torch.float32), r[:, 3]
    face, mat, steps = w1 & 0xFF, (w1 >> 8) & 0xFF, (w1 >> 16) & 0xFFFF
    miss = voxel == -1
    hit = ~miss
    assert bool((face[miss] == 0xFF).all() and (mat[miss] == 0).all() and torch.isposinf(t[miss]).all())
    assert bool((face[hit] < 6).all() and (mat[hit] != 0).all() and torch.isfinite(t[hit]).all())
    offsets = b.offsets
    for i, vw in enumerate(wl.views):
        a, e = int(offsets[i]), int(offsets[i + 1])
        npx = vw.cam.width * vw.cam.height
        kinds = (e - a) // npx
        size = wl.worlds[vw.world].sectors
        rv = r[a:e].view(kinds, npx, 4)
        vv = rv[..., 0]
        h = vv != -1
        assert bool(((vv & 0x7FF) < size[0] * 32)[h].all() and (((vv >> 11) & 0x3FF) < size[1] * 32)[h].all()
                    and (((vv >> 21) & 0x7FF) < size[2] * 32)[h].all()), f"view {i}: hit outside its world"
        cap = eff_iters(vw.max_iters, bool(vw.flags & v.VIEW_GLSL))
        assert bool((((rv[..., 1] >> 16) & 0xFFFF) <= cap).all()), f"view {i}: steps"
        assert bool((rv[0, :, 3] == torch.arange(npx, device=rv.device, dtype=torch.int32)).all())
        for k in range(1, kinds):
            ended = (rv[k - 1, :, 0] == -1) | (rv[k - 1, :, 3] == -1)
            assert bool(torch.equal(rv[k, :, 3] == -1, ended)), f"view {i}: record {k} NO_RAY mismatch"


def check_oracle_all(b, rec, wl):
    """Every view against the oracle (on all host cores), views taken in batch order so each
    world is uploaded to the oracle once."""
    host = rec.cpu().numpy().view(v.HIT_DTYPE)
    oracles = {}
    records = 0
    for i, vw in enumerate(wl.views):
        if vw.world not in oracles:
            for o in oracles.values():
                o.close()
            o = OracleWorld(wl.worlds[vw.world].sectors)
            o.upload(wl.worlds[vw.world])
            oracles = {vw.world: o}
        want = oracle_view(oracles[vw.world], vw)
        a, e = int(b.offsets[i]), int(b.offsets[i + 1])
        got = host[a:e].reshape(want.shape)
        for k in range(want.shape[0]):
            assert_hits_equal(got[k], want[k])
        records += want.size
    for o in oracles.values():
        o.close()
    assert records == b.total_records


def run_config(wl):
    worlds = load(wl)
    b, rec = launch_both(wl, worlds)
    check_invariants(b, rec, wl)
    check_oracle_all(b, rec, wl)
    b.close()
    for w in worlds:
        w.close()


def test_uneven_batch_full_size(gpu):
    """128 worlds, 1,119 views, 352.9 M records, every one against the oracle."""
    run_config(W.uneven_batch())


@pytest.mark.parametrize("aniso", [False, True])
def test_uneven_batch_full_size_glsl_modes(gpu, aniso):
    """The same batch in the GLSL traversal mode, with and without anisotropic LODs:
    batched equals per-view, the invariants hold, every record equals the oracle's."""
    wl = W.uneven_batch()
    for vw in wl.views:
        vw.flags |= v.VIEW_GLSL | (v.capi.VIEW_GLSL_ANISO if aniso else 0)
    run_config(wl)


def test_large_world_full_size(gpu):
    """2048x256x2048 world, 64 views at 1920x1080 with shadow rays (265 M records), every one
    against the oracle."""
    run_config(W.large_world())


def test_incoherent_full_size_and_stress_rays(gpu):
    """1024^3 world: 1280x720 with 4 diffuse bounces against the oracle, and all 2^26 random
    rays cast on the device against the oracle."""
    wl = W.incoherent()
    run_config(wl)
    d = wl.worlds[0]
    w = v.World(d.sectors, brick_capacity=d.n_bricks + 64)
    w.upload(d)
    size = [s * 32 for s in d.sectors]
    n = 1 << 26
    rays = v.random_rays(size, seed=9, n=n)
    dr = torch.from_numpy(rays.view(np.uint8)).cuda()
    hits = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
    w.cast_device(dr, n, hits)
    again = torch.empty_like(hits)
    w.cast_device(dr, n, again)
    torch.cuda.synchronize()
    assert torch.equal(hits, again)
    del again
    host = hits.cpu().numpy().view(v.HIT_DTYPE)
    o = OracleWorld(d.sectors)
    o.upload(d)
    block = 1 << 23
    for first in range(0, n, block):
        assert_hits_equal(host[first:first + block], o.cast(rays[first:first + block]))
    o.close()
    w.close()
