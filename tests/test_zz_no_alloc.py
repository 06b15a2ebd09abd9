"""vrt_render_views_static: the batched traversal without device allocations.

Callers that cannot allocate device memory once their frame loop runs use this
entry point; its launch scratch is a fixed device array inside the library.  Its
records must equal the CPU oracle's and those of vrt_batch (the allocating entry
point) on the same worlds and views, on calls in a row (each call reuses the array
the last one left behind), in the default traversal and in the GLSL mode with
anisotropic LODs.  Neither the device's free memory nor torch's allocator may move
across the calls.  This file is collected last so that a failure here leaves every
other test already run.
"""
import ctypes as C

import numpy as np
import pytest

import voxelrt_gb300 as v
from oracle.oracle import OracleWorld
from tests.helpers import assert_hits_equal, oracle_view

pytestmark = pytest.mark.gpu


def call_static(worlds, views, out_ptr, cfg=None, stream=None):
    wh = (C.c_void_p * len(worlds))(*[w.handle.value for w in worlds])
    va = (v.View * len(views))(*views)
    return v.lib().vrt_render_views_static(wh, len(worlds), va, len(views),
                                           C.byref(cfg) if cfg is not None else None, out_ptr, stream)


def seeded_views(worlds, rng, n, glsl=False, aniso=False):
    views = []
    for i in range(n):
        edge = worlds[i % len(worlds)].size[0]
        cam = v.look_at(rng.uniform(0, edge, 3), rng.uniform(0, edge, 3) + 0.5, 70.0,
                        *[(64, 64), (70, 37), (96, 54)][i % 3])
        kw = dict(world=i % len(worlds), glsl=glsl, aniso=aniso)
        if i % 4 == 1:
            views.append(v.make_view(cam, shadow_dir=(0.3, 0.8, 0.5), **kw))
        elif i % 4 == 2:
            views.append(v.make_view(cam, n_bounces=2, **kw))
        elif i % 8 == 7:  # the GPU renderer's whole path: sun rays among the bounces
            views.append(v.make_view(cam, n_bounces=3, shadow_dir=(0.3, 0.8, 0.5), **kw))
        else:
            views.append(v.make_view(cam, **kw))
    return views


def oracle_records(oracles, views):
    return np.concatenate([oracle_view(oracles[vw.world], vw).reshape(-1) for vw in views])


@pytest.fixture(scope="module")
def scene(gpu):
    rng = np.random.default_rng(11)
    datas = [v.synth_mix(int(rng.choice([64, 96])), seed=900 + i) for i in range(3)]
    worlds, oracles = [], []
    for d in datas:
        w = v.World(d.sectors)
        w.upload(d)
        worlds.append(w)
        o = OracleWorld(d.sectors)
        o.upload(d)
        oracles.append(o)
    yield worlds, oracles, rng
    for w in worlds:
        w.close()
    for o in oracles:
        o.close()


def device_memory(torch):
    free, _ = torch.cuda.mem_get_info()
    return free, torch.cuda.memory_allocated(), torch.cuda.memory_reserved()


def test_static_scratch_matches_oracle_and_batch(scene):
    torch = pytest.importorskip("torch")
    worlds, oracles, rng = scene
    sets = [seeded_views(worlds, rng, 12), seeded_views(worlds, rng, 9, glsl=True, aniso=True)]
    wants = [oracle_records(oracles, vs) for vs in sets]
    for vs, want in zip(sets, wants):
        assert_hits_equal(v.Batch(worlds, vs).run(), want)
    outs = [torch.empty(len(w) * 16, dtype=torch.uint8, device="cuda") for w in wants]
    # the first call of each mode loads that kernel's module, and the first fill loads
    # torch's fill kernel (modules load lazily, at first use); the device memory that
    # takes is in place before the checked calls below
    for vs, out in zip(sets, outs):
        out.fill_(0xAB)
        v.check(call_static(worlds, vs, out.data_ptr()))
    torch.cuda.synchronize()
    before = device_memory(torch)
    for call in range(2):
        for vs, want, out in zip(sets, wants, outs):
            out.fill_(0xAB)
            torch.cuda.synchronize()
            v.check(call_static(worlds, vs, out.data_ptr()))
            torch.cuda.synchronize()
            assert_hits_equal(out.cpu().numpy().view(v.HIT_DTYPE), want)
    assert device_memory(torch) == before


def test_back_to_back_calls_on_one_stream(scene):
    """Two calls queued on one stream with different views and no host wait between them:
    each call's tables reach the device intact, and each record buffer holds its own
    views' records."""
    torch = pytest.importorskip("torch")
    worlds, oracles, rng = scene
    a, b = seeded_views(worlds, rng, 10), seeded_views(worlds, rng, 7)
    want_a, want_b = oracle_records(oracles, a), oracle_records(oracles, b)
    out_a = torch.empty(len(want_a) * 16, dtype=torch.uint8, device="cuda")
    out_b = torch.empty(len(want_b) * 16, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    for _ in range(2):
        out_a.fill_(0xAB)
        out_b.fill_(0xCD)
        torch.cuda.synchronize()
        v.check(call_static(worlds, a, out_a.data_ptr(), stream=stream.cuda_stream))
        v.check(call_static(worlds, b, out_b.data_ptr(), stream=stream.cuda_stream))
        stream.synchronize()
        assert_hits_equal(out_a.cpu().numpy().view(v.HIT_DTYPE), want_a)
        assert_hits_equal(out_b.cpu().numpy().view(v.HIT_DTYPE), want_b)


def test_refusals(scene):
    """Beyond the fixed maximum the call is refused before anything runs."""
    torch = pytest.importorskip("torch")
    worlds, _, rng = scene
    views = seeded_views(worlds, rng, 2)
    out = torch.empty(1 << 20, dtype=torch.uint8, device="cuda")
    st = call_static(worlds, [views[0]] * 1025, out.data_ptr())
    assert st == v.capi.VRT_ERR_INVALID_ARG
    assert b"1024 views" in v.lib().vrt_last_error()
    st = call_static([worlds[0]] * 257, views, out.data_ptr())
    assert st == v.capi.VRT_ERR_INVALID_ARG
    assert b"256 worlds" in v.lib().vrt_last_error()
