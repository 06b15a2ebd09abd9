"""vrt_render_views_static: the batched traversal without device allocations.

Callers that cannot allocate device memory once their frame loop runs use this
entry point; its launch scratch is a fixed device array inside the library.  Its
records must equal those of vrt_batch (the allocating entry point) on the same
worlds and views, on two calls in a row (the second call reuses the array the
first one left behind).  This file is collected last so that a failure here
leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

import voxelrt_gb300 as v
from tests.helpers import assert_hits_equal

pytestmark = pytest.mark.gpu


def call_static(worlds, views, out_ptr, cfg=None, stream=None):
    wh = (C.c_void_p * len(worlds))(*[w.handle.value for w in worlds])
    va = (v.View * len(views))(*views)
    return v.lib().vrt_render_views_static(wh, len(worlds), va, len(views),
                                           C.byref(cfg) if cfg is not None else None, out_ptr, stream)


def test_static_scratch_matches_batch(gpu):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    worlds = []
    for i in range(3):
        d = v.synth_mix(int(rng.choice([64, 96])), seed=900 + i)
        w = v.World(d.sectors)
        w.upload(d)
        worlds.append(w)
    views = []
    for i in range(12):
        edge = worlds[i % 3].size[0]
        cam = v.look_at(rng.uniform(0, edge, 3), rng.uniform(0, edge, 3) + 0.5, 70.0,
                        *[(64, 64), (70, 37), (96, 54)][i % 3])
        if i % 4 == 1:
            views.append(v.make_view(cam, world=i % 3, shadow_dir=(0.3, 0.8, 0.5)))
        elif i % 4 == 2:
            views.append(v.make_view(cam, world=i % 3, n_bounces=2))
        else:
            views.append(v.make_view(cam, world=i % 3))
    want = v.Batch(worlds, views).run()
    out = torch.empty(len(want) * 16, dtype=torch.uint8, device="cuda")
    for call in range(2):
        out.fill_(0xAB)
        torch.cuda.synchronize()
        v.check(call_static(worlds, views, out.data_ptr()))
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(v.HIT_DTYPE)
        assert_hits_equal(got, want)
    # beyond the fixed maximum the call is refused before anything runs
    many = [views[0]] * 1025
    st = call_static(worlds, many, out.data_ptr())
    assert st == v.capi.VRT_ERR_INVALID_ARG
    assert b"1024 views" in v.lib().vrt_last_error()
    for w in worlds:
        w.close()
