"""The GPU renderer's whole per-pixel path and the G-buffer of the primary hits, on the
device against the oracle.

VoxelRender.comp:51-86 casts per pixel the primary ray, a sun ray from its hit, and up to
u_MaxBounces bounces, each of the first two bounce hits followed by a sun ray; a view
with both a sun direction and bounces asks for exactly that.  The G-buffer
(VoxelRender.comp:39-46,91-93) holds the albedo with the packed normal and the projected
depth of each primary hit.
"""
import numpy as np
import pytest

import voxelrt_gb300 as v
from oracle.oracle import OracleWorld
from tests.helpers import assert_hits_equal, both_worlds, cfg0_camera, cfg0_world, oracle_view

pytestmark = pytest.mark.gpu

SUN = (np.array([0.3, 0.9, -0.28]) / np.linalg.norm([0.3, 0.9, -0.28])).astype(np.float32)  # VoxelRender.comp:53

MODES = [pytest.param(dict(), id="cpu"), pytest.param(dict(glsl=True), id="glsl"),
         pytest.param(dict(glsl=True, aniso=True), id="glsl_aniso")]


@pytest.fixture(scope="module")
def cfg0(gpu):
    data = cfg0_world()
    w, o = both_worlds(data)
    yield data, w, o
    w.close()
    o.close()


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("n_bounces", [1, 2, 4])
def test_renderer_path_per_view(cfg0, mode, n_bounces):
    _, w, o = cfg0
    view = v.make_view(cfg0_camera(160, 90), n_bounces=n_bounces, shadow_dir=SUN, **mode)
    got = v.render_path(w, view)
    want = oracle_view(o, view)
    assert got.shape == want.shape == (2 + n_bounces + min(n_bounces, 2), 160 * 90)
    for k in range(len(want)):
        assert_hits_equal(got[k], want[k])
    # sun rays were cast after bounce hits, and the last bounce plane holds rays
    assert (want[3]["tag"] != v.NO_RAY).any() and (want[-1]["tag"] != v.NO_RAY).any()


@pytest.mark.parametrize("mode", MODES)
def test_renderer_path_in_batches(gpu, mode):
    """Whole-path views among other kinds in one persistent launch (and its graph replay)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(4)
    datas = [v.synth_mix(e, seed=300 + i) for i, e in enumerate((64, 96, 128))]
    worlds, oracles = [], []
    for d in datas:
        w, o = both_worlds(d)
        worlds.append(w)
        oracles.append(o)
    views = []
    for i in range(12):
        edge = datas[i % 3].sectors[0] * 32
        cam = v.look_at(rng.uniform(0, edge, 3), rng.uniform(0, edge, 3) + 0.5, 70.0, *[(64, 48), (96, 54)][i % 2])
        kind = i % 4
        kw = dict(world=i % 3, **mode)
        if kind == 0:
            views.append(v.make_view(cam, n_bounces=int(rng.integers(1, 6)), shadow_dir=SUN, **kw))
        elif kind == 1:
            views.append(v.make_view(cam, shadow_dir=SUN, **kw))
        elif kind == 2:
            views.append(v.make_view(cam, n_bounces=3, **kw))
        else:
            views.append(v.make_view(cam, **kw))
    b = v.Batch(worlds, views)
    want = np.concatenate([oracle_view(oracles[vw.world], vw).reshape(-1) for vw in views])
    assert_hits_equal(b.run(), want)
    hits = torch.empty(b.total_records * 16, dtype=torch.uint8, device="cuda")
    for graph in (False, True):
        hits.fill_(0)
        b.launch(hits, graph=graph)
        torch.cuda.synchronize()
        assert_hits_equal(hits.cpu().numpy().view(v.HIT_DTYPE), want)
    b.close()
    for w in worlds:
        w.close()


def palette(seed=0):
    rng = np.random.default_rng(seed)
    pal = rng.integers(0, 1 << 16, 256, dtype=np.uint32) | rng.integers(0, 1 << 16, 256, dtype=np.uint32) << 16
    pal[0] = 0
    return pal


def projection(near=0.1, far=2000.0, fov=70.0, aspect=16 / 9):
    """A perspective matrix times a view rotation, column-major (glm layout)."""
    f = 1.0 / np.tan(np.radians(fov) / 2)
    p = np.zeros((4, 4))
    p[0, 0], p[1, 1] = f / aspect, f
    p[2, 2], p[2, 3] = (far + near) / (near - far), 2 * far * near / (near - far)
    p[3, 2] = -1.0
    c, s = np.cos(0.3), np.sin(0.3)
    rot = np.array([[c, 0, s, 0], [0, 1, 0, 0], [-s, 0, c, -5.0], [0, 0, 0, 1]])
    return (p @ rot).T.astype(np.float32).reshape(16)  # column-major


@pytest.mark.parametrize("mode", MODES)
def test_gbuffer_matches_oracle(cfg0, mode):
    torch = pytest.importorskip("torch")
    _, w, o = cfg0
    cam = cfg0_camera(200, 120)
    view = v.make_view(cam, **mode)
    pal, proj = palette(1), projection()
    tex, depth = v.render_gbuffer(w, view, pal, proj)
    want_tex, want_depth, want_hits = o.render_gbuffer(cam, pal, proj, **mode)
    assert np.array_equal(tex, want_tex)
    assert np.array_equal(depth.view(np.uint32), want_depth.view(np.uint32))
    hit = want_hits["voxel"] != v.MISS_VOXEL
    assert hit.any() and (~hit).any()
    assert np.all(depth[~hit] == -1.0) and np.all(tex[~hit] == 0x00FFFFFF)
    # the device variant also writes the primary records
    n = cam.width * cam.height
    d_tex = torch.empty(n, dtype=torch.int32, device="cuda")
    d_depth = torch.empty(n, dtype=torch.float32, device="cuda")
    d_hits = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
    pal_c, proj_c = np.ascontiguousarray(pal), np.ascontiguousarray(proj)
    v.check(v.lib().vrt_render_gbuffer_device(w.handle, v.capi.C.byref(view), pal_c.ctypes.data, proj_c.ctypes.data,
                                              d_tex.data_ptr(), d_depth.data_ptr(), d_hits.data_ptr(), None))
    torch.cuda.synchronize()
    assert np.array_equal(d_tex.cpu().numpy().view(np.uint32), want_tex)
    assert_hits_equal(d_hits.cpu().numpy().view(v.HIT_DTYPE), want_hits)


def test_gbuffer_glsl_normal_keeps_every_axis(gpu):
    """A view of a cube's corner in the GLSL mode, where hits near the edges can take a
    normal on several axes (sideMask, VoxelTraversal.glsl:190-192) that the record's face
    cannot carry: the G-buffer is written from the full hit state and equals the oracle's."""
    vol = np.zeros((64, 64, 64), np.uint8)
    vol[:32, :32, :32] = 9
    from tests.helpers import dense_to_stream
    data = dense_to_stream(vol)
    w, o = both_worlds(data)
    cam = v.look_at((60.0, 60.0, 60.0), (31.0, 31.0, 31.0), 40.0, 96, 96)
    view = v.make_view(cam, glsl=True)
    pal, proj = palette(2), projection()
    tex, depth = v.render_gbuffer(w, view, pal, proj)
    want_tex, want_depth, _ = o.render_gbuffer(cam, pal, proj, glsl=True)
    assert np.array_equal(tex, want_tex)
    assert np.array_equal(depth.view(np.uint32), want_depth.view(np.uint32))
    w.close()
    o.close()
