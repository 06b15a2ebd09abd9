"""Request server: continuous batching, edits between frames, HBM admission, in both
scheduling modes (a launch per batch of queued requests, and one resident launch that
takes requests while it runs).

The key property: a request's records are the same whether it runs alone or inside
a mix of concurrent requests (bit-exact, t within 1e-6 relative), and they equal
the oracle replaying the same request log.
"""
import threading

import numpy as np
import pytest

import voxelrt_gb300 as v
from oracle.oracle import OracleWorld
from tests.helpers import assert_hits_equal, oracle_view

pytestmark = pytest.mark.gpu


def make_worlds(n=4, seed=0):
    rng = np.random.default_rng(seed)
    datas = [v.synth_mix(int(rng.choice([64, 96, 128])), seed=500 + i) for i in range(n)]
    worlds = []
    for d in datas:
        w = v.World(d.sectors)
        w.upload(d)
        worlds.append(w)
    return datas, worlds


def random_view(rng, world, edge, res=None):
    w, h = res or [(64, 64), (96, 54), (160, 90), (33, 17)][int(rng.integers(0, 4))]
    cam = v.look_at(rng.uniform(0, edge, 3), rng.uniform(0, edge, 3) + 0.5, float(rng.uniform(50, 90)), w, h)
    kind = int(rng.integers(0, 4))
    if kind == 1:
        return v.make_view(cam, world=world, shadow_dir=(0.3, 0.8, 0.5))
    if kind == 2:
        return v.make_view(cam, world=world, n_bounces=2)
    if kind == 3:  # the GPU renderer's whole path: sun rays among the bounces
        return v.make_view(cam, world=world, n_bounces=3, shadow_dir=(0.3, 0.8, 0.5))
    return v.make_view(cam, world=world)


def oracle_records(o: OracleWorld, view) -> np.ndarray:
    return oracle_view(o, view).reshape(-1)


@pytest.fixture(scope="module")
def setup(gpu):
    datas, worlds = make_worlds()
    oracles = []
    for d in datas:
        o = OracleWorld(d.sectors)
        o.upload(d)
        oracles.append(o)
    yield datas, worlds, oracles
    for w in worlds:
        w.close()


MODES = [pytest.param(False, id="launches"), pytest.param(True, id="resident")]


@pytest.mark.parametrize("resident", MODES)
def test_alone_equals_mix_equals_oracle(setup, resident):
    datas, worlds, oracles = setup
    rng = np.random.default_rng(1)
    srv = v.Server(worlds, max_inflight=3, resident=resident)
    views = [random_view(rng, i % 4, datas[i % 4].sectors[0] * 32) for i in range(40)]
    probe = views[7]
    # alone
    alone = v.PinnedHits(v.view_records(probe))
    srv.wait(srv.submit_render(probe, alone.array))
    # in a mix submitted from several threads at once
    outs = [v.PinnedHits(v.view_records(vw)) for vw in views]
    tickets = [None] * len(views)

    def submit(idx):
        for i in idx:
            tickets[i] = srv.submit_render(views[i], outs[i].array)

    ths = [threading.Thread(target=submit, args=(list(range(k, len(views), 4)),)) for k in range(4)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    infos = [srv.wait(t) for t in tickets]
    if not resident:  # a resident launch takes each request as soon as it is submitted
        assert max(i["batch_size"] for i in infos) > 1  # requests were batched together
    assert np.array_equal(outs[7].array.view(np.uint8), alone.array.view(np.uint8))
    for i, vw in enumerate(views):
        assert_hits_equal(outs[i].array, oracle_records(oracles[vw.world], vw))
    st = srv.stats()
    assert st["renders_done"] == len(views) + 1 and st["p99_us"] >= st["p50_us"] > 0
    srv.close()


@pytest.mark.parametrize("resident", MODES)
def test_edits_apply_between_frames_in_order(gpu, resident):
    datas, worlds = make_worlds(2, seed=3)
    oracles = []
    for d in datas:
        o = OracleWorld(d.sectors)
        o.upload(d)
        oracles.append(o)
    rng = np.random.default_rng(2)
    srv = v.Server(worlds, max_inflight=2, resident=resident)
    log = []  # replayed on the oracle in submission order
    outs = []
    for step in range(30):
        if step % 5 == 4:
            e = np.zeros(2, v.EDIT_DTYPE)
            edge = datas[0].sectors[0] * 32
            e["center"] = rng.integers(0, edge, (2, 3))
            e["radius"] = rng.integers(4, 20, 2)
            e["material"] = [0, int(rng.integers(1, 256))]
            srv.submit_edit(0, e)
            log.append(("edit", 0, e))
        else:
            vw = random_view(rng, int(rng.integers(0, 2)), datas[0].sectors[0] * 32)
            out = v.PinnedHits(v.view_records(vw))
            t = srv.submit_render(vw, out.array)
            outs.append((t, out))
            log.append(("render", vw, out))
    srv.drain()
    for entry in log:
        if entry[0] == "edit":
            oracles[entry[1]].edit(entry[2])
        else:
            vw, out = entry[1], entry[2]
            assert_hits_equal(out.array, oracle_records(oracles[vw.world], vw))
    assert srv.stats()["edits_done"] == 6
    srv.close()
    for w in worlds:
        w.close()


@pytest.mark.parametrize("resident", MODES)
def test_admission_by_budget(setup, resident):
    datas, worlds, oracles = setup
    rng = np.random.default_rng(4)
    # budget of 4 pages (256 KiB): one 160x90 request needs 225 KiB
    srv = v.Server(worlds, max_inflight=2, hbm_budget_bytes=4 * 65536, resident=resident)
    views = [random_view(rng, 0, 64, res=(160, 90)) for _ in range(6)]
    views = [v.make_view(vw.cam, world=0) for vw in views]
    outs = [v.PinnedHits(v.view_records(vw)) for vw in views]
    ts = [srv.submit_render(vw, o.array) for vw, o in zip(views, outs)]
    infos = [srv.wait(t) for t in ts]
    assert all(i["batch_size"] == 1 for i in infos)  # one fits at a time
    for vw, o in zip(views, outs):
        assert_hits_equal(o.array, oracle_records(oracles[0], vw))
    big = v.make_view(v.look_at((1, 1, 1), (9, 9, 9), 60.0, 512, 512), world=0)
    with pytest.raises(v.VrtError) as ei:
        srv.submit_render(big, np.zeros(512 * 512, v.HIT_DTYPE))
    assert ei.value.status == v.capi.VRT_ERR_OUT_OF_MEMORY
    assert srv.stats()["rejected"] == 1
    srv.close()


def test_wait_timeout_and_unknown_ticket(setup):
    _, worlds, _ = setup
    srv = v.Server(worlds)
    with pytest.raises(v.VrtError) as ei:
        srv.wait(12345, timeout_ms=1)
    assert ei.value.status == v.capi.VRT_ERR_NOT_FOUND
    srv.close()


def test_resident_mode_switches_and_idle_restart(setup):
    """Requests in another traversal mode (GLSL, GLSL with anisotropic LODs) close the
    running launch and start one in their mode; an idle launch closes itself and the next request starts a new one."""
    import time
    datas, worlds, oracles = setup
    rng = np.random.default_rng(6)
    srv = v.Server(worlds, resident=True, idle_us=200)
    views = []
    modes = (0, v.VIEW_GLSL, v.VIEW_GLSL | v.capi.VIEW_GLSL_ANISO, 0)
    for i in range(24):
        vw = random_view(rng, i % 4, datas[i % 4].sectors[0] * 32)
        vw.flags |= modes[i // 6]
        views.append(vw)
    outs = [v.PinnedHits(v.view_records(vw)) for vw in views]
    ts = [srv.submit_render(vw, o.array) for vw, o in zip(views, outs)]
    for t in ts:
        srv.wait(t)
    time.sleep(0.05)  # the launch has been idle for well over 200 us: it ends
    late = v.make_view(views[0].cam, world=views[0].world)
    lo = v.PinnedHits(v.view_records(late))
    srv.wait(srv.submit_render(late, lo.array))
    for vw, o in zip(views, outs):
        assert_hits_equal(o.array, oracle_view(oracles[vw.world], vw).reshape(-1))
    assert_hits_equal(lo.array, oracle_records(oracles[late.world], late))
    assert srv.stats()["launches"] >= 5  # 4 modes in turn, then a restart after the idle end
    srv.close()


def test_default_mode_and_mode_flags(setup):
    """With no mode flag the server runs resident on a device with host-native atomics
    (GB300), and launch mode when asked; asking for both modes is refused."""
    import ctypes as C

    from voxelrt_gb300 import capi
    datas, worlds, oracles = setup
    srv = v.Server(worlds)
    assert srv.stats()["resident"] == 1
    vw = random_view(np.random.default_rng(8), 0, datas[0].sectors[0] * 32)
    out = v.PinnedHits(v.view_records(vw))
    srv.wait(srv.submit_render(vw, out.array))
    srv.close()
    srv = v.Server(worlds, resident=False)
    assert srv.stats()["resident"] == 0
    srv.close()
    cfg = capi.ServerConfig(2, 0, 0, v.BatchConfig(), capi.SERVE_RESIDENT | capi.SERVE_LAUNCHES, 0)
    wh = (C.c_void_p * len(worlds))(*[w.handle.value for w in worlds])
    h = C.c_void_p()
    assert capi.lib().vrt_server_create(wh, len(worlds), C.byref(cfg), C.byref(h)) == capi.VRT_ERR_INVALID_ARG


@pytest.mark.parametrize("resident", MODES)
def test_concurrent_1080p_renders_with_edits(gpu, resident):
    """Four 1080p renders in flight at once with sphere edits submitted between them: every
    render equals the oracle replaying the submission log (edits in order)."""
    rng = np.random.default_rng(21)
    datas = [v.synth_mix(edge, seed=800 + i) for i, edge in enumerate((128, 192))]
    worlds, oracles = [], []
    for d in datas:
        w = v.World(d.sectors, brick_capacity=d.n_bricks + 4096)
        w.upload(d)
        worlds.append(w)
        o = OracleWorld(d.sectors)
        o.upload(d)
        oracles.append(o)
    srv = v.Server(worlds, max_inflight=3, resident=resident)
    log, outs, tickets = [], [], []
    for k in range(10):
        wi = k % 2
        edge = datas[wi].sectors[0] * 32
        if k in (2, 5, 7):
            e = np.zeros(2, v.EDIT_DTYPE)
            e["center"] = rng.integers(edge // 4, 3 * edge // 4, (2, 3))
            e["radius"] = rng.integers(4, 20, 2)
            e["material"] = [0, int(rng.integers(1, 256))]
            tickets.append(srv.submit_edit(wi, e))
            log.append(("edit", wi, e))
            continue
        cam = v.look_at(rng.uniform(0, edge, 3), rng.uniform(0, edge, 3) + 0.5, 80.0, 1920, 1080)
        vw = v.make_view(cam, world=wi) if k % 3 else v.make_view(cam, world=wi, shadow_dir=(0.3, 0.8, 0.5))
        out = v.PinnedHits(v.view_records(vw))
        outs.append(out)
        tickets.append(srv.submit_render(vw, out.array))
        log.append(("render", wi, (vw, out)))
    infos = [srv.wait(t, timeout_ms=120000) for t in tickets]
    assert all(i["state"] == v.capi.REQ_DONE for i in infos)
    renders = 0
    for kind, wi, item in log:
        if kind == "edit":
            oracles[wi].edit(item)
        else:
            vw, out = item
            assert_hits_equal(out.array, oracle_records(oracles[wi], vw))
            renders += 1
    assert renders == 7
    srv.close()
    for w in worlds:
        w.close()
