"""The GLSL traversal mode (oracle and device) against the reference's own shaders.

tests/golden/refglsl.npz holds rays and the outputs of VoxelTraversal.glsl's rayCast
and rayCastCoarse, with and without anisotropic LODs, compiled as C++ from the
reference's shader source and run by tests/golden/make_golden_glsl.py.  Worlds are
rebuilt here from their recipe.

Compared on every ray: hit or miss; the iteration count where the shader sets it
(hits and exits; a ray whose iteration cap ran out leaves it unset in the shader and
reports the cap here); on hits the distance (bit-exact), the material and, except for
rayCastCoarse's coarse hits (the shader reports the stepped-to position, the material
comes from the cell's first solid voxel), the hit voxel; the face from the shader's
normal where no direction component is zero.  A view per world adds the renderer's
shadow ray (VoxelRender.comp:56): the records of render paths against the shader's
rayCast plus rayCastCoarse(hit.pos + hit.normal*0.01, sun).
"""
from pathlib import Path

import numpy as np
import pytest

import voxelrt_gb300 as v
from oracle.oracle import OracleWorld
from tests.golden.make_golden_glsl import MODES, glsl_world
from tests.helpers import both_worlds, dense_to_stream, make_rays

FIXTURE = Path(__file__).resolve().parent / "golden" / "refglsl.npz"
_Z = np.load(FIXTURE, allow_pickle=False)
WORLDS = [str(s) for s in _Z["worlds"]]


def world_data(spec: str):
    kind, seed = spec.split(":")
    return dense_to_stream(glsl_world(kind, int(seed)))


def check(cast, wi: int) -> int:
    """Runs every ray set and mode of world wi through cast(rays, wo, cap, coarse,
    aniso) and compares; returns the number of records compared."""
    n_checked = 0
    si = 0
    while f"{wi}/{si}/origin" in _Z:
        org, d, wo = _Z[f"{wi}/{si}/origin"], _Z[f"{wi}/{si}/dir"], _Z[f"{wi}/{si}/wo"]
        rays = make_rays(org, d)
        for coarse, aniso in MODES:
            m = f"{wi}/{si}/{int(coarse)}{int(aniso)}"
            cap = 96 if coarse else 256  # VRT_GLSL_COARSE_MAX_ITERS, VRT_GLSL_MAX_ITERS
            got = cast(rays, tuple(int(c) for c in wo), cap, coarse, aniso)
            hit, dist, iters, mat = _Z[f"{m}/hit"] != 0, _Z[f"{m}/dist"], _Z[f"{m}/iters"], _Z[f"{m}/mat"]
            where = f"world {wi} set {si} coarse={coarse} aniso={aniso}"
            ghit = got["voxel"] != v.MISS_VOXEL
            bad = np.nonzero(ghit != hit)[0]
            assert bad.size == 0, f"{where}: hit/miss differs on {bad.size} rays, first {bad[:5]}"
            set_ = iters != 0xFFFFFFFF
            assert np.array_equal(got["steps"][set_], iters[set_]), f"{where}: iterations"
            assert (got["steps"][~set_] == cap).all() and not ghit[~set_].any(), f"{where}: capped rays"
            assert np.array_equal(got["t"][hit].view(np.uint32), dist[hit].view(np.uint32)), f"{where}: dist"
            assert np.array_equal(got["material"][hit], mat[hit]), f"{where}: material"
            fine = hit & ~(coarse & (iters > 30) & set_)
            want_vox = np.floor(_Z[f"{m}/pos"][fine].astype(np.float64)).astype(np.int64) + wo.astype(np.int64)
            got_vox = np.asarray(v.unpack_voxel(got["voxel"][fine]), np.int64).reshape(-1, 3)
            assert np.array_equal(got_vox, want_vox), f"{where}: hit voxel"
            nz = hit & (d != 0).all(axis=1)
            nrm = _Z[f"{m}/normal"][nz]
            axis = np.argmax(nrm != 0, axis=1)
            face = axis * 2 + (nrm[np.arange(len(nrm)), axis] > 0)
            assert np.array_equal(got["face"][nz].astype(np.int64), face), f"{where}: face"
            n_checked += len(rays)
        si += 1
    return n_checked


@pytest.mark.parametrize("wi", range(len(WORLDS)))
def test_oracle_matches_shader(wi):
    data = world_data(WORLDS[wi])
    o = OracleWorld(data.sectors)
    o.upload(data)
    n = check(lambda r, wo, cap, c, a: o.cast(r, world_origin=wo, max_iters=cap, glsl=True, coarse=c, aniso=a), wi)
    assert n > 10_000


@pytest.mark.gpu
@pytest.mark.parametrize("wi", range(len(WORLDS)))
def test_device_matches_shader(gpu, wi):
    data = world_data(WORLDS[wi])
    w, _ = both_worlds(data)
    try:
        check(lambda r, wo, cap, c, a: w.cast(r, world_origin=wo, max_iters=cap, glsl=True, coarse=c, aniso=a), wi)
    finally:
        w.close()


def check_view(render, wi: int) -> None:
    """Primary and shadow records of world wi's view against the shader's rayCast and
    its shadow ray (VoxelRender.comp:56), with and without anisotropic LODs; render(view)
    returns (primary, shadow) records."""
    from oracle.oracle import camera_rays
    cam = v.Camera.from_buffer_copy(_Z[f"{wi}/cam"].tobytes())
    sun = _Z["sun"]
    cr = camera_rays(cam)
    wo = np.array(cam.world_origin[:], np.int64)
    for aniso in (False, True):
        m = f"{wi}/view/{int(aniso)}"
        prim, shad = render(v.make_view(cam, shadow_dir=sun, glsl=True, aniso=aniso))
        where = f"world {wi} view aniso={aniso}"
        hit, iters = _Z[f"{m}/hit"] != 0, _Z[f"{m}/iters"]
        assert np.array_equal(prim["voxel"] != v.MISS_VOXEL, hit), f"{where}: primary hit/miss"
        set_ = iters != 0xFFFFFFFF
        assert np.array_equal(prim["steps"][set_], iters[set_]), f"{where}: primary iterations"
        assert np.array_equal(prim["t"][hit].view(np.uint32), _Z[f"{m}/dist"][hit].view(np.uint32)), where
        assert np.array_equal(prim["material"][hit], _Z[f"{m}/mat"][hit]), f"{where}: primary material"
        want_vox = np.floor(_Z[f"{m}/pos"][hit].astype(np.float64)).astype(np.int64) + wo
        got_vox = np.asarray(v.unpack_voxel(prim["voxel"][hit]), np.int64).reshape(-1, 3)
        assert np.array_equal(got_vox, want_vox), f"{where}: primary voxel"
        nz = hit & (cr["dir"] != 0).all(axis=1)
        nrm = _Z[f"{m}/normal"][nz]
        axis = np.argmax(nrm != 0, axis=1)
        assert np.array_equal(prim["face"][nz].astype(np.int64), axis * 2 + (nrm[np.arange(len(nrm)), axis] > 0))
        # shadow rays: cast exactly where the primary ray hit
        s_hit, s_iters = _Z[f"{m}/s_hit"], _Z[f"{m}/s_iters"]
        assert np.array_equal(shad["tag"] == v.NO_RAY, s_hit == 2), f"{where}: shadow rays cast"
        cast = s_hit != 2
        sh = s_hit == 1
        assert np.array_equal(shad["voxel"][cast] != v.MISS_VOXEL, sh[cast]), f"{where}: shadow hit/miss"
        sset = cast & (s_iters != 0xFFFFFFFF)
        assert np.array_equal(shad["steps"][sset], s_iters[sset]), f"{where}: shadow iterations"
        assert np.array_equal(shad["t"][sh].view(np.uint32), _Z[f"{m}/s_dist"][sh].view(np.uint32)), where
        assert np.array_equal(shad["material"][sh], _Z[f"{m}/s_mat"][sh]), f"{where}: shadow material"
        assert hit.sum() > 100 and sh.sum() > 10 and (cast & ~sh).sum() > 10, f"{where}: too few cases"


@pytest.mark.parametrize("wi", range(len(WORLDS)))
def test_oracle_view_shadow_matches_shader(wi):
    data = world_data(WORLDS[wi])
    o = OracleWorld(data.sectors)
    o.upload(data)
    check_view(lambda vw: o.render_view_shadow(vw.cam, np.array(vw.sun_dir[:], np.float32), glsl=True,
                                               aniso=bool(vw.flags & v.capi.VIEW_GLSL_ANISO)), wi)


@pytest.mark.gpu
@pytest.mark.parametrize("wi", range(len(WORLDS)))
def test_device_view_shadow_matches_shader(gpu, wi):
    data = world_data(WORLDS[wi])
    w, _ = both_worlds(data)
    try:
        check_view(lambda vw: tuple(v.render_path(w, vw)), wi)
    finally:
        w.close()
