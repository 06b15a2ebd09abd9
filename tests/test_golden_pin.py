"""The oracle (and the device path) against the reference's own RayCast.

tests/golden/refcast.npz holds rays and the outputs of the reference's
CpuRenderer.cpp RayCast, compiled in place from the reference sources and run on
x86-64 by tests/golden/make_golden.py.  Worlds are rebuilt here from their recipe.

Compared on every ray: hit/miss, Distance (bit-exact), face axis and normal sign,
the hit voxel and the material id.  Two reference artefacts of its SIMD lanes
are accounted for, both documented in oracle/vrt_oracle.cpp:
  * a lane that hits on iteration 0 keeps being advanced to origin + 0.001*dir while
    other lanes of its group run (sideDist starts at 0, CpuRenderer.cpp:180,200-201),
    so the reference reports that position; the oracle reports the voxel it tested;
  * with a non-zero world origin, a group whose loop ran out of iterations reads
    materials at relative coordinates (CpuRenderer.cpp:195,210); such groups'
    materials are skipped.
"""
from pathlib import Path

import numpy as np
import pytest

import voxelrt_gb300 as v
from oracle.oracle import OracleWorld
from tests.golden.make_golden import build_world
from tests.helpers import make_rays

FIXTURE = Path(__file__).resolve().parent / "golden" / "refcast.npz"


def load():
    z = np.load(FIXTURE, allow_pickle=False)
    return z, [str(c) for c in z["cases"]]


_Z, _CASES = load()


def check_against_reference(z, case, hits):
    org, d = z[f"{case}/origin"], z[f"{case}/dir"]
    wo = z[f"{case}/world_origin"].astype(np.int64)
    ref_hit = z[f"{case}/hit"].astype(bool)
    ours_hit = hits["voxel"] != v.MISS_VOXEL
    assert np.array_equal(ours_hit, ref_hit), f"{case}: hit mask differs on {np.sum(ours_hit != ref_hit)} rays"
    h = hits[ref_hit]
    dist = z[f"{case}/dist"][ref_hit]
    assert np.array_equal(h["t"].view(np.uint32), dist.view(np.uint32)), f"{case}: Distance not bit-exact"
    nrm = z[f"{case}/normal"][ref_hit].astype(np.int64)
    dh = d[ref_hit]
    axis = np.where(nrm[:, 0] != 0, 0, np.where(nrm[:, 1] != 0, 1, 2))
    assert np.array_equal(h["face"] >> 1, axis), f"{case}: face axis differs"
    sign = np.take_along_axis(np.signbit(dh), axis[:, None], 1)[:, 0]
    assert np.array_equal(np.take_along_axis(nrm, axis[:, None], 1)[:, 0], np.where(sign, 1, -1))
    # hit voxel
    pos = z[f"{case}/pos"][ref_hit]
    ref_vox = np.floor(pos.astype(np.float64)).astype(np.int64) + wo
    ours_vox = v.unpack_voxel(h["voxel"])
    first = h["steps"] == 0
    assert np.array_equal(ours_vox[~first], ref_vox[~first]), f"{case}: hit voxel differs"
    o = org[ref_hit][first]
    moved = (o + np.float32(0.001) * dh[first]).astype(np.float32)
    same_or_moved = (pos[first] == o).all(1) | (pos[first] == moved).all(1)
    assert same_or_moved.all()
    assert np.array_equal(ours_vox[first], np.floor(o.astype(np.float64)).astype(np.int64) + wo)
    # material, skipping groups whose loop ran out with a non-zero world origin
    lanes = int(_Z["lanes"][0])
    mat = z[f"{case}/material"][ref_hit]
    ok = np.ones(int(ref_hit.sum()), bool)
    if (wo != 0).any():
        exhausted = hits["steps"] >= v.capi.DEFAULT_MAX_ITERS
        grp = np.zeros((len(hits) + lanes - 1) // lanes, bool)
        np.logical_or.at(grp, np.arange(len(hits)) // lanes, exhausted)
        ok = ~grp[np.nonzero(ref_hit)[0] // lanes]
    ok &= ~first
    assert np.array_equal(h["material"][ok], mat[ok]), f"{case}: material differs"


@pytest.fixture(scope="module")
def oracle_worlds():
    view = tuple(int(c) for c in _Z["view_sectors"])
    cache = {}
    for case in _CASES:
        name = str(_Z[f"{case}/world"])
        if name not in cache:
            o = OracleWorld(view)
            o.upload(build_world(name))
            cache[name] = o
    return cache


@pytest.mark.parametrize("case", _CASES)
def test_oracle_matches_reference(oracle_worlds, case):
    z = _Z
    rays = make_rays(z[f"{case}/origin"], z[f"{case}/dir"])
    o = oracle_worlds[str(z[f"{case}/world"])]
    hits = o.cast(rays, world_origin=tuple(int(c) for c in z[f"{case}/world_origin"]), max_iters=128)
    check_against_reference(z, case, hits)


@pytest.mark.gpu
@pytest.mark.parametrize("case", _CASES)
def test_device_matches_reference(gpu, case):
    z = _Z
    view = tuple(int(c) for c in z["view_sectors"])
    with v.World(view) as w:
        w.upload(build_world(str(z[f"{case}/world"])))
        rays = make_rays(z[f"{case}/origin"], z[f"{case}/dir"])
        hits = w.cast(rays, world_origin=tuple(int(c) for c in z[f"{case}/world_origin"]), max_iters=128)
    check_against_reference(z, case, hits)


PICK_FIXTURE = Path(__file__).resolve().parent / "golden" / "refpick.npz"
_P = np.load(PICK_FIXTURE, allow_pickle=False)
_PICK_WORLDS = [str(w) for w in _P["worlds"]]


def check_pick(z, world, got):
    """VoxelMap::RayCast outputs: Distance, VoxelPos, Normal, UV, bit-exact."""
    dist = z[f"{world}/distance"]
    assert np.array_equal(got["distance"].view(np.uint64), dist.view(np.uint64)), f"{world}: distance"
    hit = dist > 0
    assert np.array_equal(got["voxel"][hit], z[f"{world}/voxel"][hit]), f"{world}: voxel"
    assert np.array_equal(got["normal"][hit].view(np.uint32), z[f"{world}/normal"][hit].view(np.uint32))
    assert np.array_equal(got["uv"][hit].view(np.uint32), z[f"{world}/uv"][hit].view(np.uint32))
    assert hit.mean() > 0.5


@pytest.mark.parametrize("world", _PICK_WORLDS)
def test_oracle_pick_matches_reference(world):
    o = OracleWorld(tuple(int(c) for c in _P["view_sectors"]))
    o.upload(build_world(world))
    check_pick(_P, world, o.pick(_P[f"{world}/rays"], 1024))


@pytest.mark.gpu
@pytest.mark.parametrize("world", _PICK_WORLDS)
def test_device_pick_matches_reference(gpu, world):
    with v.World(tuple(int(c) for c in _P["view_sectors"])) as w:
        w.upload(build_world(world))
        check_pick(_P, world, w.pick(_P[f"{world}/rays"], 1024))
