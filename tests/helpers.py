"""Seeded worlds, cameras and comparison helpers shared by the tests."""
from __future__ import annotations

import numpy as np

import voxelrt_gb300 as v
from oracle.oracle import OracleWorld

CFG0_TERRAIN = dict(size=(256, 256, 256), base=96, amplitude=48, seed=1)


def cfg0_world() -> v.SectorData:
    """256^3 heightfield y < 96 + 48*fbm(x/128, z/128), seed 1; material 1 + min(3, y/32)."""
    return v.synth_terrain(**CFG0_TERRAIN)


def cfg0_camera(width=640, height=360):
    return v.look_at((128, 200, -40), (128, 80, 128), 90.0, width, height)


def both_worlds(data: v.SectorData):
    w = v.World(data.sectors)
    w.upload(data)
    o = OracleWorld(data.sectors)
    o.upload(data)
    return w, o


def assert_hits_equal(got: np.ndarray, want: np.ndarray, rtol_t: float = 1e-6) -> None:
    """Integer fields bit-exact; t within rtol_t relative (inf == inf)."""
    assert got.shape == want.shape
    for f in ("voxel", "face", "material", "steps", "tag"):
        bad = np.nonzero(got[f] != want[f])[0]
        assert bad.size == 0, f"{f} differs on {bad.size} rays, first {bad[:5]}: got {got[bad[:5]]} want {want[bad[:5]]}"
    tg, tw = got["t"].astype(np.float64), want["t"].astype(np.float64)
    fin = np.isfinite(tw)
    assert np.array_equal(np.isfinite(tg), fin)
    assert np.array_equal(tg[~fin], tw[~fin])
    np.testing.assert_allclose(tg[fin], tw[fin], rtol=rtol_t, atol=0)


def single_voxel_world(pos, material=7, sectors=(2, 2, 2)) -> v.SectorData:
    x, y, z = pos
    sx, sy, sz = x >> 5, y >> 5, z >> 5
    b = ((x >> 3) & 3) | ((z >> 3) & 3) << 2 | ((y >> 3) & 3) << 4
    brick = np.zeros(512, np.uint8)
    brick[(x & 7) | (z & 7) << 3 | (y & 7) << 6] = material
    idx = np.array([v.sector_index(sx, sy, sz)], np.int32)
    return v.SectorData(sectors, idx, np.array([1 << b], np.uint64), brick[None])


def dense_to_stream(vol: np.ndarray) -> v.SectorData:
    """(Y, Z, X) u8 volume with extents multiple of 32 -> sector stream of non-empty bricks."""
    Y, Z, X = vol.shape
    sectors = (X // 32, Y // 32, Z // 32)
    idx, masks, bricks = [], [], []
    for sy in range(sectors[1]):
        for sz in range(sectors[2]):
            for sx in range(sectors[0]):
                m = 0
                for b in range(64):
                    bx, bz, by = b & 3, (b >> 2) & 3, b >> 4
                    y0, z0, x0 = sy * 32 + by * 8, sz * 32 + bz * 8, sx * 32 + bx * 8
                    blk = vol[y0:y0 + 8, z0:z0 + 8, x0:x0 + 8]
                    if blk.any():
                        m |= 1 << b
                        bricks.append(blk.reshape(-1).copy())
                if m:
                    idx.append(v.sector_index(sx, sy, sz))
                    masks.append(m)
    b = np.stack(bricks) if bricks else np.zeros((0, 512), np.uint8)
    return v.SectorData(sectors, np.array(idx, np.int32), np.array(masks, np.uint64), b)


def make_rays(origins, dirs, tags=None) -> np.ndarray:
    origins = np.asarray(origins, np.float32).reshape(-1, 3)
    dirs = np.asarray(dirs, np.float32).reshape(-1, 3)
    r = np.zeros(len(origins), v.RAY_DTYPE)
    r["origin"] = origins
    r["dir"] = dirs
    r["tag"] = np.arange(len(r)) if tags is None else tags
    return r


def oracle_view(o: OracleWorld, view) -> np.ndarray:
    """All records of a vrt_view from the oracle, shaped (kinds, width*height)."""
    glsl = bool(view.flags & v.VIEW_GLSL)
    aniso = bool(view.flags & v.capi.VIEW_GLSL_ANISO)
    if view.flags & v.VIEW_SHADOW and view.n_bounces:
        return o.render_view_path(view.cam, np.array(view.sun_dir[:], np.float32), view.n_bounces, view.max_iters,
                                  glsl=glsl, aniso=aniso)
    if view.flags & v.VIEW_SHADOW:
        p, s = o.render_view_shadow(view.cam, np.array(view.sun_dir[:], np.float32), view.max_iters, glsl=glsl,
                                    aniso=aniso)
        return np.stack([p, s])
    if view.n_bounces:
        return o.render_view_bounces(view.cam, view.n_bounces, view.max_iters, glsl=glsl, aniso=aniso)
    return o.render_view(view.cam, view.max_iters, glsl=glsl, aniso=aniso)[None]


def cell_corner_world(shape=(32, 32, 128), material=7) -> v.SectorData:
    """(Y, Z, X) world with one solid voxel at offset (3, 3, 3) of every 4^3 cell: every
    brick is allocated, every cell non-empty, every 2^3 block at the cell origin empty."""
    vol = np.zeros(shape, np.uint8)
    vol[3::4, 3::4, 3::4] = material
    return dense_to_stream(vol)
