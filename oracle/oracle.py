"""ctypes binding of the CPU oracle (oracle/_build/libvrt_oracle.so).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py, as the checker.  The oracle restates the reference CPU
traversal (src/VoxelRT/CpuRenderer.cpp:20-224) as scalar C++; see vrt_oracle.h.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "_build" / "libvrt_oracle.so"

RAY_DTYPE = np.dtype([("origin", "<f4", 3), ("dir", "<f4", 3), ("tag", "<u4"), ("reserved", "<u4")])
HIT_DTYPE = np.dtype([("voxel", "<u4"), ("face", "u1"), ("material", "u1"), ("steps", "<u2"), ("t", "<f4"),
                      ("tag", "<u4")])
PICK_DTYPE = np.dtype([("distance", "<f8"), ("voxel", "<i4", 3), ("normal", "<f4", 3), ("uv", "<f4", 2),
                       ("iters", "<u4"), ("reserved", "<u4")])
EDIT_DTYPE = np.dtype([("center", "<i4", 3), ("radius", "<u4"), ("material", "u1"), ("mode", "u1"),
                       ("reserved", "<u2")])


class Stats(C.Structure):
    _fields_ = [("rays", C.c_uint64), ("step_calls", C.c_uint64), ("occ_fetches", C.c_uint64),
                ("hits", C.c_uint64)]


class _CastParams(C.Structure):
    _fields_ = [("world_origin", C.c_int32 * 3), ("max_iters", C.c_uint32), ("flags", C.c_uint32)]


_vp = C.c_void_p
_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} missing: run `python -m voxelrt_gb300.build`")
        L = C.CDLL(str(LIB_PATH))
        L.ora_world_create.restype = _vp
        L.ora_world_create.argtypes = [C.c_uint32] * 3
        L.ora_world_destroy.argtypes = [_vp]
        L.ora_world_sync.argtypes = [_vp, C.c_uint32, _vp, _vp, _vp, _vp]
        L.ora_world_sector_mask.restype = C.c_uint64
        L.ora_world_sector_mask.argtypes = [_vp, C.c_int32]
        L.ora_world_read_sector.argtypes = [_vp, C.c_int32, _vp, _vp]
        L.ora_world_get_voxel.restype = C.c_uint8
        L.ora_world_get_voxel.argtypes = [_vp, C.c_int32, C.c_int32, C.c_int32]
        L.ora_world_brick_occupancy.argtypes = [_vp, C.c_int32, C.c_int32, C.c_int32, _vp]
        L.ora_world_allocated_bricks.restype = C.c_uint64
        L.ora_world_allocated_bricks.argtypes = [_vp]
        L.ora_cast.argtypes = [_vp, _vp, C.c_uint64, C.POINTER(_CastParams), _vp, C.c_int, C.POINTER(Stats)]
        L.ora_ray_cell_lut.argtypes = [_vp]
        L.ora_camera_rays.argtypes = [_vp, _vp]
        L.ora_render_view.argtypes = [_vp, _vp, C.c_uint32, C.c_uint32, _vp, C.c_int, C.POINTER(Stats)]
        L.ora_render_view_shadow.argtypes = [_vp, _vp, _vp, C.c_uint32, C.c_uint32, _vp, _vp, C.c_int,
                                             C.POINTER(Stats)]
        L.ora_render_view_bounces.argtypes = [_vp, _vp, C.c_uint32, C.c_uint32, C.c_uint32, _vp, C.c_int,
                                              C.POINTER(Stats)]
        L.ora_render_view_path.argtypes = [_vp, _vp, _vp, C.c_uint32, C.c_uint32, C.c_uint32, _vp, C.c_int,
                                           C.POINTER(Stats)]
        L.ora_render_gbuffer.argtypes = [_vp, _vp, C.c_uint32, C.c_uint32, _vp, _vp, _vp, _vp, _vp, C.c_int]
        L.ora_world_edit.argtypes = [_vp, _vp, C.c_uint32]
        L.ora_pick.argtypes = [_vp, _vp, C.c_uint64, C.c_uint32, _vp]
        _lib = L
    return _lib


def _chk(rc: int) -> None:
    if rc != 0:
        raise RuntimeError(f"oracle call failed ({rc})")


def _stats(s: Stats) -> dict:
    return {f: getattr(s, f) for f, _ in s._fields_}


def ray_cell_lut() -> np.ndarray:
    """The oracle's RayCellInteractionMaskLUT: 512 u64 masks, entry idx + octant*64."""
    out = np.zeros(512, np.uint64)
    _chk(lib().ora_ray_cell_lut(out.ctypes.data))
    return out


def _mode(glsl: bool, aniso: bool) -> int:
    """Traversal mode of the render calls: 0 CPU, 1 GLSL, 3 GLSL with anisotropic LODs."""
    return (1 if glsl or aniso else 0) | (2 if aniso else 0)


class OracleWorld:
    def __init__(self, sectors):
        self.sectors = tuple(int(s) for s in sectors)
        h = lib().ora_world_create(*self.sectors)
        if not h:
            raise ValueError("bad world extent")
        self._h = h
        self.last_stats = None

    def close(self):
        if self._h:
            lib().ora_world_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync_sectors(self, sector_idx, alloc_mask, bricks=None, dirty_mask=None):
        si = np.ascontiguousarray(sector_idx, dtype=np.int32)
        am = np.ascontiguousarray(alloc_mask, dtype=np.uint64)
        dm = None if dirty_mask is None else np.ascontiguousarray(dirty_mask, dtype=np.uint64)
        b = None if bricks is None else np.ascontiguousarray(bricks, dtype=np.uint8)
        _chk(lib().ora_world_sync(self._h, len(si), si.ctypes.data, am.ctypes.data,
                                  None if dm is None else dm.ctypes.data, None if b is None else b.ctypes.data))

    def upload(self, data) -> None:
        self.sync_sectors(data.sector_idx, data.alloc_mask, data.bricks)

    def sector_mask(self, idx: int) -> int:
        return lib().ora_world_sector_mask(self._h, int(idx))

    def read_sector(self, idx: int):
        m = C.c_uint64()
        _chk(lib().ora_world_read_sector(self._h, int(idx), C.addressof(m), None))
        bricks = np.zeros((bin(m.value).count("1"), 512), np.uint8)
        _chk(lib().ora_world_read_sector(self._h, int(idx), C.addressof(m), bricks.ctypes.data))
        return m.value, bricks

    def voxel(self, x, y, z) -> int:
        return lib().ora_world_get_voxel(self._h, int(x), int(y), int(z))

    def brick_occupancy(self, bx, by, bz) -> np.ndarray:
        out = np.zeros(8, np.uint64)
        _chk(lib().ora_world_brick_occupancy(self._h, int(bx), int(by), int(bz), out.ctypes.data))
        return out

    def allocated_bricks(self) -> int:
        return lib().ora_world_allocated_bricks(self._h)

    def cast(self, rays, world_origin=(0, 0, 0), max_iters=0, threads=0, glsl=False, coarse=False,
             aniso=False) -> np.ndarray:
        """glsl: the GPU renderer's rayCast (flag VRT_CAST_GLSL) instead of the CPU traversal;
        with coarse its rayCastCoarse (VRT_CAST_GLSL_COARSE), with aniso its anisotropic
        LODs (VRT_CAST_GLSL_ANISO)."""
        rays = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
        hits = np.zeros(len(rays), HIT_DTYPE)
        p = _CastParams((C.c_int32 * 3)(*world_origin), int(max_iters), (1 if glsl else 0) | (2 if coarse else 0) | (4 if aniso else 0))
        s = Stats()
        _chk(lib().ora_cast(self._h, rays.ctypes.data, len(rays), C.byref(p), hits.ctypes.data, int(threads),
                            C.byref(s)))
        self.last_stats = _stats(s)
        return hits

    def render_view(self, cam, max_iters=0, threads=0, glsl=False, aniso=False) -> np.ndarray:
        hits = np.zeros(cam.width * cam.height, HIT_DTYPE)
        s = Stats()
        _chk(lib().ora_render_view(self._h, C.addressof(cam), int(max_iters), _mode(glsl, aniso), hits.ctypes.data,
                                   int(threads), C.byref(s)))
        self.last_stats = _stats(s)
        return hits

    def render_view_shadow(self, cam, sun_dir, max_iters=0, threads=0, glsl=False, aniso=False):
        n = cam.width * cam.height
        prim, shad = np.zeros(n, HIT_DTYPE), np.zeros(n, HIT_DTYPE)
        sd = np.ascontiguousarray(sun_dir, dtype=np.float32)
        s = Stats()
        _chk(lib().ora_render_view_shadow(self._h, C.addressof(cam), sd.ctypes.data, int(max_iters), _mode(glsl, aniso),
                                          prim.ctypes.data, shad.ctypes.data, int(threads), C.byref(s)))
        self.last_stats = _stats(s)
        return prim, shad

    def render_view_bounces(self, cam, n_bounces, max_iters=0, threads=0, glsl=False, aniso=False) -> np.ndarray:
        n = cam.width * cam.height
        hits = np.zeros((n_bounces + 1) * n, HIT_DTYPE)
        s = Stats()
        _chk(lib().ora_render_view_bounces(self._h, C.addressof(cam), int(n_bounces), int(max_iters), _mode(glsl, aniso),
                                           hits.ctypes.data, int(threads), C.byref(s)))
        self.last_stats = _stats(s)
        return hits.reshape(n_bounces + 1, n)

    def render_view_path(self, cam, sun_dir, n_bounces, max_iters=0, threads=0, glsl=False, aniso=False) -> np.ndarray:
        """The GPU renderer's per-pixel path (primary, sun, bounces with a sun ray after the
        first two): (2 + n + min(n, 2), width*height) records."""
        n = cam.width * cam.height
        kinds = 2 + n_bounces + min(n_bounces, 2)
        hits = np.zeros(kinds * n, HIT_DTYPE)
        sd = np.ascontiguousarray(sun_dir, dtype=np.float32)
        s = Stats()
        _chk(lib().ora_render_view_path(self._h, C.addressof(cam), sd.ctypes.data, int(n_bounces), int(max_iters),
                                        _mode(glsl, aniso), hits.ctypes.data, int(threads), C.byref(s)))
        self.last_stats = _stats(s)
        return hits.reshape(kinds, n)

    def render_gbuffer(self, cam, palette, proj, max_iters=0, threads=0, glsl=False, aniso=False):
        """(albedo_normal u32, depth f32, primary records) of a view's primary hits."""
        n = cam.width * cam.height
        pal = np.ascontiguousarray(palette, dtype=np.uint32)
        pm = np.ascontiguousarray(proj, dtype=np.float32).reshape(16)
        tex, dep, hits = np.zeros(n, np.uint32), np.zeros(n, np.float32), np.zeros(n, HIT_DTYPE)
        _chk(lib().ora_render_gbuffer(self._h, C.addressof(cam), int(max_iters), _mode(glsl, aniso), pal.ctypes.data,
                                      pm.ctypes.data, tex.ctypes.data, dep.ctypes.data, hits.ctypes.data, int(threads)))
        return tex, dep, hits

    def pick(self, rays: np.ndarray, max_iters: int = 0) -> np.ndarray:
        """rays: (n, 6) float64 (origin, dir) -> PICK_DTYPE records."""
        r = np.ascontiguousarray(rays, dtype=np.float64).reshape(-1, 6)
        out = np.zeros(len(r), PICK_DTYPE)
        _chk(lib().ora_pick(self._h, r.ctypes.data, len(r), int(max_iters), out.ctypes.data))
        return out

    def edit(self, edits) -> None:
        e = np.ascontiguousarray(edits, dtype=EDIT_DTYPE)
        _chk(lib().ora_world_edit(self._h, e.ctypes.data, len(e)))


def camera_rays(cam) -> np.ndarray:
    rays = np.zeros(cam.width * cam.height, RAY_DTYPE)
    _chk(lib().ora_camera_rays(C.addressof(cam), rays.ctypes.data))
    return rays
