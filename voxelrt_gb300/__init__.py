"""GB300 brickmap ray traversal: Python handle over libvrt.so.

The library (C ABI in include/vrt.h) owns the device-resident brickmap and runs the
sm_103a kernels; this module only converts numpy arrays and torch tensors into
pointers.  It mirrors the reference's storage boundary:

* ``World.sync_sectors`` is ``GpuVoxelStorage::SyncBuffers(VoxelMap&)``
  (src/VoxelRT/GpuRenderer.cpp:45-167) fed with DirtyLocs-shaped records;
* ``World.render_view`` is one ``GpuRenderer::RenderFrame`` traversal dispatch
  (GpuRenderer.cpp:239-273) writing hit records;
* ``World.cast`` traverses explicit rays.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import (CAST_GLSL, EDIT_DTYPE, HIT_DTYPE, MISS_FACE, MISS_VOXEL, NO_RAY, PACKED_DTYPE, PACKED_NO_RAY,
                   RAY_DTYPE, VIEW_GLSL, VIEW_SHADOW, BatchConfig, Camera,
                   CastParams, View, VrtError, check, check_synth, lib, ptr, synth_lib)

__all__ = ["Server", "PinnedHits", "view_records", "render_path", "render_gbuffer", "cvox_read", "cvox_write", "World", "Camera", "View",
           "make_view", "Batch", "BatchConfig", "VIEW_SHADOW", "VIEW_GLSL", "CAST_GLSL", "look_at", "synth_terrain", "synth_mix", "random_rays", "SectorData", "VrtError",
           "RAY_DTYPE", "HIT_DTYPE", "EDIT_DTYPE", "MISS_VOXEL", "MISS_FACE", "NO_RAY", "unpack_voxel", "sector_index",
           "PACKED_DTYPE", "PACKED_NO_RAY", "pack_hits", "lib"]


def pack_hits(hits: np.ndarray) -> np.ndarray:
    """The 12-byte records (vrt_hit_packed) of 16-byte ones: the tag dropped, and a record of a
    ray never cast (tag NO_RAY) marked with material PACKED_NO_RAY."""
    out = np.empty(len(hits), PACKED_DTYPE)
    for f in PACKED_DTYPE.names:
        out[f] = hits[f]
    out["material"][hits["tag"] == NO_RAY] = PACKED_NO_RAY
    return out


def sector_index(x: int, y: int, z: int) -> int:
    """WorldSectorIndexer packing (VoxelMap.h:100): x | z<<12 | y<<24 in 12/12/8-bit
    fields, as a signed 32-bit value (vrt_sector_index computes the same)."""
    u = (x & 4095) | (z & 4095) << 12 | (y & 255) << 24
    return u - (1 << 32) if u >= (1 << 31) else u


def unpack_voxel(v: np.ndarray) -> np.ndarray:
    """Packed x | y<<11 | z<<21 hit voxels -> (n, 3) int array (misses give 2047/1023/2047)."""
    v = np.asarray(v, dtype=np.uint32)
    return np.stack([v & 0x7FF, (v >> 11) & 0x3FF, v >> 21], axis=-1).astype(np.int64)


def look_at(pos, target, vfov_deg: float, width: int, height: int) -> Camera:
    """vrt_camera_look_at, from the host-only input library (the same code as libvrt.so's)."""
    cam = Camera()
    p = (C.c_double * 3)(*map(float, pos))
    t = (C.c_double * 3)(*map(float, target))
    check_synth(synth_lib().vrt_camera_look_at(p, t, float(vfov_deg), int(width), int(height), C.byref(cam)))
    return cam


class SectorData:
    """A sector stream in host memory: records (sector_idx, alloc_mask) + packed bricks."""

    def __init__(self, sectors, sector_idx, alloc_mask, bricks, owner=None):
        self.sectors = tuple(int(s) for s in sectors)
        self.sector_idx = np.ascontiguousarray(sector_idx, dtype=np.int32)
        self.alloc_mask = np.ascontiguousarray(alloc_mask, dtype=np.uint64)
        self.bricks = np.ascontiguousarray(bricks, dtype=np.uint8).reshape(-1, 512)
        self._owner = owner

    @property
    def n_bricks(self) -> int:
        return self.bricks.shape[0]

    @classmethod
    def _from_native(cls, sp, owner=None) -> "SectorData":
        """Copy a native sector stream; `owner` is the library that made it (it frees it)."""
        s = sp.contents
        n, nb = s.n_sectors, s.n_bricks
        idx = np.ctypeslib.as_array(s.sector_idx, shape=(max(n, 1),))[:n].copy()
        mask = np.ctypeslib.as_array(s.alloc_mask, shape=(max(n, 1),))[:n].copy()
        bricks = np.ctypeslib.as_array(s.bricks, shape=(max(nb, 1) * 512,))[: nb * 512].copy()
        sectors = (s.sectors_x, s.sectors_y, s.sectors_z)
        (owner or lib()).vrt_sector_stream_free(sp)
        return cls(sectors, idx, mask, bricks)

    def dense(self) -> np.ndarray:
        """Dense (Y, Z, X) voxel volume (tests and small worlds only)."""
        sx, sy, sz = self.sectors
        vol = np.zeros((sy * 32, sz * 32, sx * 32), np.uint8)
        k = 0
        for idx, m in zip(self.sector_idx.tolist(), self.alloc_mask.tolist()):
            x, z, y = idx & 4095, (idx >> 12) & 4095, (idx >> 24) & 255
            for b in range(64):
                if (m >> b) & 1:
                    bx, bz, by = b & 3, (b >> 2) & 3, b >> 4
                    brick = self.bricks[k].reshape(8, 8, 8)  # (y, z, x)
                    y0, z0, x0 = y * 32 + by * 8, z * 32 + bz * 8, x * 32 + bx * 8
                    vol[y0:y0 + 8, z0:z0 + 8, x0:x0 + 8] = brick
                    k += 1
        return vol


def synth_terrain(size, base, amplitude, seed, scale=128.0, octaves=4, cave_octaves=0, cave_scale=64.0,
                  cave_threshold=0.35, cave_seed=0, threads=0) -> SectorData:
    d = _terrain_desc(size, base, amplitude, seed, scale, octaves, cave_octaves, cave_scale, cave_threshold, cave_seed)
    out = C.POINTER(capi.SectorStream)()
    check_synth(synth_lib().vrt_synth_terrain_world(C.byref(d), int(threads), C.byref(out)))
    return SectorData._from_native(out, synth_lib())


def terrain_height(x, z, size, base, amplitude, seed, scale=128.0, octaves=4) -> float:
    d = _terrain_desc(size, base, amplitude, seed, scale, octaves, 0, 64.0, 0.35, 0)
    return synth_lib().vrt_synth_terrain_height(C.byref(d), float(x), float(z))


def _terrain_desc(size, base, amplitude, seed, scale, octaves, cave_octaves, cave_scale, cave_threshold, cave_seed):
    d = capi.SynthTerrain()
    d.size[:] = [int(v) for v in size]
    d.base, d.amplitude, d.scale = float(base), float(amplitude), float(scale)
    d.octaves, d.seed = int(octaves), int(seed)
    d.cave_octaves, d.cave_scale, d.cave_threshold, d.cave_seed = (int(cave_octaves), float(cave_scale),
                                                                    float(cave_threshold), int(cave_seed))
    return d


def cvox_write(path, data: SectorData) -> None:
    """Write a cvox v4 world file (VoxelMap::Serialize format)."""
    check(lib().vrt_cvox_write(str(path).encode(), len(data.sector_idx), ptr(data.sector_idx), ptr(data.alloc_mask),
                               ptr(data.bricks)))


def cvox_read(path) -> SectorData:
    """Read a cvox v4 world file (VoxelMap::Deserialize format)."""
    out = C.POINTER(capi.SectorStream)()
    check(lib().vrt_cvox_read(str(path).encode(), C.byref(out)))
    return SectorData._from_native(out)


def synth_mix(edge: int, seed: int, threads: int = 0) -> SectorData:
    out = C.POINTER(capi.SectorStream)()
    check_synth(synth_lib().vrt_synth_mix_world(int(edge), int(seed), int(threads), C.byref(out)))
    return SectorData._from_native(out, synth_lib())


def random_rays(size, seed: int, n: int, first: int = 0, threads: int = 0) -> np.ndarray:
    rays = np.zeros(n, RAY_DTYPE)
    s = (C.c_uint32 * 3)(*[int(v) for v in size])
    check_synth(synth_lib().vrt_synth_random_rays(s, int(seed), int(first), int(n), int(threads), rays.ctypes.data))
    return rays


def cast_flags(glsl: bool, coarse: bool, aniso: bool = False) -> int:
    return ((CAST_GLSL if glsl or coarse or aniso else 0) | (capi.CAST_GLSL_COARSE if coarse else 0) |
            (capi.CAST_GLSL_ANISO if aniso else 0))


def _stream_ptr(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream  # torch.cuda.Stream


class World:
    """A device-resident brickmap (vrt_world)."""

    def __init__(self, sectors, brick_capacity: int = 0, device: int = 0, flags: int = 0):
        d = capi.WorldDesc(int(sectors[0]), int(sectors[1]), int(sectors[2]), int(brick_capacity), int(device),
                           int(flags))
        h = C.c_void_p()
        check(lib().vrt_world_create(C.byref(d), C.byref(h)))
        self._h = h
        self.sectors = tuple(int(s) for s in sectors)
        self.size = tuple(32 * s for s in self.sectors)

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def close(self) -> None:
        if self._h:
            lib().vrt_world_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def stats(self) -> dict:
        s = capi.WorldStats()
        check(lib().vrt_world_get_stats(self._h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def sync_sectors(self, sector_idx, alloc_mask, bricks=None, dirty_mask=None, stream=None) -> None:
        sector_idx = np.ascontiguousarray(sector_idx, dtype=np.int32)
        alloc_mask = np.ascontiguousarray(alloc_mask, dtype=np.uint64)
        dirty = None if dirty_mask is None else np.ascontiguousarray(dirty_mask, dtype=np.uint64)
        b = None if bricks is None else np.ascontiguousarray(bricks, dtype=np.uint8)
        check(lib().vrt_world_sync_sectors(self._h, len(sector_idx), ptr(sector_idx), ptr(alloc_mask), ptr(dirty),
                                           ptr(b), _stream_ptr(stream)))

    def upload(self, data: SectorData, stream=None) -> None:
        self.sync_sectors(data.sector_idx, data.alloc_mask, data.bricks, None, stream)

    def pick(self, rays, max_iters: int = 0, stream=None) -> np.ndarray:
        """Picking ray cast (VoxelMap::RayCast): rays (n, 6) float64 origin+dir -> PICK_DTYPE records."""
        r = np.ascontiguousarray(rays, dtype=np.float64).reshape(-1, 6)
        out = np.zeros(len(r), capi.PICK_DTYPE)
        check(lib().vrt_pick(self._h, ptr(r), len(r), int(max_iters), ptr(out), _stream_ptr(stream)))
        return out

    def edit(self, edits, stream=None, wait: bool = True) -> None:
        """Apply vrt_edit records (EDIT_DTYPE array) in order, on the device; with `wait`
        (the default) return once the device has applied them (vrt_world_wait)."""
        e = np.ascontiguousarray(edits, dtype=EDIT_DTYPE)
        check(lib().vrt_world_edit(self._h, ptr(e), len(e), _stream_ptr(stream)))
        if wait:
            check(lib().vrt_world_wait(self._h))

    def defrag(self, capacity: int = 0, stream=None) -> None:
        """Pack the live bricks from slot 0 (vrt_world_defrag); capacity 0 keeps the pool size."""
        check(lib().vrt_world_defrag(self._h, int(capacity), _stream_ptr(stream)))

    def save_cvox(self, path) -> None:
        check(lib().vrt_world_save_cvox(self._h, str(path).encode()))

    def load_cvox(self, path, stream=None) -> None:
        check(lib().vrt_world_load_cvox(self._h, str(path).encode(), _stream_ptr(stream)))

    def read_sector(self, sector_idx: int):
        mask = C.c_uint64()
        check(lib().vrt_world_read_sector(self._h, int(sector_idx), C.byref(mask), None, 0, None))
        n = bin(mask.value).count("1")
        bricks = np.zeros((n, 512), np.uint8)
        check(lib().vrt_world_read_sector(self._h, int(sector_idx), C.byref(mask), ptr(bricks), bricks.nbytes, None))
        return mask.value, bricks

    def cast(self, rays: np.ndarray, world_origin=(0, 0, 0), max_iters: int = 0, stream=None,
             glsl: bool = False, coarse: bool = False, aniso: bool = False) -> np.ndarray:
        """glsl: the GPU renderer's rayCast (VRT_CAST_GLSL) instead of the CPU traversal;
        coarse: its rayCastCoarse (VRT_CAST_GLSL_COARSE); aniso: its anisotropic LODs
        (VRT_CAST_GLSL_ANISO)."""
        rays = np.ascontiguousarray(rays, dtype=RAY_DTYPE)
        hits = np.zeros(len(rays), HIT_DTYPE)
        p = CastParams((C.c_int32 * 3)(*world_origin), int(max_iters), cast_flags(glsl, coarse, aniso))
        check(lib().vrt_cast(self._h, ptr(rays), len(rays), C.byref(p), ptr(hits), _stream_ptr(stream)))
        return hits

    def cast_device(self, rays, n: int, hits, world_origin=(0, 0, 0), max_iters: int = 0, stream=None,
                    glsl: bool = False, coarse: bool = False, aniso: bool = False) -> None:
        p = CastParams((C.c_int32 * 3)(*world_origin), int(max_iters), cast_flags(glsl, coarse, aniso))
        check(lib().vrt_cast_device(self._h, ptr(rays), int(n), C.byref(p), ptr(hits), _stream_ptr(stream)))

    def render_view(self, cam: Camera, max_iters: int = 0, stream=None) -> np.ndarray:
        hits = np.zeros(cam.width * cam.height, HIT_DTYPE)
        check(lib().vrt_render_view(self._h, C.byref(cam), int(max_iters), ptr(hits), _stream_ptr(stream)))
        return hits

    def render_view_device(self, cam: Camera, hits, max_iters: int = 0, stream=None) -> None:
        check(lib().vrt_render_view_device(self._h, C.byref(cam), int(max_iters), ptr(hits), _stream_ptr(stream)))


def make_view(cam: Camera, world: int = 0, max_iters: int = 0, n_bounces: int = 0, shadow_dir=None,
              glsl: bool = False, aniso: bool = False) -> View:
    """A view: primary rays plus shadow rays toward shadow_dir, or n_bounces diffuse bounces,
    or with both the GPU renderer's whole path (sun rays after the primary and the first two
    bounce hits).
    glsl: trace with the GPU renderer's rayCast (VRT_VIEW_GLSL) instead of the CPU traversal;
    aniso: with its anisotropic LODs (VRT_VIEW_GLSL_ANISO)."""
    vw = View()
    vw.cam = cam
    vw.world = int(world)
    vw.max_iters = int(max_iters)
    vw.n_bounces = int(n_bounces)
    vw.flags = ((VIEW_SHADOW if shadow_dir is not None else 0) | (VIEW_GLSL if glsl or aniso else 0) |
                (capi.VIEW_GLSL_ANISO if aniso else 0))
    if shadow_dir is not None:
        vw.sun_dir[:] = [float(c) for c in shadow_dir]
    return vw


def view_records(view: View) -> int:
    return lib().vrt_view_records(C.byref(view))


def render_path(world: "World", view: View, stream=None) -> np.ndarray:
    """One view with its secondary rays, one plain launch; (kinds, h*w) records."""
    n = view_records(view)
    hits = np.zeros(n, HIT_DTYPE)
    check(lib().vrt_render_path(world.handle, C.byref(view), ptr(hits), _stream_ptr(stream)))
    return hits.reshape(-1, view.cam.width * view.cam.height)


def render_gbuffer(world: "World", view: View, palette, proj, stream=None):
    """G-buffer of a view's primary hits (vrt_render_gbuffer): (albedo_normal u32, depth f32),
    each width*height.  palette: 256 material words; proj: 4x4 column-major (16 floats)."""
    n = view.cam.width * view.cam.height
    pal = np.ascontiguousarray(palette, dtype=np.uint32)
    pm = np.ascontiguousarray(proj, dtype=np.float32).reshape(16)
    if pal.size != 256:
        raise ValueError("palette needs 256 entries")
    tex, depth = np.zeros(n, np.uint32), np.zeros(n, np.float32)
    check(lib().vrt_render_gbuffer(world.handle, C.byref(view), ptr(pal), ptr(pm), ptr(tex), ptr(depth),
                                   _stream_ptr(stream)))
    return tex, depth


class Batch:
    """Many views over many worlds behind one persistent launch (vrt_batch)."""

    def __init__(self, worlds, views, config: BatchConfig | None = None):
        self.worlds = list(worlds)
        self.views = list(views)
        wh = (C.c_void_p * len(self.worlds))(*[w.handle.value for w in self.worlds])
        va = (View * len(self.views))(*self.views)
        h = C.c_void_p()
        check(lib().vrt_batch_create(wh, len(self.worlds), va, len(self.views),
                                     C.byref(config) if config is not None else None, C.byref(h)))
        self._h = h
        offs = (C.c_uint64 * (len(self.views) + 1))()
        check(lib().vrt_batch_output_layout(h, offs))
        self.offsets = np.array(offs[:], np.uint64)
        self.total_records = int(self.offsets[-1])

    def close(self):
        if self._h:
            lib().vrt_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def launch(self, hits_device, stream=None, graph: bool = False) -> None:
        fn = lib().vrt_batch_launch_graph if graph else lib().vrt_batch_launch
        check(fn(self._h, ptr(hits_device), _stream_ptr(stream)))

    def launch_per_view(self, hits_device, stream=None) -> None:
        check(lib().vrt_batch_launch_per_view(self._h, ptr(hits_device), _stream_ptr(stream)))

    def run(self, hits_host=None, stream=None) -> np.ndarray:
        """Launch and copy all records to host memory (hits_host: numpy array or pinned tensor)."""
        if hits_host is None:
            hits_host = np.zeros(self.total_records, HIT_DTYPE)
        check(lib().vrt_batch_run(self._h, ptr(hits_host), _stream_ptr(stream)))
        return hits_host

    def run_packed(self, records_host=None, stream=None) -> np.ndarray:
        """vrt_batch_run with 12-byte records (PACKED_DTYPE) delivered to host memory."""
        if records_host is None:
            records_host = np.zeros(self.total_records, PACKED_DTYPE)
        check(lib().vrt_batch_run_packed(self._h, ptr(records_host), _stream_ptr(stream)))
        return records_host

    def update_cameras(self, cams, stream=None) -> None:
        arr = (Camera * len(cams))(*cams)
        check(lib().vrt_batch_update_cameras(self._h, arr, _stream_ptr(stream)))

    def stats(self) -> dict:
        s = capi.BatchStats()
        check(lib().vrt_batch_get_stats(self._h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def measure(self, hits_device, stream=None) -> dict:
        s = capi.BatchStats()
        check(lib().vrt_batch_measure(self._h, ptr(hits_device), _stream_ptr(stream), C.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def view_hits(self, hits: np.ndarray, v: int) -> np.ndarray:
        a, b = int(self.offsets[v]), int(self.offsets[v + 1])
        cam = self.views[v].cam
        return hits[a:b].reshape(-1, cam.width * cam.height)


class PinnedHits:
    """Pinned host buffer of hit records (vrt_host_alloc), viewed as a numpy array
    (dtype HIT_DTYPE, or PACKED_DTYPE for vrt_batch_run_packed)."""

    def __init__(self, n: int, dtype=HIT_DTYPE):
        p = C.c_void_p()
        check(lib().vrt_host_alloc(max(1, n) * dtype.itemsize, C.byref(p)))
        self._p = p
        buf = (C.c_uint8 * (max(1, n) * dtype.itemsize)).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dtype)[:n]

    def close(self):
        if self._p:
            self.array = None
            lib().vrt_host_free(self._p)
            self._p = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Request server with continuous batching over resident worlds (vrt_server)."""

    def __init__(self, worlds, max_inflight: int = 2, max_batch_requests: int = 0, hbm_budget_bytes: int = 0,
                 batch: BatchConfig | None = None, resident: bool | None = None, idle_us: int = 0):
        """resident=True: one persistent launch takes requests while it runs (VRT_SERVE_RESIDENT);
        False: each batch of queued requests is its own launch, max_inflight at a time
        (VRT_SERVE_LAUNCHES); None: resident where the device supports it."""
        self.worlds = list(worlds)
        cfg = capi.ServerConfig(int(max_inflight), int(max_batch_requests), int(hbm_budget_bytes),
                                batch if batch is not None else BatchConfig(),
                                {None: 0, True: capi.SERVE_RESIDENT, False: capi.SERVE_LAUNCHES}[resident],
                                int(idle_us))
        wh = (C.c_void_p * len(self.worlds))(*[w.handle.value for w in self.worlds])
        h = C.c_void_p()
        check(lib().vrt_server_create(wh, len(self.worlds), C.byref(cfg), C.byref(h)))
        self._h = h
        self._keep = {}

    def close(self, timeout_ms: int = 60000):
        if self._h:
            st = lib().vrt_server_destroy(self._h, int(timeout_ms))
            self._h = C.c_void_p()
            self._keep.clear()
            check(st)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit_render(self, view: View, out: np.ndarray) -> int:
        """out: HIT_DTYPE array of view_records(view) entries (pinned for asynchronous copies)."""
        assert out.dtype == HIT_DTYPE and out.size >= view_records(view) and out.flags.c_contiguous
        t = C.c_uint64()
        check(lib().vrt_server_submit_render(self._h, C.byref(view), ptr(out), C.byref(t)))
        self._keep[t.value] = out
        return t.value

    def submit_edit(self, world: int, edits) -> int:
        e = np.ascontiguousarray(edits, dtype=EDIT_DTYPE)
        t = C.c_uint64()
        check(lib().vrt_server_submit_edit(self._h, int(world), ptr(e), len(e), C.byref(t)))
        return t.value

    def wait(self, ticket: int, timeout_ms: int = 60000) -> dict:
        info = capi.RequestInfo()
        st = lib().vrt_server_wait(self._h, int(ticket), int(timeout_ms), C.byref(info))
        self._keep.pop(ticket, None)
        check(st)
        return {f: getattr(info, f) for f, _ in info._fields_}

    def drain(self, timeout_ms: int = 60000) -> None:
        check(lib().vrt_server_drain(self._h, int(timeout_ms)))

    def stats(self, reset: bool = False) -> dict:
        s = capi.ServerStats()
        check(lib().vrt_server_get_stats(self._h, int(reset), C.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_}
