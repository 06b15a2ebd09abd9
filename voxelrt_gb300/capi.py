"""ctypes binding of libvrt.so (include/vrt.h, include/vrt_synth.h).

Only plumbing: every operation runs in the native library.  Importing this module
fails loudly when the library has not been built - there is no Python fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libvrt.so"
_SYNTH_PATH = Path(__file__).resolve().parent / "_lib" / "libvrt_synth.so"

VRT_OK = 0
VRT_ERR_INVALID_ARG = 1
VRT_ERR_OUT_OF_MEMORY = 2
VRT_ERR_QUEUE_TIMEOUT = 3
VRT_ERR_DEVICE = 4
VRT_ERR_NO_DEVICE = 5
VRT_ERR_SLOTS_EXHAUSTED = 6
VRT_ERR_NOT_FOUND = 7
VRT_ERR_IO = 8
VRT_ERR_FORMAT = 9

MISS_VOXEL = 0xFFFFFFFF
MISS_FACE = 0xFF
NO_RAY = 0xFFFFFFFF
PACKED_NO_RAY = 0xFF  # vrt_hit_packed.material of a record whose ray was never cast
DEFAULT_MAX_ITERS = 128
EDIT_FILL = 0
EDIT_REPLACE = 1


class Ray(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("dir", C.c_float * 3), ("tag", C.c_uint32), ("reserved", C.c_uint32)]


class Hit(C.Structure):
    _fields_ = [("voxel", C.c_uint32), ("face", C.c_uint8), ("material", C.c_uint8), ("steps", C.c_uint16),
                ("t", C.c_float), ("tag", C.c_uint32)]


class CastParams(C.Structure):
    _fields_ = [("world_origin", C.c_int32 * 3), ("max_iters", C.c_uint32), ("flags", C.c_uint32)]


class Camera(C.Structure):
    _fields_ = [("world_origin", C.c_int32 * 3), ("origin", C.c_float * 3), ("d0", C.c_float * 3),
                ("du", C.c_float * 3), ("dv", C.c_float * 3), ("width", C.c_uint32), ("height", C.c_uint32)]


class Edit(C.Structure):
    _fields_ = [("center", C.c_int32 * 3), ("radius", C.c_uint32), ("material", C.c_uint8), ("mode", C.c_uint8),
                ("reserved", C.c_uint16)]


class View(C.Structure):
    _fields_ = [("cam", Camera), ("world", C.c_uint32), ("max_iters", C.c_uint32), ("n_bounces", C.c_uint32),
                ("flags", C.c_uint32), ("sun_dir", C.c_float * 3)]


class BatchConfig(C.Structure):
    _fields_ = [("tile_w", C.c_uint32), ("tile_h", C.c_uint32), ("morton", C.c_uint32),
                ("warps_per_block", C.c_uint32), ("blocks_per_sm", C.c_uint32), ("refill_threshold", C.c_uint32),
                ("chunk_tiles", C.c_uint32), ("inner_iters", C.c_uint32)]


class BatchStats(C.Structure):
    _fields_ = [("rays_cast", C.c_uint64), ("step_calls", C.c_uint64), ("occ_fetches", C.c_uint64),
                ("hits", C.c_uint64)]


WORLD_L2_PERSIST = 1  # VRT_WORLD_L2_PERSIST: the brick table persisting in L2 on the caller's streams
VIEW_SHADOW = 1
VIEW_GLSL = 2        # the GPU renderer's rayCast (VoxelTraversal.glsl) instead of the CPU traversal
CAST_GLSL = 1
CAST_GLSL_COARSE = 2
CAST_GLSL_ANISO = 4
VIEW_GLSL_ANISO = 4
GLSL_MAX_ITERS = 256


class ServerConfig(C.Structure):
    _fields_ = [("max_inflight", C.c_uint32), ("max_batch_requests", C.c_uint32), ("hbm_budget_bytes", C.c_uint64),
                ("batch", BatchConfig), ("flags", C.c_uint32), ("idle_us", C.c_uint32)]


SERVE_RESIDENT = 1
SERVE_LAUNCHES = 2


class RequestInfo(C.Structure):
    _fields_ = [("state", C.c_uint32), ("kind", C.c_uint32), ("status", C.c_int), ("batch_size", C.c_uint32),
                ("rays", C.c_uint64), ("submit_us", C.c_double), ("start_us", C.c_double), ("done_us", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("renders_done", C.c_uint64), ("edits_done", C.c_uint64), ("rejected", C.c_uint64),
                ("launches", C.c_uint64), ("records", C.c_uint64), ("p50_us", C.c_double), ("p99_us", C.c_double),
                ("p999_us", C.c_double), ("max_us", C.c_double), ("busy_seconds", C.c_double),
                ("resident", C.c_uint32), ("reserved", C.c_uint32)]


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = 0, 1, 2, 3


class WorldDesc(C.Structure):
    _fields_ = [("sectors_x", C.c_uint32), ("sectors_y", C.c_uint32), ("sectors_z", C.c_uint32),
                ("brick_capacity", C.c_uint32), ("device", C.c_int32), ("flags", C.c_uint32)]


class WorldStats(C.Structure):
    _fields_ = [("sectors_x", C.c_uint32), ("sectors_y", C.c_uint32), ("sectors_z", C.c_uint32),
                ("allocated_bricks", C.c_uint32), ("brick_capacity", C.c_uint32), ("free_ranges", C.c_uint32),
                ("device_bytes", C.c_uint64), ("compactions", C.c_uint32), ("reserved", C.c_uint32)]


class SectorStream(C.Structure):
    _fields_ = [("sectors_x", C.c_uint32), ("sectors_y", C.c_uint32), ("sectors_z", C.c_uint32),
                ("n_sectors", C.c_uint32), ("n_bricks", C.c_uint64), ("sector_idx", C.POINTER(C.c_int32)),
                ("alloc_mask", C.POINTER(C.c_uint64)), ("bricks", C.POINTER(C.c_uint8))]


class SynthTerrain(C.Structure):
    _fields_ = [("size", C.c_uint32 * 3), ("base", C.c_double), ("amplitude", C.c_double), ("scale", C.c_double),
                ("octaves", C.c_uint32), ("seed", C.c_uint64), ("cave_octaves", C.c_uint32),
                ("cave_scale", C.c_double), ("cave_threshold", C.c_double), ("cave_seed", C.c_uint64)]


RAY_DTYPE = np.dtype([("origin", "<f4", 3), ("dir", "<f4", 3), ("tag", "<u4"), ("reserved", "<u4")])
HIT_DTYPE = np.dtype([("voxel", "<u4"), ("face", "u1"), ("material", "u1"), ("steps", "<u2"), ("t", "<f4"),
                      ("tag", "<u4")])
# vrt_hit_packed: vrt_hit without its tag
PACKED_DTYPE = np.dtype([("voxel", "<u4"), ("face", "u1"), ("material", "u1"), ("steps", "<u2"), ("t", "<f4")])
PICK_DTYPE = np.dtype([("distance", "<f8"), ("voxel", "<i4", 3), ("normal", "<f4", 3), ("uv", "<f4", 2),
                       ("iters", "<u4"), ("reserved", "<u4")])
EDIT_DTYPE = np.dtype([("center", "<i4", 3), ("radius", "<u4"), ("material", "u1"), ("mode", "u1"),
                       ("reserved", "<u2")])
assert RAY_DTYPE.itemsize == C.sizeof(Ray) == 32
assert HIT_DTYPE.itemsize == C.sizeof(Hit) == 16
assert PACKED_DTYPE.itemsize == 12
assert EDIT_DTYPE.itemsize == C.sizeof(Edit) == 20
assert PICK_DTYPE.itemsize == 48

_vp = C.c_void_p
_st = C.c_int
_u32 = C.c_uint32
_i32 = C.c_int32
_u64 = C.c_uint64

# name -> (restype, argtypes); every symbol declared in include/*.h
PROTOTYPES = {
    "vrt_last_error": (C.c_char_p, []),
    "vrt_abi_version": (_u32, []),
    "vrt_sector_index": (_i32, [_i32, _i32, _i32]),
    "vrt_world_create": (_st, [C.POINTER(WorldDesc), C.POINTER(_vp)]),
    "vrt_world_destroy": (_st, [_vp]),
    "vrt_world_get_stats": (_st, [_vp, C.POINTER(WorldStats)]),
    "vrt_world_sync_sectors": (_st, [_vp, _u32, _vp, _vp, _vp, _vp, _vp]),
    "vrt_world_edit": (_st, [_vp, _vp, _u32, _vp]),
    "vrt_world_wait": (_st, [_vp]),
    "vrt_world_defrag": (_st, [_vp, _u32, _vp]),
    "vrt_world_read_sector": (_st, [_vp, _i32, C.POINTER(_u64), _vp, C.c_size_t, _vp]),
    "vrt_cvox_write": (_st, [C.c_char_p, _u32, _vp, _vp, _vp]),
    "vrt_cvox_read": (_st, [C.c_char_p, C.POINTER(C.POINTER(SectorStream))]),
    "vrt_world_save_cvox": (_st, [_vp, C.c_char_p]),
    "vrt_world_load_cvox": (_st, [_vp, C.c_char_p, _vp]),
    "vrt_cast": (_st, [_vp, _vp, _u32, C.POINTER(CastParams), _vp, _vp]),
    "vrt_cast_device": (_st, [_vp, _vp, _u32, C.POINTER(CastParams), _vp, _vp]),
    "vrt_render_view": (_st, [_vp, C.POINTER(Camera), _u32, _vp, _vp]),
    "vrt_render_view_device": (_st, [_vp, C.POINTER(Camera), _u32, _vp, _vp]),
    "vrt_pick": (_st, [_vp, _vp, _u32, _u32, _vp, _vp]),
    "vrt_camera_look_at": (_st, [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_double, _u32, _u32,
                                 C.POINTER(Camera)]),
    "vrt_view_records": (_u64, [C.POINTER(View)]),
    "vrt_render_path": (_st, [_vp, C.POINTER(View), _vp, _vp]),
    "vrt_render_path_device": (_st, [_vp, C.POINTER(View), _vp, _vp]),
    "vrt_render_gbuffer": (_st, [_vp, C.POINTER(View), _vp, _vp, _vp, _vp, _vp]),
    "vrt_render_gbuffer_device": (_st, [_vp, C.POINTER(View), _vp, _vp, _vp, _vp, _vp, _vp]),
    "vrt_batch_create": (_st, [C.POINTER(_vp), _u32, C.POINTER(View), _u32, C.POINTER(BatchConfig), C.POINTER(_vp)]),
    "vrt_batch_destroy": (_st, [_vp]),
    "vrt_batch_output_layout": (_st, [_vp, C.POINTER(_u64)]),
    "vrt_batch_launch": (_st, [_vp, _vp, _vp]),
    "vrt_batch_launch_graph": (_st, [_vp, _vp, _vp]),
    "vrt_batch_launch_per_view": (_st, [_vp, _vp, _vp]),
    "vrt_batch_run": (_st, [_vp, _vp, _vp]),
    "vrt_batch_run_packed": (_st, [_vp, _vp, _vp]),
    "vrt_batch_update_cameras": (_st, [_vp, C.POINTER(Camera), _vp]),
    "vrt_batch_get_stats": (_st, [_vp, C.POINTER(BatchStats)]),
    "vrt_batch_measure": (_st, [_vp, _vp, _vp, C.POINTER(BatchStats)]),
    "vrt_render_views_static": (_st, [C.POINTER(_vp), _u32, C.POINTER(View), _u32, C.POINTER(BatchConfig), _vp,
                                       _vp]),
    "vrt_host_alloc": (_st, [C.c_size_t, C.POINTER(_vp)]),
    "vrt_host_free": (_st, [_vp]),
    "vrt_server_create": (_st, [C.POINTER(_vp), _u32, C.POINTER(ServerConfig), C.POINTER(_vp)]),
    "vrt_server_destroy": (_st, [_vp, _u32]),
    "vrt_server_submit_render": (_st, [_vp, C.POINTER(View), _vp, C.POINTER(_u64)]),
    "vrt_server_submit_edit": (_st, [_vp, _u32, _vp, _u32, C.POINTER(_u64)]),
    "vrt_server_wait": (_st, [_vp, _u64, _u32, C.POINTER(RequestInfo)]),
    "vrt_server_drain": (_st, [_vp, _u32]),
    "vrt_server_get_stats": (_st, [_vp, C.c_int, C.POINTER(ServerStats)]),
    "vrt_sector_stream_free": (None, [C.POINTER(SectorStream)]),
}

# libvrt_synth.so (include/vrt_synth.h): host-only generators of seeded inputs, plus its
# own copies of vrt_camera_look_at and vrt_sector_stream_free
SYNTH_PROTOTYPES = {
    "vrt_synth_last_error": (C.c_char_p, []),
    "vrt_synth_terrain_world": (_st, [C.POINTER(SynthTerrain), C.c_int, C.POINTER(C.POINTER(SectorStream))]),
    "vrt_synth_terrain_height": (C.c_double, [C.POINTER(SynthTerrain), C.c_double, C.c_double]),
    "vrt_synth_mix_world": (_st, [_u32, _u64, C.c_int, C.POINTER(C.POINTER(SectorStream))]),
    "vrt_synth_random_rays": (_st, [C.POINTER(_u32), _u64, _u64, _u64, C.c_int, _vp]),
    "vrt_camera_look_at": PROTOTYPES["vrt_camera_look_at"],
    "vrt_sector_stream_free": PROTOTYPES["vrt_sector_stream_free"],
}


class VrtError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"vrt status {status}: {msg}")
        self.status = status


_lib = None
_synth = None


def _load(path: Path, prototypes: dict) -> C.CDLL:
    if not path.exists():
        raise ImportError(f"{path} is missing: run `python -m voxelrt_gb300.build` first")
    L = C.CDLL(str(path))
    for name, (res, args) in prototypes.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def synth_lib() -> C.CDLL:
    """Load libvrt_synth.so, the host-only input generators (raises if it has not been built)."""
    global _synth
    if _synth is None:
        _synth = _load(_SYNTH_PATH, SYNTH_PROTOTYPES)
    return _synth


def check_synth(status: int) -> None:
    if status != VRT_OK:
        raise VrtError(status, synth_lib().vrt_synth_last_error().decode(errors="replace"))


def lib() -> C.CDLL:
    """Load libvrt.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        _lib = _load(_LIB_PATH, PROTOTYPES)
    return _lib


def check(status: int) -> None:
    if status != VRT_OK:
        raise VrtError(status, lib().vrt_last_error().decode(errors="replace"))


def ptr(a) -> int | None:
    """Address of a numpy array, a torch tensor, or None."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    if isinstance(a, int):
        return a
    raise TypeError(type(a))
