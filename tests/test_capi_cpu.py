"""The C ABI library loads without a GPU and exports every symbol include/*.h declares."""
import ctypes as C
import re
from pathlib import Path

import numpy as np

import voxelrt_gb300 as v

ROOT = Path(__file__).resolve().parent.parent
DECL = re.compile(r"^[A-Za-z_][\w\s\*]*?\b(vrt_\w+)\s*\(", re.M)


def declared_symbols(header="vrt.h"):
    text = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / header).read_text(), flags=re.S)
    return {m.group(1) for m in DECL.finditer(text)}


def test_every_declared_symbol_is_exported():
    lib = C.CDLL(str(ROOT / "voxelrt_gb300" / "_lib" / "libvrt.so"))
    names = declared_symbols()
    assert len(names) > 40
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding declares a prototype for each of them
    assert names <= set(v.capi.PROTOTYPES), sorted(names - set(v.capi.PROTOTYPES))
    # the synthetic-input generators are not part of the product library
    assert not any(hasattr(lib, n) for n in declared_symbols("vrt_synth.h"))


def test_synth_library_is_host_only():
    """libvrt_synth.so exports what include/vrt_synth.h declares (plus the camera builder and
    the stream release of vrt.h) and links no CUDA library."""
    path = ROOT / "voxelrt_gb300" / "_lib" / "libvrt_synth.so"
    lib = C.CDLL(str(path))
    names = declared_symbols("vrt_synth.h") | {"vrt_camera_look_at", "vrt_sector_stream_free"}
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert names <= set(v.capi.SYNTH_PROTOTYPES)
    needed = [ln for ln in path.read_bytes().split(b"\0") if ln.startswith(b"libcuda")]
    assert not needed, needed


def test_struct_layouts_match_header():
    assert C.sizeof(v.capi.Ray) == 32 and C.sizeof(v.capi.Hit) == 16 and C.sizeof(v.capi.Edit) == 20
    assert C.sizeof(v.Camera) == 68 and C.sizeof(v.View) == 96


def test_host_logic_without_gpu():
    assert v.lib().vrt_abi_version() == 1
    # WorldSectorIndexer packing (VoxelMap.h:95-100): x | z<<12 | y<<24, 12/8/12 signed bits
    assert v.sector_index(1, 2, 3) == 1 | 3 << 12 | 2 << 24
    assert v.sector_index(-1, 0, 0) == 0xFFF
    for xyz in [(1, 2, 3), (-1, 0, 0), (5, -2, 7), (-3, -128, 2047), (100, 127, -100)]:
        assert v.sector_index(*xyz) == v.lib().vrt_sector_index(*xyz)
    cam = v.look_at((128, 200, -40), (128, 80, 128), 90.0, 640, 360)
    # the product library's camera builder is the same code
    cam2 = v.Camera()
    p3, t3 = (C.c_double * 3)(128, 200, -40), (C.c_double * 3)(128, 80, 128)
    v.check(v.lib().vrt_camera_look_at(p3, t3, 90.0, 640, 360, C.byref(cam2)))
    assert bytes(cam) == bytes(cam2)
    assert list(cam.world_origin) == [128, 200, -40] and cam.width == 640
    # the centre pixel looks at the target
    d = np.array(cam.d0[:]) + 320 * np.array(cam.du[:]) + 180 * np.array(cam.dv[:])
    tgt = np.array([0.0, -120.0, 168.0])
    assert np.allclose(d / np.linalg.norm(d), tgt / np.linalg.norm(tgt), atol=1e-6)
    # unknown world flags are refused before any device is touched
    try:
        v.World((1, 1, 1), flags=v.capi.WORLD_L2_PERSIST << 1)
        raise AssertionError("unknown flag accepted")
    except v.VrtError as e:
        assert e.status == v.capi.VRT_ERR_INVALID_ARG and "flags" in str(e)
    # no device: creating a world fails with a status, not a crash
    import torch
    if not torch.cuda.is_available():
        with np.testing.assert_raises(v.VrtError):
            v.World((1, 1, 1))


def test_synthetic_worlds_are_deterministic():
    a = v.synth_terrain((64, 64, 64), base=20, amplitude=10, seed=5, cave_octaves=2, threads=1)
    b = v.synth_terrain((64, 64, 64), base=20, amplitude=10, seed=5, cave_octaves=2, threads=4)
    assert np.array_equal(a.sector_idx, b.sector_idx) and np.array_equal(a.bricks, b.bricks)
    m1, m2 = v.synth_mix(64, seed=3, threads=1), v.synth_mix(64, seed=3, threads=3)
    assert np.array_equal(m1.bricks, m2.bricks) and m1.n_bricks > 0
    # the stream holds only non-empty bricks, masks match the brick count
    assert all(m1.bricks.reshape(-1, 512).any(axis=1))
    assert sum(bin(int(m)).count("1") for m in m1.alloc_mask) == m1.n_bricks
    r1 = v.random_rays((64, 64, 64), seed=1, n=1000)
    r2 = v.random_rays((64, 64, 64), seed=1, n=500, first=500)
    assert np.array_equal(r1[500:], r2)
    n = np.linalg.norm(r1["dir"].astype(np.float64), axis=1)
    assert np.allclose(n, 1.0, atol=1e-6)
