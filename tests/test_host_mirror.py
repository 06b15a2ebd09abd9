"""The C++ host mirror (include/vrt.hpp): VoxelMap edits and GpuRenderer frames.

A small C++ program drives VoxelMap::Set / RegionDispatch and GpuRenderer the way
the reference's application does; its host model must equal the oracle after the
same edits, and its frames must equal the oracle's render of that model.
"""
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

import voxelrt_gb300 as v
from oracle.oracle import OracleWorld
from tests.helpers import assert_hits_equal

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "host_model_test.cpp"
EXE = ROOT / "tests" / "cpp" / "_build" / "host_model_test"


@pytest.fixture(scope="module")
def exe():
    EXE.parent.mkdir(exist_ok=True)
    lib = ROOT / "voxelrt_gb300" / "_lib"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"), str(SRC), "-o", str(EXE),
                    "-L", str(lib), "-lvrt", f"-Wl,-rpath,{lib}"], check=True)
    return EXE


def read_sectors(buf):
    n = struct.unpack_from("<I", buf, 0)[0]
    off, recs = 4, {}
    for _ in range(n):
        k, m = struct.unpack_from("<IQ", buf, off)
        off += 12
        nb = bin(m).count("1")
        recs[k] = (m, np.frombuffer(buf, np.uint8, nb * 512, off).reshape(nb, 512))
        off += nb * 512
    return recs, off


def oracle_model():
    """The same world built with the oracle: column heights, then the same spheres."""
    vol = np.zeros((64, 64, 64), np.uint8)  # (y, z, x)
    for x in range(64):
        for z in range(64):
            h = 10 + (x * 7 + z * 3) % 13
            for y in range(h):
                vol[y, z, x] = 1 + y // 8
    from tests.helpers import dense_to_stream
    o = OracleWorld((2, 2, 2))
    o.upload(dense_to_stream(vol))
    e = np.zeros(4, v.EDIT_DTYPE)
    e["center"] = [(30, 20, 30), (10, 40, 50), (50, 8, 10), (0, 0, 0)]
    e["radius"] = [12, 9, 6, 3]
    e["material"] = [0, 77, 0, 200]
    o.edit(e)
    return o


def test_host_model_edits_match_oracle(exe, tmp_path):
    out = tmp_path / "edits.bin"
    subprocess.run([str(exe), "edits", str(out)], check=True)
    recs, _ = read_sectors(out.read_bytes())
    o = oracle_model()
    for sy in range(2):
        for sz in range(2):
            for sx in range(2):
                idx = v.sector_index(sx, sy, sz) & 0xFFFFFFFF
                m, bricks = o.read_sector(idx)
                if m == 0:
                    assert idx not in recs
                    continue
                gm, gb = recs[idx]
                assert gm == m and np.array_equal(gb, bricks)


@pytest.mark.gpu
def test_gpu_renderer_frames_match_oracle(exe, tmp_path, gpu):
    out = tmp_path / "render.bin"
    subprocess.run([str(exe), "render", str(out)], check=True)
    buf = out.read_bytes()
    _, off = read_sectors(buf)
    n = struct.unpack_from("<Q", buf, off)[0]
    off += 8
    a = np.frombuffer(buf, v.HIT_DTYPE, n, off)
    b = np.frombuffer(buf, v.HIT_DTYPE, n, off + 16 * n)
    c = np.frombuffer(buf, v.HIT_DTYPE, n, off + 32 * n)
    cam = v.Camera.from_buffer_copy(buf[off + 48 * n: off + 48 * n + 68])
    o = oracle_model()
    assert_hits_equal(a, o.render_view(cam))
    e = np.zeros(1, v.EDIT_DTYPE)
    e["center"], e["radius"], e["material"] = (32, 12, 32), 10, 0
    o.edit(e)
    assert_hits_equal(b, o.render_view(cam))
    assert not np.array_equal(a["voxel"], b["voxel"])
    # GpuRenderer::UseAnisotropicLods: the next frame in the GLSL mode with anisotropic LODs
    assert_hits_equal(c, o.render_view(cam, glsl=True, aniso=True))
