"""cvox v4 world files (VoxelMap::Serialize / Deserialize, VoxelMap.cpp:205-273).

Files are written with zstd frames of stored blocks; the system's libzstd (when the
host has one) must decode them, and files whose blobs are zstd-compressed, as the
reference writes them, must read back through it.
"""
import ctypes as C
import ctypes.util
import struct

import numpy as np
import pytest

import voxelrt_gb300 as v


def zstd():
    for name in ("libzstd.so.1", ctypes.util.find_library("zstd")):
        if not name:
            continue
        try:
            z = C.CDLL(name)
        except OSError:
            continue
        z.ZSTD_decompress.restype = C.c_size_t
        z.ZSTD_decompress.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t]
        z.ZSTD_compress.restype = C.c_size_t
        z.ZSTD_compress.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_int]
        z.ZSTD_compressBound.restype = C.c_size_t
        z.ZSTD_compressBound.argtypes = [C.c_size_t]
        z.ZSTD_isError.restype = C.c_uint
        z.ZSTD_isError.argtypes = [C.c_size_t]
        return z
    return None


def blobs(buf):
    """Split a cvox file into (raw size, frame bytes) of the palette and packs."""
    off = 12
    n = struct.unpack_from("<I", buf, off)[0]
    out = [(4096, buf[off + 4: off + 4 + n])]
    off += 4 + n
    while off < len(buf):
        raw, n = struct.unpack_from("<II", buf, off)
        out.append((raw, buf[off + 8: off + 8 + n]))
        off += 8 + n
    return out


def test_round_trip(tmp_path):
    d = v.synth_mix(96, seed=5)
    p = tmp_path / "w.cvox"
    v.cvox_write(p, d)
    buf = p.read_bytes()
    assert buf[:8] == b"cvox\x04\x00\x00\x00" and struct.unpack_from("<I", buf, 8)[0] == len(d.sector_idx)
    r = v.cvox_read(p)
    assert np.array_equal(r.sector_idx, d.sector_idx) and np.array_equal(r.alloc_mask, d.alloc_mask)
    assert np.array_equal(r.bricks, d.bricks)
    assert r.sectors == d.sectors


def test_frames_decode_with_system_zstd(tmp_path):
    z = zstd()
    if z is None:
        pytest.skip("no libzstd on this host")
    d = v.synth_terrain((128, 64, 128), base=20, amplitude=12, seed=3)
    p = tmp_path / "w.cvox"
    v.cvox_write(p, d)
    for raw, frame in blobs(p.read_bytes()):
        out = C.create_string_buffer(max(raw, 1))
        src = C.create_string_buffer(frame, len(frame))
        r = z.ZSTD_decompress(out, raw, src, len(frame))
        assert not z.ZSTD_isError(r) and r == raw


def test_reads_zstd_compressed_files(tmp_path):
    z = zstd()
    if z is None:
        pytest.skip("no libzstd on this host")
    d = v.synth_mix(64, seed=9)
    p = tmp_path / "raw.cvox"
    v.cvox_write(p, d)
    parts = blobs(p.read_bytes())
    out = bytearray(p.read_bytes()[:12])
    for i, (raw, frame) in enumerate(parts):
        plain = C.create_string_buffer(max(raw, 1))
        z.ZSTD_decompress(plain, raw, C.create_string_buffer(frame, len(frame)), len(frame))
        cap = z.ZSTD_compressBound(raw)
        comp = C.create_string_buffer(cap)
        n = z.ZSTD_compress(comp, cap, plain, raw, 3)
        assert not z.ZSTD_isError(n)
        if i > 0:
            out += struct.pack("<I", raw)
        out += struct.pack("<I", n) + comp.raw[:n]
    q = tmp_path / "zstd.cvox"
    q.write_bytes(bytes(out))
    assert len(out) < p.stat().st_size  # really compressed
    r = v.cvox_read(q)
    assert np.array_equal(r.bricks, d.bricks) and np.array_equal(r.alloc_mask, d.alloc_mask)


def test_rejects_bad_files(tmp_path):
    p = tmp_path / "bad.cvox"
    p.write_bytes(b"cvox\x03\x00\x00\x00" + b"\x00" * 20)
    with pytest.raises(v.VrtError) as e:
        v.cvox_read(p)
    assert e.value.status == v.capi.VRT_ERR_FORMAT
    d = v.synth_mix(64, seed=1)
    good = tmp_path / "good.cvox"
    v.cvox_write(good, d)
    buf = good.read_bytes()
    (tmp_path / "short.cvox").write_bytes(buf[: len(buf) // 2])
    with pytest.raises(v.VrtError):
        v.cvox_read(tmp_path / "short.cvox")
    with pytest.raises(v.VrtError) as e:
        v.cvox_read(tmp_path / "missing.cvox")
    assert e.value.status == v.capi.VRT_ERR_IO


def _sorted_stream(idx, masks, bricks):
    """Sector records in ascending index order (files keep the writer's order)."""
    order = np.argsort(np.asarray(idx, np.int64), kind="stable")
    counts = np.array([bin(int(m)).count("1") for m in masks], np.int64)
    starts = np.concatenate([[0], np.cumsum(counts)])
    out = [bricks[starts[i]:starts[i + 1]] for i in order]
    return (np.asarray(idx)[order], np.asarray(masks)[order],
            np.concatenate(out) if out else np.zeros((0, 512), np.uint8))


def test_reads_the_reference_writer():
    """tests/golden/refworld.cvox was written by the reference's own VoxelMap::Serialize with
    its zstd framing (compressed packs, checksums), compiled in place by
    tests/golden/make_golden_cvox.py; reading it gives back the seeded world byte for byte."""
    from tests.golden.make_golden_cvox import OUT_FILE, build_world
    data = build_world()
    try:
        got = v.cvox_read(OUT_FILE)
    except v.VrtError as e:
        if "libzstd" in str(e):
            pytest.skip("compressed packs need the system libzstd.so.1")
        raise
    want = _sorted_stream(data.sector_idx, data.alloc_mask, data.bricks)
    have = _sorted_stream(got.sector_idx, got.alloc_mask, got.bricks)
    assert np.array_equal(have[0], want[0]) and np.array_equal(have[1], want[1])
    assert np.array_equal(have[2], want[2])


def test_reference_reads_this_writer(tmp_path):
    """The reference's own VoxelMap::Deserialize read a file written by vrt_cvox_write
    (tests/golden/refcvox.npz holds what it read and the file's SHA-256): it read the seeded
    world byte for byte, and vrt_cvox_write still writes that same file."""
    import hashlib
    from tests.golden.make_golden_cvox import OUT_NPZ, build_world
    z = np.load(OUT_NPZ)
    data = build_world()
    p = tmp_path / "ours.cvox"
    v.cvox_write(p, data)
    assert hashlib.sha256(p.read_bytes()).hexdigest() == str(z["ours_sha256"])
    want = _sorted_stream(data.sector_idx, data.alloc_mask, data.bricks)
    assert np.array_equal(z["sector_idx"], want[0]) and np.array_equal(z["alloc_mask"], want[1])
    assert np.array_equal(z["bricks"], want[2])
