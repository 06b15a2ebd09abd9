"""The device traversal step compiled for the host, against the oracle (no GPU).

tests/cpp/device_logic_test.cpp includes voxelrt_gb300/csrc/trace_core.cuh with the
CUDA rounding intrinsics mapped to IEEE host operations; the worlds are laid out
exactly as the device stores them (brick table, voxel codes, brick-slot pools).  Every record
must match the oracle, which checks the kernel's control flow on each CPU run.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import voxelrt_gb300 as v
from oracle.oracle import OracleWorld
from tests.helpers import assert_hits_equal, cell_corner_world, cfg0_world, dense_to_stream, make_rays

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "device_logic_test.cpp"
EXE = ROOT / "tests" / "cpp" / "_build" / "device_logic_test"


@pytest.fixture(scope="module")
def exe():
    EXE.parent.mkdir(exist_ok=True)
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-I", str(ROOT / "include"),
                    str(SRC), "-o", str(EXE)], check=True)
    return EXE


def forward_boxes() -> np.ndarray:
    """(64 cells, 8 octants) u64: the cells of a 4^3 block on or ahead of the cell along
    the octant's directions (octant bit per axis set for dir >= 0), bit x + z*4 + y*16."""
    c = np.arange(64)
    x, z, y = c & 3, (c >> 2) & 3, c >> 4
    out = np.zeros((64, 8), np.uint64)
    for o in range(8):
        ok = lambda a, b, pos: (b >= a) if pos else (b <= a)
        keep = (ok(x[:, None], x[None, :], o & 1) & ok(y[:, None], y[None, :], o & 2) &
                ok(z[:, None], z[None, :], o & 4))
        out[:, o] = (keep.astype(np.uint64) << c[None, :].astype(np.uint64)).sum(axis=1, dtype=np.uint64)
    return out


def skip_level(masked: np.ndarray, idx: np.ndarray) -> np.ndarray:
    """2 when the 4^3 mask is empty, 1 when the aligned 2^3 block around idx is, else 0."""
    c = np.arange(64)
    x, z, y = c & 3, (c >> 2) & 3, c >> 4
    blk = np.zeros(64, np.uint64)
    for i in range(64):
        inb = ((x >> 1) == (x[i] >> 1)) & ((z >> 1) == (z[i] >> 1)) & ((y >> 1) == (y[i] >> 1))
        blk[i] = (inb.astype(np.uint64) << c.astype(np.uint64)).sum(dtype=np.uint64)
    return np.where(masked == 0, 2, np.where((masked & blk[idx]) == 0, 1, 0)).astype(np.uint32)


def aniso_bits(alloc: np.ndarray, sector_any: np.ndarray) -> np.ndarray:
    """Bits 5 and 15-30 of every brick position's table entry (only empty ones use them)."""
    nby, nbz, nbx = alloc.shape
    sy, sz, sx = nby // 4, nbz // 4, nbx // 4
    bits = np.uint64(1) << np.arange(64, dtype=np.uint64)
    # sector masks (bit bx&3 | (bz&3)<<2 | (by&3)<<4) and group masks over padded sectors
    sm = (alloc.reshape(sy, 4, sz, 4, sx, 4).transpose(0, 2, 4, 1, 3, 5).reshape(sy, sz, sx, 64).astype(np.uint64)
          * bits).sum(axis=3, dtype=np.uint64)
    gy, gz, gx = sector_any.shape[0] // 4, sector_any.shape[1] // 4, sector_any.shape[2] // 4
    gm = (sector_any.reshape(gy, 4, gz, 4, gx, 4).transpose(0, 2, 4, 1, 3, 5).reshape(gy, gz, gx, 64)
          .astype(np.uint64) * bits).sum(axis=3, dtype=np.uint64)
    by, bz, bx = np.meshgrid(np.arange(nby), np.arange(nbz), np.arange(nbx), indexing="ij")
    ys, zs, xs = by >> 2, bz >> 2, bx >> 2
    empty_sector = sm[ys, zs, xs] == 0
    lm = np.where(empty_sector, gm[ys >> 2, zs >> 2, xs >> 2], sm[ys, zs, xs])
    li = np.where(empty_sector, (xs & 3) | (zs & 3) << 2 | (ys & 3) << 4, (bx & 3) | (bz & 3) << 2 | (by & 3) << 4)
    fwd = forward_boxes()
    out = np.where(empty_sector, 1 << 5, 0).astype(np.uint32)
    for o in range(8):
        out |= skip_level(lm & fwd[li, o], li) << (15 + 2 * o)
    return out


def device_layout(data: v.SectorData) -> bytes:
    """Brick table + slot pools as the device holds them (slots in stream order).

    Derived here from the geometric definitions, independently of the device's bit
    tricks: an empty brick position skips to level 5 when its sector holds no brick,
    to 4 when the aligned 2x2x2 group of bricks around it is empty, else 3, stored as
    the alignment mask (1 << level) - 1; an empty voxel of an allocated brick skips to
    level 2 when its aligned 4^3 cell is empty, 1 when its aligned 2^3 block is, else 0,
    coded as the same mask (3, 1, 0); a solid voxel codes 2."""
    sx, sy, sz = data.sectors
    alloc = np.zeros((sy * 4, sz * 4, sx * 4), bool)          # (by, bz, bx)
    slot_of = np.zeros((sy * 4, sz * 4, sx * 4), np.uint32)
    slot = 0
    for idx, m in zip(data.sector_idx.tolist(), data.alloc_mask.tolist()):
        x, z, y = idx & 4095, (idx >> 12) & 4095, (idx >> 24) & 255
        for b in range(64):
            if m >> b & 1:
                bx, bz, by = x * 4 + (b & 3), z * 4 + ((b >> 2) & 3), y * 4 + (b >> 4)
                alloc[by, bz, bx] = True
                slot_of[by, bz, bx] = slot
                slot += 1
    sector_any = alloc.reshape(sy, 4, sz, 4, sx, 4).any(axis=(1, 3, 5))
    group_any = alloc.reshape(sy * 2, 2, sz * 2, 2, sx * 2, 2).any(axis=(1, 3, 5))
    up4 = lambda a: a.repeat(4, 0).repeat(4, 1).repeat(4, 2)
    up2 = lambda a: a.repeat(2, 0).repeat(2, 1).repeat(2, 2)
    level = np.where(~up4(sector_any), 31, np.where(~up2(group_any), 15, 7)).astype(np.uint32)
    # GLSL mode (bits 8-15): where the sector is empty, the 4th level over groups of 4^3
    # sectors: 127 when the whole group is empty, 63 when the aligned 2^3 block of
    # sectors is, else 31; elsewhere the same mask as bits 0-7
    py_, pz, px = (-sy) % 4, (-sz) % 4, (-sx) % 4
    sa = np.pad(sector_any, ((0, py_), (0, pz), (0, px)))
    gy, gz, gxx = sa.shape[0] // 4, sa.shape[1] // 4, sa.shape[2] // 4
    g4 = sa.reshape(gy, 4, gz, 4, gxx, 4).any(axis=(1, 3, 5)).repeat(4, 0).repeat(4, 1).repeat(4, 2)
    g2 = sa.reshape(gy * 2, 2, gz * 2, 2, gxx * 2, 2).any(axis=(1, 3, 5)).repeat(2, 0).repeat(2, 1).repeat(2, 2)
    g4, g2 = g4[:sy, :sz, :sx], g2[:sy, :sz, :sx]
    sector_level = np.where(~g4, 127, np.where(~g2, 63, 31)).astype(np.uint32)
    glsl = np.where(~up4(sector_any), up4(sector_level), level).astype(np.uint32)
    # anisotropic LODs (bit 5, bits 15-30): per ray octant, the skip level of the brick's
    # sector mask (or, in an empty sector, its sector-group mask) kept only on the 4^3 cells
    # from the brick (sector) towards the ray; bit 5 marks the group scale
    table = np.where(alloc, slot_of, np.uint32(0x80000000) | level | glsl << 8 | aniso_bits(alloc, sa)).astype(
        np.uint32)
    nb = data.n_bricks
    solid = data.bricks.reshape(nb, 8, 8, 8) != 0             # (n, y, z, x)
    cell_any = solid.reshape(nb, 2, 4, 2, 4, 2, 4).any(axis=(2, 4, 6))
    block_any = solid.reshape(nb, 4, 2, 4, 2, 4, 2).any(axis=(2, 4, 6))
    up = lambda a, k: a.repeat(k, 1).repeat(k, 2).repeat(k, 3)
    code = np.where(solid, 2, np.where(~up(cell_any, 4), 3, np.where(~up(block_any, 2), 1, 0))).astype(np.uint8)
    head = np.array([sx, sy, sz, nb], np.uint32).tobytes()
    # the raw masks the anisotropic LODs read on allocated bricks: 8 cell masks per slot
    # (cell cx | cz<<1 | cy<<2, bit vx + vz*4 + vy*16)
    bits = np.uint64(1) << np.arange(64, dtype=np.uint64)
    cv = solid.reshape(nb, 2, 4, 2, 4, 2, 4).transpose(0, 1, 3, 5, 2, 4, 6)  # (n, cy, cz, cx, vy, vz, vx)
    cells = (cv.reshape(nb, 8, 64).astype(np.uint64) * bits).sum(axis=2, dtype=np.uint64)
    # one code byte per voxel, x | z<<3 | y<<6 within the slot (the payload's order)
    return head + table.tobytes() + code.tobytes() + data.bricks.tobytes() + cells.tobytes()


def run(exe, tmp_path, data, rays, max_iters=128, wo=(0, 0, 0), glsl=False, coarse=False, aniso=False):
    (tmp_path / "w.bin").write_bytes(device_layout(data))
    np.ascontiguousarray(rays, v.RAY_DTYPE).tofile(tmp_path / "r.bin")
    subprocess.run([str(exe), str(tmp_path / "w.bin"), str(tmp_path / "r.bin"), str(tmp_path / "o.bin"),
                    str(max_iters), *map(str, wo), "1" if glsl else "0", "1" if coarse else "0",
                    "1" if aniso else "0"], check=True)
    return np.fromfile(tmp_path / "o.bin", v.HIT_DTYPE)


def oracle_for(data):
    o = OracleWorld(data.sectors)
    o.upload(data)
    return o


def test_random_rays_cfg0(exe, tmp_path):
    data = cfg0_world()
    rays = v.random_rays((256, 256, 256), seed=11, n=200_000)
    assert_hits_equal(run(exe, tmp_path, data, rays), oracle_for(data).cast(rays))


def test_dense_world_corner_rays(exe, tmp_path):
    rng = np.random.default_rng(12)
    vol = ((rng.random((64, 64, 64)) < 0.08) * rng.integers(1, 256, (64, 64, 64))).astype(np.uint8)
    data = dense_to_stream(vol)
    n = 40_000
    orig = rng.uniform(0, 6, (n, 3)).astype(np.float32)
    orig[n // 2:] = (rng.integers(0, 8, (n - n // 2, 3)) * 8 + rng.choice([0.0, 0.25, 7.75], (n - n // 2, 3)))
    rays = make_rays(orig, rng.normal(size=(n, 3)).astype(np.float32))
    assert_hits_equal(run(exe, tmp_path, data, rays), oracle_for(data).cast(rays))


@pytest.mark.parametrize("seed", [3, 4])
def test_mix_worlds_and_degenerate_rays(exe, tmp_path, seed):
    data = v.synth_mix(96, seed=seed)
    rng = np.random.default_rng(seed)
    rays = v.random_rays((96, 96, 96), seed=seed, n=60_000)
    d = rays["dir"]
    z = rng.random(d.shape) < 0.1
    d[z] = 0.0
    rays["dir"] = d
    rays["origin"][: 5000] = np.floor(rays["origin"][: 5000])
    for wo, iters in (((0, 0, 0), 128), ((5, -3, 7), 40)):
        r = rays.copy()
        r["origin"] -= np.asarray(wo, np.float32)
        assert_hits_equal(run(exe, tmp_path, data, r, iters, wo), oracle_for(data).cast(r, world_origin=wo,
                                                                                          max_iters=iters))


@pytest.mark.parametrize("seed", [5, 6])
def test_glsl_mode_against_oracle(exe, tmp_path, seed):
    """The GLSL-mode step (4th level from the brick table's bits 8-15, +5-ulp bias) on
    sparse and mixed worlds, from camera-like frames and from the world frame."""
    rng = np.random.default_rng(seed)
    vol = np.zeros((128, 320, 288), np.uint8)
    for _ in range(60):
        y, z, x = rng.integers(0, (128, 320, 288))
        vol[max(0, y - 5):y + 5, max(0, z - 5):z + 5, max(0, x - 5):x + 5] = rng.integers(1, 256)
    for data in (dense_to_stream(vol), v.synth_mix(96, seed=seed)):
        size = [s * 32 for s in data.sectors]
        o = oracle_for(data)
        eye = rng.uniform((0, 0, 0), size)
        wo = tuple(int(c) for c in np.floor(eye))
        d = rng.normal(size=(30_000, 3)).astype(np.float32)
        d[rng.random(d.shape) < 0.02] = 0.0
        rays = make_rays(np.tile((eye - np.floor(eye)).astype(np.float32), (30_000, 1)), d)
        assert_hits_equal(run(exe, tmp_path, data, rays, 256, wo, glsl=True),
                          o.cast(rays, world_origin=wo, max_iters=256, glsl=True))
        world_rays = v.random_rays(size, seed=seed, n=20_000)
        assert_hits_equal(run(exe, tmp_path, data, world_rays, 64, (0, 0, 0), glsl=True),
                          o.cast(world_rays, max_iters=64, glsl=True))
        # rayCastCoarse (the GPU renderer's shadow and bounce rays): 0.001 bias, coarse
        # hits from iteration 31, cap 96
        assert_hits_equal(run(exe, tmp_path, data, rays, 96, wo, glsl=True, coarse=True),
                          o.cast(rays, world_origin=wo, max_iters=96, glsl=True, coarse=True))
        # anisotropic LODs (raw masks restricted to the cells ahead of the ray), alone and
        # with rayCastCoarse
        # (the cast API caps a coarse ray at 96 iterations; this harness takes the cap as given)
        for coarse, cap in ((False, 256), (True, 96)):
            assert_hits_equal(run(exe, tmp_path, data, rays, cap, wo, glsl=True, coarse=coarse, aniso=True),
                              o.cast(rays, world_origin=wo, max_iters=cap, glsl=True, coarse=coarse, aniso=True))


def test_glsl_coarse_known_answer(exe, tmp_path):
    data = cell_corner_world()
    d = np.array([1.0, 1e-3, 1e-3], np.float32)
    rays = make_rays([[1.5, 0.5, 0.5], [1.5, 1.5, 0.5]], [d / np.linalg.norm(d)] * 2)
    got = run(exe, tmp_path, data, rays, 96, (0, 0, 0), glsl=True, coarse=True)
    assert_hits_equal(got, oracle_for(data).cast(rays, max_iters=96, glsl=True, coarse=True))
    assert tuple(v.unpack_voxel(got["voxel"][:1])[0]) == (67, 3, 3)
