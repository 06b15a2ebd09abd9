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
from tests.helpers import assert_hits_equal, cfg0_world, dense_to_stream, make_rays

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "device_logic_test.cpp"
EXE = ROOT / "tests" / "cpp" / "_build" / "device_logic_test"


@pytest.fixture(scope="module")
def exe():
    EXE.parent.mkdir(exist_ok=True)
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-I", str(ROOT / "include"),
                    str(SRC), "-o", str(EXE)], check=True)
    return EXE


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
    table = np.where(alloc, slot_of, np.uint32(0x80000000) | level).astype(np.uint32)
    nb = data.n_bricks
    solid = data.bricks.reshape(nb, 8, 8, 8) != 0             # (n, y, z, x)
    cell_any = solid.reshape(nb, 2, 4, 2, 4, 2, 4).any(axis=(2, 4, 6))
    block_any = solid.reshape(nb, 4, 2, 4, 2, 4, 2).any(axis=(2, 4, 6))
    up = lambda a, k: a.repeat(k, 1).repeat(k, 2).repeat(k, 3)
    code = np.where(solid, 2, np.where(~up(cell_any, 4), 3, np.where(~up(block_any, 2), 1, 0))).astype(np.uint32)
    code = code.reshape(nb, 32, 16)                          # voxel x | z<<3 | y<<6 -> word, position
    words = (code << (2 * np.arange(16, dtype=np.uint32))).sum(axis=2, dtype=np.uint64).astype(np.uint32)
    head = np.array([sx, sy, sz, nb], np.uint32).tobytes()
    return head + table.tobytes() + words.tobytes() + data.bricks.tobytes()


def run(exe, tmp_path, data, rays, max_iters=128, wo=(0, 0, 0)):
    (tmp_path / "w.bin").write_bytes(device_layout(data))
    np.ascontiguousarray(rays, v.RAY_DTYPE).tofile(tmp_path / "r.bin")
    subprocess.run([str(exe), str(tmp_path / "w.bin"), str(tmp_path / "r.bin"), str(tmp_path / "o.bin"),
                    str(max_iters), *map(str, wo)], check=True)
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
