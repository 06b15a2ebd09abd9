"""The device traversal step compiled for the host, against the oracle (no GPU).

tests/cpp/device_logic_test.cpp includes voxelrt_gb300/csrc/trace_core.cuh with the
CUDA rounding intrinsics mapped to IEEE host operations; the worlds are laid out
exactly as the device stores them (sector records, brick-slot pools).  Every record
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
    """Sector table + slot pools as the device holds them (sectors in stream order)."""
    sx, sy, sz = data.sectors
    table = np.zeros((sx * sy * sz, 4), np.uint32)
    nb = data.n_bricks
    occ = np.zeros((nb, 8), np.uint64)
    slot = 0
    for idx, m in zip(data.sector_idx.tolist(), data.alloc_mask.tolist()):
        x, z, y = idx & 4095, (idx >> 12) & 4095, (idx >> 24) & 255
        s = x + z * sx + y * sx * sz
        table[s] = [m & 0xFFFFFFFF, m >> 32, slot, 0]
        slot += bin(m).count("1")
    # cell masks: bit vx + vz*4 + vy*16 of cell cx | cz<<1 | cy<<2
    b = data.bricks.reshape(nb, 8, 8, 8) != 0  # (y, z, x)
    for c in range(8):
        cx, cz, cy = c & 1, (c >> 1) & 1, c >> 2
        cell = b[:, cy * 4:cy * 4 + 4, cz * 4:cz * 4 + 4, cx * 4:cx * 4 + 4]  # (n, vy, vz, vx)
        bits = cell.reshape(nb, 64).astype(np.uint64)
        occ[:, c] = (bits << np.arange(64, dtype=np.uint64)).sum(axis=1, dtype=np.uint64)
    head = np.array([sx, sy, sz, len(table), nb], np.uint32).tobytes()
    return head + table.tobytes() + occ.tobytes() + data.bricks.tobytes()


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
