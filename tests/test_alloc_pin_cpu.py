"""The host brick-slot allocator pinned to the reference's own BrickSlotAllocator (no GPU).

tests/golden/refalloc.npz holds seeded runs of sector edits through the reference's
BrickSlotAllocator / FreeList (src/VoxelRT/BrickSlotAllocator.cpp:5-94), compiled in place
by tests/golden/make_golden_alloc.py: the base slot and allocation mask of the edited sector
after every op, and the free ranges at the end.  tests/cpp/freelist_test.cpp runs the same
ops through libvrt.so's FreeList, sector_alloc and sector_free, the allocator of bulk syncs
(best fit, grow in place when the next free range is strictly larger, coalescing frees).
Every placement must be the reference's.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from voxelrt_gb300 import build

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "freelist_test.cpp"
EXE = ROOT / "tests" / "cpp" / "_build" / "freelist_test"
GOLDEN = ROOT / "tests" / "golden" / "refalloc.npz"
RUNS = ("small", "medium", "large")


@pytest.fixture(scope="module")
def exe():
    lib = build.build_library()
    EXE.parent.mkdir(exist_ok=True)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(build.CSRC), str(SRC), "-L", str(lib.parent), "-lvrt",
                    f"-Wl,-rpath,{lib.parent}", "-o", str(EXE)], check=True)
    return EXE


def run_ours(exe, tmp_path, g):
    ops = tmp_path / "ops.bin"
    res = tmp_path / "res.bin"
    with open(ops, "wb") as f:
        np.array([len(RUNS)], np.uint32).tofile(f)
        for name in RUNS:
            n = len(g[f"{name}_sector"])
            np.array([*g[f"{name}_bounds"], n], np.uint32).tofile(f)
            g[f"{name}_sector"].astype(np.uint32).tofile(f)
            g[f"{name}_add"].astype(np.uint64).tofile(f)
            g[f"{name}_remove"].astype(np.uint64).tofile(f)
    subprocess.run([str(exe), str(ops), str(res)], check=True)
    buf = res.read_bytes()
    out, off = {}, 0
    for name in RUNS:
        n = len(g[f"{name}_sector"])
        base = np.frombuffer(buf, np.uint32, n, off)
        off += 4 * n
        mask = np.frombuffer(buf, np.uint64, n, off)
        off += 8 * n
        nr = int(np.frombuffer(buf, np.uint32, 1, off)[0])
        off += 4
        ranges = np.frombuffer(buf, np.uint32, 2 * nr, off).reshape(-1, 2)
        off += 8 * nr
        failed = int(np.frombuffer(buf, np.uint32, 1, off)[0])
        off += 4
        out[name] = (base, mask, ranges, failed)
    assert off == len(buf)
    return out


def test_slot_placements_match_the_reference(exe, tmp_path):
    g = np.load(GOLDEN)
    ours = run_ours(exe, tmp_path, g)
    for name in RUNS:
        base, mask, ranges, failed = ours[name]
        n = len(g[f"{name}_sector"])
        assert n > 0 and failed == n, name
        assert np.array_equal(mask, g[f"{name}_mask"]), name
        bad = np.nonzero(base != g[f"{name}_base"])[0]
        assert bad.size == 0, f"{name}: first differing op {bad[:1]}"
        assert np.array_equal(ranges, g[f"{name}_ranges"]), name


def test_the_runs_exercise_the_allocator():
    """The fixture covers growth in place, moves to a best-fit range, frees to empty and a
    fragmented end state, not only appends."""
    g = np.load(GOLDEN)
    moved = grown_in_place = emptied = 0
    for name in RUNS:
        sec, base, mask = g[f"{name}_sector"], g[f"{name}_base"], g[f"{name}_mask"]
        last = {}
        for s, b, m in zip(sec, base, mask):
            prev = last.get(int(s))
            if prev is not None and prev[0] and b:
                if b != prev[0]:
                    moved += 1
                elif bin(int(m)).count("1") > bin(int(prev[1])).count("1"):
                    grown_in_place += 1
            if prev is not None and prev[0] and not b:
                emptied += 1
            last[int(s)] = (int(b), int(m))
        assert len(g[f"{name}_ranges"]) > 1, name
    assert moved > 50 and grown_in_place > 50 and emptied > 20, (moved, grown_in_place, emptied)
