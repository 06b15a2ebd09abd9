"""The batch planner of libvrt.so on the host (no GPU).

tests/cpp/plan_test.cpp links the product library and calls its planner: the launch-config
fields a caller leaves to the library (refill threshold and chunk size follow the views and
the grid), the tile-queue and record layout of ragged views, and the planner's refusals.
"""
import subprocess
from pathlib import Path

import pytest

from voxelrt_gb300 import build

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "plan_test.cpp"
EXE = ROOT / "tests" / "cpp" / "_build" / "plan_test"


def cuda_include() -> Path | None:
    """The CUDA runtime headers next to nvcc (batch_internal.h includes cuda_runtime.h)."""
    try:
        inc = Path(build._nvcc()).resolve().parent.parent / "include"
    except RuntimeError:
        return None
    return inc if (inc / "cuda_runtime.h").exists() else None


def test_planner_defaults_and_layout():
    inc = cuda_include()
    if inc is None:
        pytest.skip("CUDA runtime headers not found")
    lib = build.build_library()
    EXE.parent.mkdir(exist_ok=True)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"), "-I", str(build.CSRC), "-I", str(inc),
                    str(SRC), "-L", str(lib.parent), "-lvrt", f"-Wl,-rpath,{lib.parent}", "-o", str(EXE)],
                   check=True)
    res = subprocess.run([str(EXE)], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "ok: 0 failures" in res.stdout
