"""Shared test setup: the `gpu` marker, in-tree build, and seeded worlds."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from voxelrt_gb300 import build
    build.build_all()
    yield


def has_gpu() -> bool:
    try:
        import voxelrt_gb300 as v
        import ctypes as C
        d = v.capi.WorldDesc(1, 1, 1, 0, 0, 0)
        h = C.c_void_p()
        st = v.lib().vrt_world_create(C.byref(d), C.byref(h))
        if st == 0:
            v.lib().vrt_world_destroy(h)
        return st == 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    if not has_gpu():
        pytest.fail("no CUDA device: -m gpu tests need a GPU")
    return True
