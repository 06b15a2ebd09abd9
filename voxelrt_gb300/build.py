"""Build recipe for libvrt.so (sm_103a CUDA + host C++) and the CPU oracle.

Run as ``python -m voxelrt_gb300.build`` or through ``__graft_entry__.build()``.
Translation units compile in parallel; outputs stay in-tree:

* ``voxelrt_gb300/_lib/libvrt.so`` - the product library (C ABI of include/vrt.h);
* ``voxelrt_gb300/_lib/libvrt_synth.so`` - host-only generators of seeded worlds, cameras
  and rays (include/vrt_synth.h), for tests and the benchmark; no CUDA;
* ``oracle/_build/libvrt_oracle.so`` - the CPU oracle, a test/benchmark checker.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "voxelrt_gb300"
CSRC = PKG / "csrc"
LIB_DIR = PKG / "_lib"
OBJ_DIR = PKG / "_build"
LIBVRT = LIB_DIR / "libvrt.so"
LIBSYNTH = LIB_DIR / "libvrt_synth.so"
# host sources of the synthetic-input library (and nothing of it goes into libvrt.so)
SYNTH_SRC = ["synth.cpp"]
SHARED_HOST_SRC = ["host_common.cpp"]
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "libvrt_oracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off"]
# Host code must give identical results on x86-64 and arm64: no -march, no FMA contraction.
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-pthread", "-Wall"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    nvcc = _nvcc()
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted(p for p in CSRC.glob("*.cpp") if p.name not in SYNTH_SRC)
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    jobs = []
    objs = []
    for src in cu + cpp:
        obj = OBJ_DIR / (src.name + ".o")
        objs.append(obj)
        if not force and not _stale(obj, [src] + headers):
            continue
        if src.suffix == ".cu":
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj)]
        else:
            cmd = ["g++", *CXX_FLAGS, "-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj)]
        jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, _ in zip(jobs, ex.map(_run, jobs)):
            if verbose:
                print(" ".join(cmd))
    if force or jobs or _stale(LIBVRT, objs):
        tmp = LIBVRT.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", str(tmp), *map(str, objs), "-lpthread"])
        os.replace(tmp, LIBVRT)
    return LIBVRT


def build_synth(force: bool = False) -> Path:
    srcs = [CSRC / n for n in SYNTH_SRC + SHARED_HOST_SRC]
    deps = srcs + sorted(CSRC.glob("*.h")) + sorted((ROOT / "include").glob("*.h"))
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    if force or _stale(LIBSYNTH, deps):
        tmp = LIBSYNTH.with_suffix(".so.tmp")
        _run(["g++", *CXX_FLAGS, "-shared", "-I", str(ROOT / "include"), "-o", str(tmp), *map(str, srcs)])
        os.replace(tmp, LIBSYNTH)
    return LIBSYNTH


def build_oracle(force: bool = False) -> Path:
    src = ORACLE_DIR / "vrt_oracle.cpp"
    deps = [src, ORACLE_DIR / "vrt_oracle.h", ROOT / "include" / "vrt.h"]
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    if force or _stale(ORACLE_LIB, deps):
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        _run(["g++", *CXX_FLAGS, "-shared", "-o", str(tmp), str(src)])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_all(force: bool = False, verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_library, force, verbose), ex.submit(build_oracle, force), ex.submit(build_synth, force)]
        for f in futs:
            f.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIBVRT)
    print(LIBSYNTH)
    print(ORACLE_LIB)
