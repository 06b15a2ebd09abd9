"""Builds oracle/_ref/libglsl_ref.so: the reference's traversal shaders
(src/VoxelRT/Shaders/VoxelTraversal.glsl with its include VoxelMap.glsl), compiled as
C++ against oracle/glsl_pin/glsl_shim.h.  Test infrastructure: the pin of the GLSL
traversal mode, run where the reference checkout exists.

The shader text is read in place and rewritten mechanically into oracle/_ref (never
into the repository) where GLSL syntax has no C++ spelling:
  * `#include "X"` is replaced by that file's text;
  * `layout(...)`, `readonly` and `uniform` qualifiers are dropped (uniforms become
    globals the driver sets);
  * a `buffer` block with an instance name becomes a struct variable, one without
    becomes its members at global scope (GLSL scoping), and an unsized array member
    becomes a pointer the driver points at its data;
  * `out T x` / `inout T x` parameters become references `T& x`;
  * float literals get the `f` suffix (GLSL literals are single precision).
The sizes the shader is compiled for (BRICK_SIZE, NUM_SECTORS_XZ, NUM_SECTORS_Y; the
reference sets them from its view size, GpuRenderer.cpp:9-14) are given per build.

Usage: python oracle/glsl_pin/build_glsl.py [reference checkout] [sectors_xz] [sectors_y]
"""
import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"


def rewrite(text: str, shader_dir: Path) -> str:
    text = re.sub(r'#include\s+"([^"]+)"', lambda m: (shader_dir / m.group(1)).read_text(), text)
    text = re.sub(r"\blayout\s*\([^)]*\)\s*", "", text)
    text = re.sub(r"\b(readonly|writeonly|uniform)\s+", "", text)
    # blocks without an instance name: their members live at global scope
    text = re.sub(r"\bbuffer\s+\w+\s*\{([^{}]*)\}\s*;", r"\1", text)
    text = re.sub(r"\bbuffer\s+(\w+)\s*\{", r"struct \1 {", text)
    text = re.sub(r"\b(\w+)\s+(\w+)\s*\[\s*\]\s*;", r"\1* \2;", text)
    text = re.sub(r"\b(?:inout|out)\s+(\w+)\s+(\w+)", r"\1& \2", text)
    text = re.sub(r"(?<![\w.])(\d+\.\d*|\.\d+)([eE][+-]?\d+)?(?![\w.])", r"\1\2f", text)
    return text


def main() -> None:
    ref_arg = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VRT_REFERENCE_DIR")
    if not ref_arg:
        sys.exit("usage: build_glsl.py <reference checkout> [sectors_xz sectors_y] (or $VRT_REFERENCE_DIR)")
    ref = Path(ref_arg)
    sxz = int(sys.argv[2]) if len(sys.argv) > 2 else 8
    sy = int(sys.argv[3]) if len(sys.argv) > 3 else 4
    shaders = ref / "src" / "VoxelRT" / "Shaders"
    OUT.mkdir(parents=True, exist_ok=True)
    gen = OUT / f"voxel_traversal_{sxz}x{sy}.inc"
    gen.write_text(rewrite((shaders / "VoxelTraversal.glsl").read_text(), shaders))
    lib = OUT / f"libglsl_ref_{sxz}x{sy}.so"
    cmd = ["g++", "-std=gnu++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-w",
           f"-DBRICK_SIZE=8", f"-DNUM_SECTORS_XZ={sxz}", f"-DNUM_SECTORS_Y={sy}", "-DTRAVERSAL_METRICS=0",
           f'-DGLSL_TRAVERSAL_SOURCE="{gen}"', "-I", str(HERE), str(HERE / "glsl_driver.cpp"),
           "-o", str(lib) + ".tmp"]
    subprocess.run(cmd, check=True)
    Path(str(lib) + ".tmp").rename(lib)
    print(lib)


if __name__ == "__main__":
    main()
