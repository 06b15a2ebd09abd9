#!/bin/sh
# Builds oracle/_ref/libvrt_ref.so from the reference's own sources, in place, with
# the shim headers of oracle/ref_pin/shim.  x86-64 with AVX-512 only (the reference's
# SIMD layer supports nothing else); run where the reference checkout exists.
# Float semantics: no -ffast-math and no FMA contraction (the reading the oracle pins).
# The world-file framing (src/LibGlimpsw/Common/BinaryIO.cpp) compiles in place too and
# links the system's libzstd.so.1 (its header is the declaration stand-in in shim/zstd.h);
# without that library the build falls back to no world-file support.
set -e
REF=${1:-$VRT_REFERENCE_DIR}
if [ -z "$REF" ]; then
    echo "usage: build_ref.sh <reference checkout> (or set VRT_REFERENCE_DIR)" >&2
    exit 2
fi
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/../_ref"
mkdir -p "$OUT"
ZSTD=${VRT_ZSTD_LIB:-$(ldconfig -p 2>/dev/null | awk '/libzstd\.so\.1 /{print $NF; exit}')}
if [ -n "$ZSTD" ] && [ -f "$ZSTD" ]; then
    IO="$REF/src/LibGlimpsw/Common/BinaryIO.cpp $ZSTD"
    IO_DEF=-DVRT_REF_BINARY_IO=1
else
    IO=""
    IO_DEF=-DVRT_REF_BINARY_IO=0
fi
g++ -std=gnu++20 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -w \
    -mavx512f -mavx512cd -mavx512bw -mavx512dq -mavx512vl -mavx512vbmi -mavx512vpopcntdq -mavx512bitalg \
    -mgfni -mfma -mbmi -mbmi2 -mlzcnt -mpopcnt -mf16c $IO_DEF \
    -I "$HERE/shim" -I "$REF/src/LibGlimpsw" -iquote "$REF/src/VoxelRT" \
    "$HERE/ref_driver.cpp" $IO -o "$OUT/libvrt_ref.so.tmp"
mv "$OUT/libvrt_ref.so.tmp" "$OUT/libvrt_ref.so"
echo "$OUT/libvrt_ref.so"
