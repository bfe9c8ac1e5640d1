#!/usr/bin/env bash
# Builds the reference library from its own sources, where they lie, into
# oracle/_ref/libparament_ref.so.  Used only to pin the oracle's host-side
# arithmetic (order tables, norm bound, error strings) against the reference;
# those entry points need no GPU.  Nothing is copied out of the reference tree.
#
# deviceInfo.c is left out: it reads cudaDeviceProp::memoryClockRate, a field
# that CUDA 13 removed, and it is not on the equiprop path.  No source is
# edited.  Usage: oracle/build_ref.sh <reference-root>, or with the root in
# $PARAMENT_REFERENCE_ROOT.
set -euo pipefail
REF=${1:-${PARAMENT_REFERENCE_ROOT:-}}
if [ -z "$REF" ]; then
    echo "usage: $0 <reference-root> (or set PARAMENT_REFERENCE_ROOT)" >&2
    exit 2
fi
SRC="$REF/src/cuda"
OUT="$(cd "$(dirname "$0")" && pwd)/_ref"
if [ ! -f "$SRC/parament.cpp" ]; then
    echo "reference sources not found under $SRC" >&2
    exit 1
fi
mkdir -p "$OUT"
nvcc -O2 -std=c++17 -shared -Xcompiler -fPIC -DPARAMENT_BUILD_DLL -DNDEBUG \
    -gencode arch=compute_103a,code=sm_103a \
    -I"$SRC" \
    "$SRC/parament.cpp" "$SRC/mathhelper.cpp" "$SRC/control_expansion.cu" "$SRC/diagonal_add.cu" \
    "$SRC/debugfuncs.cpp" "$SRC/printFuncs.cpp" \
    -lcublas -o "$OUT/libparament_ref.so"
echo "built $OUT/libparament_ref.so"
