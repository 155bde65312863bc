#!/bin/sh
# Builds oracle/_ref/libref_cubature.so from HyperFox's own Cubature.cpp and
# ErrorHandle.cpp where they lie in the HyperFox source tree (first argument,
# else $HYPERFOX_REFERENCE). Only the cubature part of the reference builds
# without external libraries; ReferenceElement needs Eigen and Boost.Math.
# Also records the tree's location in oracle/_ref/REFERENCE_ROOT, where the
# host-only tests that read the reference's mesh fixtures find it.
set -e
REF=${1:-$HYPERFOX_REFERENCE}
[ -n "$REF" ] || { echo "no HyperFox tree given (argument or HYPERFOX_REFERENCE); skipping"; exit 0; }
HERE=$(cd "$(dirname "$0")" && pwd)
[ -f "$REF/src/element/Cubature.cpp" ] || { echo "no HyperFox tree at $REF; skipping"; exit 0; }
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++17 -shared -fPIC -I"$REF/src/element" -I"$REF/src/globals" \
    "$HERE/ref_cubature_shim.cpp" "$REF/src/element/Cubature.cpp" "$REF/src/globals/ErrorHandle.cpp" \
    -o "$HERE/_ref/libref_cubature.so"
printf '%s\n' "$REF" > "$HERE/_ref/REFERENCE_ROOT"
echo "built $HERE/_ref/libref_cubature.so"
