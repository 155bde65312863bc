#!/bin/sh
# Builds oracle/_ref/libref_cubature.so from HyperFox's own Cubature.cpp and
# ErrorHandle.cpp where they lie in the HyperFox source tree (first argument,
# default /root/reference). Only the cubature part of the reference builds
# without external libraries; ReferenceElement needs Eigen and Boost.Math.
set -e
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
[ -f "$REF/src/element/Cubature.cpp" ] || { echo "no HyperFox tree at $REF; skipping"; exit 0; }
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++17 -shared -fPIC -I"$REF/src/element" -I"$REF/src/globals" \
    "$HERE/ref_cubature_shim.cpp" "$REF/src/element/Cubature.cpp" "$REF/src/globals/ErrorHandle.cpp" \
    -o "$HERE/_ref/libref_cubature.so"
echo "built $HERE/_ref/libref_cubature.so"
