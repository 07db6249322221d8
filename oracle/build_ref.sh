#!/bin/sh
# Compile the reference's own CPU spot-finder sources IN PLACE (they are not
# copied into this repository) together with oracle/ref_shim.cc into
# oracle/_ref/libref.so. Validation and fixture generation only.
#
# Usage: oracle/build_ref.sh [reference-root]   (default /root/reference)
# Exits 0 without building when the reference tree is absent.
set -eu
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
if [ ! -f "$REF/src/spots/dext.cc" ]; then
  echo "build_ref: no reference tree at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$HERE/_ref"
# ISO C++20 with contraction off, as the reference's own build
# (CMakeLists.txt:8-10 sets CMAKE_CXX_EXTENSIONS OFF).
g++ -std=c++20 -O2 -ffp-contract=off -fPIC -shared \
  -I"$REF/src/spots" -I"$REF/tests/spots" \
  "$REF/src/spots/dext.cc" "$REF/src/spots/dials_spots.cc" \
  "$REF/src/spots/signal_order.cc" "$REF/src/spots/refl.cc" \
  "$HERE/ref_shim.cc" -o "$HERE/_ref/libref.so.tmp"
mv "$HERE/_ref/libref.so.tmp" "$HERE/_ref/libref.so"
echo "build_ref: built $HERE/_ref/libref.so"
