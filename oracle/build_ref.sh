#!/bin/sh
# Builds the reference's own STSC skycube (HybridCube + MommyQ + lattice
# utilities) from the reference checkout, unmodified, into oracle/_ref/.
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
# Needs an x86-64 host with AVX2 (the reference's dominance tests use AVX
# intrinsics when __AVX__ is defined). Nothing is written outside oracle/_ref.
set -e
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -f "$REF/src/stsc/HybridCube.cpp" ] || { echo "reference sources not found at $REF" >&2; exit 2; }
mkdir -p "$OUT"
CXXFLAGS="-O3 -std=c++17 -fopenmp -mavx2 -fPIC -w -include cstdint -include cmath -include cstring -I$HERE/ref_shim -I$REF/src"
g++ $CXXFLAGS -shared -o "$OUT/libskycube_ref.so" \
  "$HERE/ref_driver.cpp" \
  "$REF/src/stsc/HybridCube.cpp" \
  "$REF/src/hybrid/mommyq.cpp" \
  "$REF/src/utilities/lattice_utilities.cpp"
echo "built $OUT/libskycube_ref.so"
