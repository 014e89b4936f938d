#!/bin/sh
# Builds the reference's own STSC skycube (HybridCube + MommyQ + lattice
# utilities) from unmodified reference sources into oracle/_ref/. Test
# infrastructure and the CPU reference arm of bench.py, never the product.
#
# Usage:
#   oracle/build_ref.sh [--shim] [REFERENCE_ROOT]
#       REFERENCE_ROOT: a reference checkout; default $SKC_REFERENCE_ROOT,
#       else the staged copy in oracle/_ref/src (see --stage).
#       On an x86-64 host the reference builds as it ships, with its AVX
#       dominance tests (-mavx2) -> oracle/_ref/libskycube_ref.so.
#       On any other host (the aarch64 GPU hosts), or with --shim, the same
#       sources build with __AVX__ defined and oracle/ref_shim/immintrin.h (a
#       portable definition of the eight intrinsics the reference uses) on
#       the include path. On x86-64, --shim writes
#       oracle/_ref/libskycube_ref_shim.so instead, so the two builds can be
#       compared (tests/test_oracle.py).
#   oracle/build_ref.sh --pq [REFERENCE_ROOT]
#       The reference's PQSkycube (ExecuteQSkycubeGLPMR, src/qskycube/) with
#       oracle/ref_pq_driver.cpp -> oracle/_ref/libskycube_ref_pq.so: a
#       second reference algorithm the CPU tests check skylines against
#       (portable C++, no intrinsics).
#   oracle/build_ref.sh --stage [REFERENCE_ROOT]
#       (default $SKC_REFERENCE_ROOT, else /root/reference)
#       Copies the reference files these builds read into
#       oracle/_ref/src (git-ignored), so a host without the checkout can
#       build them. Nothing outside oracle/_ref is written.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
FILES="src/stsc/HybridCube.cpp src/stsc/HybridCube.h src/hybrid/mommyq.cpp src/hybrid/mommyq.h
src/skycube/Hashcube.h src/skycube/NodeAuxilliary.h src/skycube/Skycube.h
src/utilities/SubTuple.h src/utilities/common2.h src/utilities/dt_avx2.h
src/utilities/pq_filter.h src/utilities/lattice_utilities.h src/utilities/lattice_utilities.cpp
src/qskycube/BSkyTreeEM.cc src/qskycube/BSkyTreeEM.h src/qskycube/BSkyTreeP.cc src/qskycube/BSkyTreeP.h
src/qskycube/Common.cc src/qskycube/Common.h src/qskycube/PivotSelection.cc src/qskycube/PivotSelection.h
src/qskycube/QSkycube.h src/qskycube/QSkycubeG.h src/qskycube/SkyTreeUtil.cc src/qskycube/SkyTreeUtil.h"

if [ "$1" = "--stage" ]; then
  REF=${2:-${SKC_REFERENCE_ROOT:-/root/reference}}
  [ -f "$REF/src/stsc/HybridCube.cpp" ] || { echo "reference sources not found at $REF" >&2; exit 2; }
  for f in $FILES; do
    mkdir -p "$OUT/src/$(dirname "$f")"
    cp "$REF/$f" "$OUT/src/$(dirname "$f")/"
  done
  echo "staged reference sources in $OUT/src"
  exit 0
fi

if [ "$1" = "--pq" ]; then
  REF=${2:-${SKC_REFERENCE_ROOT:-$OUT/src}}
  [ -f "$REF/src/qskycube/QSkycubeG.h" ] || { echo "reference QSkycube sources not found at $REF" >&2; exit 2; }
  CXXFLAGS="-O2 -std=c++17 -fopenmp -fPIC -w -include cstdint -include cmath -include cstring -include bitset -include cassert -I$HERE/ref_shim -I$REF/src"
  OBJ="$OUT/obj_libskycube_ref_pq.so"
  mkdir -p "$OBJ"
  pids=""
  for src in "$HERE/ref_pq_driver.cpp" "$REF"/src/qskycube/*.cc; do
    g++ $CXXFLAGS -c "$src" -o "$OBJ/$(basename "$src" | sed 's/\.c[cp]*$//').o" &
    pids="$pids $!"
  done
  rc=0
  for p in $pids; do wait "$p" || rc=1; done
  [ $rc = 0 ] || { echo "reference PQSkycube build failed" >&2; exit 1; }
  g++ -shared -fopenmp -o "$OUT/libskycube_ref_pq.so" "$OBJ"/*.o
  echo "built $OUT/libskycube_ref_pq.so"
  exit 0
fi

SHIM=0
if [ "$1" = "--shim" ]; then SHIM=1; shift; fi
REF=${1:-${SKC_REFERENCE_ROOT:-$OUT/src}}
[ -f "$REF/src/stsc/HybridCube.cpp" ] || { echo "reference sources not found at $REF" >&2; exit 2; }

NAME=libskycube_ref.so
case "$(uname -m)" in
  x86_64)
    if [ $SHIM = 1 ]; then NAME=libskycube_ref_shim.so; fi ;;
  *) SHIM=1 ;;
esac
if [ $SHIM = 1 ]; then
  ARCHFLAGS="-D__AVX__=1 -I$HERE/ref_shim"
else
  ARCHFLAGS="-mavx2"
fi
CXXFLAGS="-O3 -std=c++17 -fopenmp -fPIC -w $ARCHFLAGS -include cstdint -include cmath -include cstring -I$HERE/ref_shim -I$REF/src"

OBJ="$OUT/obj_$NAME"
mkdir -p "$OBJ"
# The four translation units compile in parallel.
pids=""
for src in "$HERE/ref_driver.cpp" "$REF/src/stsc/HybridCube.cpp" "$REF/src/hybrid/mommyq.cpp" \
           "$REF/src/utilities/lattice_utilities.cpp"; do
  o="$OBJ/$(basename "$src" .cpp).o"
  g++ $CXXFLAGS -c "$src" -o "$o" &
  pids="$pids $!"
done
rc=0
for p in $pids; do wait "$p" || rc=1; done
[ $rc = 0 ] || { echo "reference STSC build failed" >&2; exit 1; }
g++ -shared -fopenmp -o "$OUT/$NAME" "$OBJ"/*.o
echo "built $OUT/$NAME ($( [ $SHIM = 1 ] && echo portable intrinsics || echo AVX2 ))"
