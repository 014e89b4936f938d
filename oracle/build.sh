#!/bin/sh
# Builds the C oracle (test infrastructure) into oracle/_build/liboracle.so.
# Portable C11 + OpenMP: builds the same on x86-64 and aarch64.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$HERE/_build"
${CC:-gcc} -O3 -std=c11 -fopenmp -fPIC -shared -o "$HERE/_build/liboracle.so" "$HERE/skycube_oracle.c"
