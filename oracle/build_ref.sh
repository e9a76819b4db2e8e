#!/bin/sh
# Build the reference's own solver headers (darcy-cpp v1.0.0, header-only
# C++17 + OpenMP) into oracle/_ref/libdarcy_ref.so through the small C-ABI shim
# oracle/ref_driver.cpp. Needs the reference checkout (REF, default
# /root/reference); nothing is copied from it. Flags follow the reference's
# CMakeLists.txt:64-65 (-O3 -fno-math-errno, C++17 without extensions).
set -e
REF=${REF:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
if [ ! -f "$REF/include/darcy/solver.hpp" ]; then
  echo "reference headers not found under $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$HERE/_ref"
g++ -O3 -fno-math-errno -std=c++17 -fopenmp -fPIC -shared -I"$REF/include" \
    "$HERE/ref_driver.cpp" -o "$HERE/_ref/libdarcy_ref.so"
echo "built $HERE/_ref/libdarcy_ref.so"
