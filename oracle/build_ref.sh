#!/bin/sh
# Builds the reference's own gravity headers, unmodified and read from where
# they lie, into oracle/_ref/libvipp_ref.so behind the test shim ref_shim.cpp.
# Test infrastructure only (golden fixtures, oracle validation). The reference
# tree is only present in the development container; elsewhere this is a no-op.
# CMake is bypassed: the reference's CMakeLists hard-codes clang/libc++ and a
# network googletest fetch. The headers rely on transitive std includes, which
# are force-included here.
set -e
REF="${VIPP_REFERENCE_DIR:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ ! -d "$REF/gravity/include" ]; then
  echo "reference sources not present; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$HERE/_ref"
${CXX:-g++} -std=c++17 -O2 -fPIC -shared -fopenmp -ffp-contract=off \
  -include vector -include cmath -include complex -include optional -include tuple \
  -include chrono -include functional -include algorithm -include iterator -include limits \
  -include variant -include stdexcept \
  -I"$REF/gravity/include" "$HERE/ref_shim.cpp" -o "$HERE/_ref/libvipp_ref.so"
# where the sources were read, for the tests that compile against the reference's headers
echo "$REF" > "$HERE/_ref/REFERENCE_DIR"
echo "built $HERE/_ref/libvipp_ref.so"
