#!/bin/sh
# Builds the oracle (CPU restatement of the reference path; test
# infrastructure) into oracle/liboracle.so. -ffp-contract=off keeps the
# arithmetic unfused on every host so results do not depend on FMA contraction.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
${CXX:-g++} -std=c++17 -O3 -fPIC -shared -fopenmp -ffp-contract=off \
  "$HERE/oracle_capi.cpp" -o "$HERE/liboracle.so"
echo "built $HERE/liboracle.so"
