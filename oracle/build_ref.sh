#!/usr/bin/env bash
# Builds the reference's own StatTile arithmetic (src/statistics/estimator.h of
# the reference tree, read in place and never copied) into oracle/_ref/ with the
# stand-in headers of oracle/ref_shim/. Four variants, matching the reference's
# build switches: Float = float / double (PBRT_FLOAT_AS_DOUBLE, src/core/pbrt.h:169)
# and the single Box-Cox build / the multi-transform build (FULL_MULTI_TRANSFORM=1,
# scripts/alternate-builds/build-mt.sh). -ffp-contract=off keeps every operation
# separately rounded, as on the reference's x86 builds.
# Test infrastructure only: the outputs are used to generate tests/golden/.
set -euo pipefail
REF=${STATER_REFERENCE:-/root/reference}
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/src/statistics/estimator.h" ]; then
  echo "reference tree not found at $REF; nothing to build" >&2
  exit 0
fi
mkdir -p "$OUT"
CXX=${CXX:-g++}
FLAGS="-std=c++17 -O2 -fPIC -shared -ffp-contract=off -I$HERE/ref_shim -I$REF/src/statistics"
$CXX $FLAGS                                              "$HERE/ref_harness.cpp" -o "$OUT/libref_f32.so"
$CXX $FLAGS -DPBRT_FLOAT_AS_DOUBLE                       "$HERE/ref_harness.cpp" -o "$OUT/libref_f64.so"
$CXX $FLAGS -DFULL_MULTI_TRANSFORM=1                     "$HERE/ref_harness.cpp" -o "$OUT/libref_mt_f32.so"
$CXX $FLAGS -DFULL_MULTI_TRANSFORM=1 -DPBRT_FLOAT_AS_DOUBLE "$HERE/ref_harness.cpp" -o "$OUT/libref_mt_f64.so"
echo "built $OUT"
