#!/usr/bin/env bash
# Builds oracle/_ref/libpdref.so from the reference's own kernel source, and
# oracle/_ref/libpdscene.so from the reference's example Scene (OBJ reading,
# mesh fill with mesh_query0.1's inside test).
# TEST INFRASTRUCTURE ONLY: the library is a checker for the oracle
# restatement (pd_oracle.c) and the source of tests/golden/ fixtures.
#
# The kernel text is streamed from the reference tree straight into the
# compiler (nothing is copied to disk); the reference headers are included in
# place with -I.  Line ranges (paths inside the reference project):
#   src/core/cg_solver.cuh:26-383      device helpers, calculatePDForceDerivative, computeAx
#   src/core/implicit_euler.cuh:18-179 fillMatrix/fillVectorB/updatePosition (implicit Euler)
#   src/core/newmark_beta.cuh:18-201   fillMatrix/fillVectorB/updateVelocity/updatePosition (Newmark)
#   src/core/simulator.cu:802-822      frand, getstretch
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default: $PD_REFERENCE_ROOT; no
# machine-specific default: without either the script exits 3)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${PD_REFERENCE_ROOT:-}}"
if [ -z "$REF" ]; then
  echo "build_ref.sh: give the reference root as an argument or in PD_REFERENCE_ROOT" >&2
  exit 3
fi
CORE="$REF/src/core"
if [ ! -f "$CORE/cg_solver.cuh" ]; then
  echo "build_ref.sh: reference source not found under $REF" >&2
  exit 3
fi
CUDA_INC="${CUDA_HOME:-/usr/local/cuda}/include"
OUT="$HERE/_ref"
mkdir -p "$OUT"
{
  cat "$HERE/ref_shim.h"
  echo '#line 26 "src/core/cg_solver.cuh"'
  sed -n '26,383p' "$CORE/cg_solver.cuh"
  echo '#line 18 "src/core/implicit_euler.cuh"'
  sed -n '18,179p' "$CORE/implicit_euler.cuh"
  echo '#line 18 "src/core/newmark_beta.cuh"'
  sed -n '18,201p' "$CORE/newmark_beta.cuh"
  echo '#line 802 "src/core/simulator.cu"'
  sed -n '802,822p' "$CORE/simulator.cu"
  echo '#line 1 "oracle/ref_driver.cpp"'
  cat "$HERE/ref_driver.cpp"
} | g++ -std=c++17 -O2 -ffp-contract=off -fopenmp -fPIC -shared -w \
      -I"$CORE" -I"$CUDA_INC" -x c++ - -o "$OUT/libpdref.so"
echo "built $OUT/libpdref.so"
# The example Scene: compiled as it lies in the reference tree.  Monitor's
# CUDA-event code is not needed; helper_cuda.h (which no longer compiles
# against CUDA 13's cudaDeviceProp) is kept out through its include guard.
EX="$REF/src/examples"
MQ="$EX/mesh_query0.1"
g++ -std=c++17 -O2 -ffp-contract=off -fPIC -shared -w -DHELPER_CUDA_H \
    -include cstring -include vector -include cuda_runtime_api.h \
    -I"$REF/src" -I"$CORE" -I"$EX" -I"$CUDA_INC" \
    "$EX/scene.cpp" "$MQ/mesh_query.cpp" "$MQ/predicates.cpp" "$MQ/bounding_box_tree.cpp" \
    "$HERE/ref_scene_driver.cpp" -o "$OUT/libpdscene.so"
echo "built $OUT/libpdscene.so"
