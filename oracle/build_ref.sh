#!/usr/bin/env bash
# Builds oracle/_ref/ from the reference sources where they lie (never copied):
#   libreflbm_f32.so / libreflbm_f64.so  reference kernels + set-up, run on the
#                                        CPU through ref_shim/ (test oracle pin)
#   latticegen                           the reference lattice generator
#   libref_multiphase.so                 the reference's serial CPU colour-
#                                        gradient functions (Multiphase.cu)
# TEST INFRASTRUCTURE ONLY.  Usage: oracle/build_ref.sh [reference-root]
# Exits 0 without building when the reference tree is absent.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${THESIS_REFERENCE_ROOT:-/root/reference}}"
S="$REF/Source code/lbm-solver_final"
G="$REF/Source code/latticegen2_W8"
OUT="$HERE/_ref"
if [ ! -d "$S" ]; then
  echo "build_ref: reference tree not found at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
CUDA_INC="${CUDA_HOME:-/usr/local/cuda}/include"
SRCS=(GpuInit GpuCollision GpuStream GpuBoundaries GpuUpdateMacro CellFunctions)
build_solver() {  # $1 = suffix, $2 = extra define
  local tmp; tmp="$(mktemp -d)"
  local objs=()
  for s in "${SRCS[@]}"; do
    "$CXX" -x c++ -std=c++17 -O2 -fPIC -w $2 -include "$HERE/ref_shim/cuda_host_shim.h" \
      -I"$S/include" -I"$CUDA_INC" -c "$S/$s.cu" -o "$tmp/$s.o" &
    objs+=("$tmp/$s.o")
  done
  "$CXX" -x c++ -std=c++17 -O2 -fPIC -w $2 -include "$HERE/ref_shim/cuda_host_shim.h" \
    -I"$S/include" -I"$CUDA_INC" -c "$HERE/ref_shim/ref_harness.cpp" -o "$tmp/harness.o" &
  wait
  "$CXX" -shared -o "$OUT/libreflbm_$1.so" "${objs[@]}" "$tmp/harness.o" -lm
  rm -rf "$tmp"
}
build_solver f32 ""
build_solver f64 "-DUSE_DOUBLE"
# reference lattice generator, built from its own sources
tmp="$(mktemp -d)"
( cd "$G" && "$CXX" -O2 -w main.cpp FluidTracking.cpp GeomRead.cpp Intersect.cpp MeshGen.cpp \
    Vector2D.cpp Vector3D.cpp -o "$OUT/latticegen" -lm )
# reference serial colour-gradient CPU functions (Multiphase.cu), host-only
"$CXX" -x c++ -std=c++17 -O2 -fPIC -shared -w -D__global__= -D__device__= -D__host__= \
  -I"$S/include" -I"$CUDA_INC" "$S/Multiphase.cu" "$S/CellFunctions.cu" -x none "$HERE/ref_shim/ref_cpu_cg.cpp" \
  -o "$OUT/libref_multiphase.so" -lm 2>"$tmp/mp.log" \
  || echo "build_ref: Multiphase.cu host build failed (see $tmp/mp.log)" >&2
echo "build_ref: built $(ls "$OUT" | tr '\n' ' ')"
