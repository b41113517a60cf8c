#!/usr/bin/env bash
# Build the compiled drop-in boundary check (TEST INFRASTRUCTURE ONLY):
# the reference's own CPU core (objects of oracle/build_ref.sh) with its
# *_CUDA stubs weakened, kodama_gb300/cxx/kodama_cuda_backend.cpp compiled
# against the reference's headers, tests/boundary/boundary_driver.cpp, and
# libkodama_gb300.so, linked into oracle/_ref/boundary/boundary_driver.
# Needs the reference checkout (KODAMA_REF_SRC, default /root/reference) and
# the two libraries already built; without them it exits 0 and builds nothing.
set -euo pipefail
REF="${KODAMA_REF_SRC:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
ROOT="$(cd "$HERE/.." && pwd)"
OBJ="$HERE/_ref"
OUT="$OBJ/boundary"
LIB="$ROOT/kodama_gb300/_lib"
if [ ! -f "$REF/inst/include/kodama/kodama.hpp" ] || [ ! -f "$OBJ/core.o" ] || [ ! -f "$LIB/libkodama_gb300.so" ]; then
  echo "reference sources, reference objects or libkodama_gb300.so missing; skipping the boundary build" >&2
  exit 0
fi
mkdir -p "$OUT"
UNITS="common core graph_cluster kodama_matrix knncv native_knn pca passing_message preprocessing plscv resident_ivf spatial_features visualization metal_backend_stub"
objs=()
for u in $UNITS; do
  cp "$OBJ/$u.o" "$OUT/$u.o"
  # every defined *_CUDA function of the reference becomes weak, so a strong
  # definition in kodama_cuda_backend.cpp takes its place at link time
  syms=$(nm --defined-only "$OUT/$u.o" | awk '$2 == "T" && $3 ~ /_CUDA/ {print $3}')
  args=()
  for s in $syms; do args+=("--weaken-symbol=$s"); done
  if [ ${#args[@]} -gt 0 ]; then objcopy "${args[@]}" "$OUT/$u.o"; fi
  objs+=("$OUT/$u.o")
done
CXX="g++ -std=c++17 -O2 -fPIC -fopenmp -I$REF/inst/include -I$REF/src -I$ROOT/include -DKODAMA_DISABLE_NATIVE_PROGRESS"
$CXX -c "$ROOT/kodama_gb300/cxx/kodama_cuda_backend.cpp" -o "$OUT/kodama_cuda_backend.o"
$CXX -c "$ROOT/tests/boundary/boundary_driver.cpp" -o "$OUT/boundary_driver.o"
g++ -fopenmp -o "$OUT/boundary_driver" "$OUT/boundary_driver.o" "$OUT/kodama_cuda_backend.o" "${objs[@]}" \
    -L"$LIB" -lkodama_gb300 -Wl,-rpath,"$LIB" -L/usr/local/cuda/lib64 -Wl,-rpath-link,/usr/local/cuda/lib64
echo "built $OUT/boundary_driver"
