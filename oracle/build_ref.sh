#!/usr/bin/env bash
# Compile the reference's CPU core from its own sources (read in place, never
# copied) plus oracle/ref_driver.cpp into oracle/_ref/libkodama_ref.so.
#
# TEST INFRASTRUCTURE ONLY: the result pins the CPU restatement in
# oracle/kodama_oracle.cpp and generates tests/golden fixtures.  Needs the
# reference checkout (default /root/reference, override with KODAMA_REF_SRC);
# without it the script exits 0 and builds nothing.
set -euo pipefail
REF="${KODAMA_REF_SRC:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/inst/include/kodama/kodama.hpp" ]; then
  echo "reference sources not present at $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$OUT"
CXXFLAGS="-std=c++17 -O2 -fopenmp -fPIC -I$REF/inst/include -DKODAMA_DISABLE_NATIVE_PROGRESS"
UNITS="common core graph_cluster kodama_matrix knncv native_knn pca passing_message preprocessing plscv resident_ivf spatial_features visualization metal_backend_stub"
stamp="$OUT/.stamp"
need=0
[ -f "$OUT/libkodama_ref.so" ] || need=1
[ -f "$stamp" ] && [ "$HERE/ref_driver.cpp" -nt "$stamp" ] && need=1
if [ "$need" = 0 ]; then exit 0; fi
pids=()
for u in $UNITS; do
  g++ $CXXFLAGS -c "$REF/src/$u.cpp" -o "$OUT/$u.o" &
  pids+=($!)
done
g++ $CXXFLAGS -c "$HERE/ref_driver.cpp" -o "$OUT/ref_driver.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
objs=""
for u in $UNITS; do objs="$objs $OUT/$u.o"; done
g++ -shared -fopenmp -o "$OUT/libkodama_ref.so" $objs "$OUT/ref_driver.o"
touch "$stamp"
echo "built $OUT/libkodama_ref.so"
