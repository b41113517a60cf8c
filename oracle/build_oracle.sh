#!/usr/bin/env bash
# Build the CPU restatement (test infrastructure) into oracle/_build/liboracle.so.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
out="$HERE/_build/liboracle.so"
srcs=("$HERE/kodama_oracle.cpp" "$HERE/pls_oracle.cpp")
deps=("${srcs[@]}" "$HERE/pls_oracle.h" "$HERE/../kodama_gb300/csrc/ext80.h")
if [ -f "$out" ]; then
  fresh=1
  for f in "${deps[@]}"; do [ "$out" -nt "$f" ] || fresh=0; done
  if [ "$fresh" = 1 ]; then exit 0; fi
fi
g++ -std=c++17 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -pthread \
    -o "$out.tmp" "${srcs[@]}"
mv "$out.tmp" "$out"
