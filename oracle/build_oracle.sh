#!/usr/bin/env bash
# Build the CPU restatement (test infrastructure) into oracle/_build/liboracle.so.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
out="$HERE/_build/liboracle.so"
if [ -f "$out" ] && [ "$out" -nt "$HERE/kodama_oracle.cpp" ] && [ "$out" -nt "$HERE/../kodama_gb300/csrc/ext80.h" ]; then exit 0; fi
g++ -std=c++17 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -pthread \
    -o "$out.tmp" "$HERE/kodama_oracle.cpp"
mv "$out.tmp" "$out"
