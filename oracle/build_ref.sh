#!/bin/sh
# Builds oracle/_ref/libreftile.so from the reference checkout's own
# src/tile_format.h (compiled where it lies) plus oracle/ref_shim.cpp.
# TEST INFRASTRUCTURE: used only to pin the oracle and to write the golden
# fixtures under tests/golden/.  Skipped when the reference is absent.
set -e
REF=${SPG_REFERENCE_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
if [ ! -f "$REF/src/tile_format.h" ]; then
  echo "reference not found at $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++17 -fPIC -shared -I "$REF/src" -o "$HERE/_ref/libreftile.so" "$HERE/ref_shim.cpp"
echo "$HERE/_ref/libreftile.so"
