#!/bin/sh
# Builds oracle/_ref/libreftile.so from the reference checkout's own
# src/tile_format.h (compiled where it lies) plus oracle/ref_shim.cpp, and
# oracle/_ref/ref_kernels.cubin from its kernel headers.
# TEST INFRASTRUCTURE: used only to pin the oracle and to write the golden
# fixtures under tests/golden/.  Skipped when the reference is absent.
# The checkout is the first argument, else $SPG_REFERENCE_DIR, else a
# "reference" directory beside this repository.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${SPG_REFERENCE_DIR:-$HERE/../../reference}}
if [ ! -f "$REF/src/tile_format.h" ]; then
  echo "reference not found at $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++17 -fPIC -shared -I "$REF/src" -o "$HERE/_ref/libreftile.so" "$HERE/ref_shim.cpp"
echo "$HERE/_ref/libreftile.so"
# the reference's own kernels as a cubin (no host code): driven on a GPU by
# tests/golden/make_cstruct_golden.py to record C-structure golden fixtures
if command -v nvcc >/dev/null 2>&1; then
  nvcc -cubin -gencode arch=compute_103a,code=sm_103a -std=c++17 -I "$REF/src" \
       -o "$HERE/_ref/ref_kernels.cubin" "$HERE/ref_kernels_shim.cu"
  echo "$HERE/_ref/ref_kernels.cubin"
fi
