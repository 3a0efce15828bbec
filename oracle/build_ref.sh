#!/usr/bin/env bash
# Compiles the reference's own colouring sources, where they lie, into
# oracle/_ref/ (git-ignored).  Only the host colouring functions of
# src_v2026_2_1/cudatest_coloring_gtx1060_optimized.cu (lines 50-106) are
# called from the result; they pin the product's colouring bit-exactly
# through tests/golden/make_golden.py.  Needs the reference tree, so it runs
# only where that tree is mounted; the fixtures it feeds are committed.
set -euo pipefail
REF=${VDR_REFERENCE_ROOT:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
SRC="$REF/src_v2026_2_1/cudatest_coloring_gtx1060_optimized.cu"
if [ ! -f "$SRC" ]; then
  echo "reference tree not found at $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$HERE/_ref"
nvcc -gencode arch=compute_103a,code=sm_103a -O2 -shared -Xcompiler -fPIC \
  -I"$REF/src_v2026_2_1" -o "$HERE/_ref/libref_coloring.so" "$SRC"
echo "built $HERE/_ref/libref_coloring.so"
