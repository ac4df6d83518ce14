#!/usr/bin/env bash
# Compiles the reference's own CPU NTT (test/cpuNTT.cpp, test/cpuNTT_nega.cpp, src/Math.cu) from the sources
# where they lie, with the one-header shim in oracle/ref_shim standing in for the OpenFHE-dependent
# CKKS/Context.cuh.  Output: oracle/_ref/libref_cpuntt.so (git-ignored).  Test infrastructure only.
set -euo pipefail
REF=${FIDES_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
  echo "reference tree not found at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
NVCC=${NVCC:-nvcc}
FLAGS=(-std=c++20 -O2 -Xcompiler -fPIC -x cu -Wno-deprecated-gpu-targets -diag-suppress 20044
       -I "$HERE/ref_shim" -I "$REF/src" -I "$REF/test" -I "$REF/nvtx/c/include")
"$NVCC" "${FLAGS[@]}" -c "$REF/test/cpuNTT_nega.cpp" -o "$OUT/cpuNTT_nega.o"
"$NVCC" "${FLAGS[@]}" -c "$REF/test/cpuNTT.cpp" -o "$OUT/cpuNTT.o"
"$NVCC" "${FLAGS[@]}" -c "$REF/src/Math.cu" -o "$OUT/Math.o"
"$NVCC" "${FLAGS[@]}" -c "$HERE/ref_shim/ref_entry.cu" -o "$OUT/ref_entry.o"
"$NVCC" -shared -o "$OUT/libref_cpuntt.so" "$OUT/cpuNTT_nega.o" "$OUT/cpuNTT.o" "$OUT/Math.o" "$OUT/ref_entry.o"
rm -f "$OUT"/*.o
echo "$OUT/libref_cpuntt.so"
