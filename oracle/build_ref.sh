#!/usr/bin/env bash
# Builds the reference's own code from the sources where they lie (test infrastructure only; nothing here is linked
# into the product), into oracle/_ref/ (git-ignored; it travels to the GPU host with the rest of the tree):
#   * libref_cpuntt.so: the reference's CPU NTT (test/cpuNTT.cpp, test/cpuNTT_nega.cpp, src/Math.cu) with the
#     one-header shim in oracle/ref_shim standing in for the OpenFHE-dependent CKKS/Context.cuh;
#   * ref_kernels.cubin: the reference's GPU kernels of src/CKKS/Conv.cu and src/NTT.cu in one sm_103a module
#     (oracle/ref_kernels/bundle.cu), with ref_kernels.json naming its entry points (from ptxas' report) and
#     ref_layout.json giving the byte layout of the constant blocks they read (oracle/ref_kernels/layout.cu).
# The reference tree is taken from $FIDES_REFERENCE (default: the checkout this recipe was written against); when
# it is absent the recipe does nothing.
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
INC=(-I "$HERE/ref_shim" -I "$REF/src" -I "$REF/test" -I "$REF/nvtx/c/include")
FLAGS=(-std=c++20 -O2 -Xcompiler -fPIC -x cu -Wno-deprecated-gpu-targets -diag-suppress 20044 "${INC[@]}")
"$NVCC" "${FLAGS[@]}" -c "$REF/test/cpuNTT_nega.cpp" -o "$OUT/cpuNTT_nega.o"
"$NVCC" "${FLAGS[@]}" -c "$REF/test/cpuNTT.cpp" -o "$OUT/cpuNTT.o"
"$NVCC" "${FLAGS[@]}" -c "$REF/src/Math.cu" -o "$OUT/Math.o"
"$NVCC" "${FLAGS[@]}" -c "$HERE/ref_shim/ref_entry.cu" -o "$OUT/ref_entry.o"
"$NVCC" -shared -o "$OUT/libref_cpuntt.so" "$OUT/cpuNTT_nega.o" "$OUT/cpuNTT.o" "$OUT/Math.o" "$OUT/ref_entry.o"
rm -f "$OUT"/*.o

# GPU kernels: asserts compiled out (-DNDEBUG), as in a release build of the reference.
if [ ! -f "$OUT/ref_kernels.cubin" ] || [ "$HERE/ref_kernels/bundle.cu" -nt "$OUT/ref_kernels.cubin" ]; then
  "$NVCC" -std=c++20 -O3 -DNDEBUG -cubin -gencode arch=compute_103a,code=sm_103a -Xptxas -v -Wno-deprecated-gpu-targets \
    -diag-suppress 20044 "${INC[@]}" "$HERE/ref_kernels/bundle.cu" -o "$OUT/ref_kernels.cubin" > "$OUT/ref_kernels.ptxas.txt" 2>&1
  python3 - "$OUT/ref_kernels.ptxas.txt" "$OUT/ref_kernels.json" <<'PY'
import json, re, subprocess, sys
names = re.findall(r"Compiling entry function '([^']+)'", open(sys.argv[1]).read())
dem = subprocess.run(["c++filt"], input="\n".join(names), capture_output=True, text=True).stdout.split("\n")
json.dump(dict(zip(dem, names)), open(sys.argv[2], "w"), indent=0)
PY
  rm -f "$OUT/ref_kernels.ptxas.txt"
fi
if [ ! -f "$OUT/ref_layout.json" ] || [ "$HERE/ref_kernels/layout.cu" -nt "$OUT/ref_layout.json" ]; then
  "$NVCC" -std=c++20 -Wno-deprecated-gpu-targets -diag-suppress 20044 "${INC[@]}" -x cu "$HERE/ref_kernels/layout.cu" \
    -o "$OUT/ref_layout"
  "$OUT/ref_layout" > "$OUT/ref_layout.json"
  rm -f "$OUT/ref_layout"
fi
echo "$OUT/libref_cpuntt.so"
