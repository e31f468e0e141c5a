#!/usr/bin/env bash
# Recipe: the reference's own batched Kyber kernels (Kyber_GPU_Batched) compiled by nvcc for
# sm_103a, driven by baseline/ref_gpu_kyber.cu, into baseline/_ref/librefgpu_kyber{3,4}.so.
# A measurement baseline and GPU parity check only; libpqcgpu never links it.
#
# Usage: build_ref_gpu.sh [REFERENCE_TREE]   (or REFERENCE_TREE in $PQC_REFERENCE_DIR)
# Step 1 (only when a reference tree is given): stage the reference's files, unmodified, into
# baseline/_ref/src (git-ignored, shipped with the working tree so that step 2 can run on a
# machine without the reference).
# Step 2: compile with relocatable device code, as the reference's project does
# (Kyber_GPU_Batched/Kyber_GPU_Batched.vcxproj:89), once per KYBER_K.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
SRC="$OUT/src/Kyber_GPU_Batched"
REF="${1:-${PQC_REFERENCE_DIR:-}}"
FILES="cbd.cu fips202.cu ntt.cu poly.cu polyvec.cu reduce.cu symmetric-fips202.cu indcpa.cu"
if [ -n "$REF" ] && [ -d "$REF/Kyber_GPU_Batched" ]; then
  mkdir -p "$SRC"
  cp "$REF/Kyber_GPU_Batched"/*.h "$SRC/"
  for f in $FILES; do cp "$REF/Kyber_GPU_Batched/$f" "$SRC/$f"; done
fi
if [ ! -f "$SRC/indcpa.cu" ]; then
  echo "reference sources not staged; skipping baseline/_ref" >&2
  exit 0
fi
if ! command -v nvcc >/dev/null 2>&1; then
  echo "nvcc not found; skipping baseline/_ref" >&2
  exit 0
fi
srcs=()
for f in $FILES; do srcs+=("$SRC/$f"); done
pids=()
for K in 3 4; do
  nvcc -gencode arch=compute_103a,code=sm_103a -O3 -rdc=true -w -Xcompiler -fPIC -shared \
    -DKYBER_K=$K -I"$SRC" -o "$OUT/librefgpu_kyber$K.so" "$HERE/ref_gpu_kyber.cu" "${srcs[@]}" &
  pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
echo "built: $(cd "$OUT" && ls librefgpu_kyber*.so | tr '\n' ' ')"
