#!/usr/bin/env bash
# Recipe: compile the reference's own batched Kyber and NewHope device code for the host, via
# the CUDA shim in oracle/ref_shim, into oracle/_ref/*.so.  TEST INFRASTRUCTURE ONLY.
# FrodoKEM-976: the reference's host KEM flow (FrodoKEM_GPU/kem.c) with its sampler, pack /
# unpack, SHAKE and matrix kernels, via oracle/ref_shim_sync (CTA barriers) and
# oracle/ref_glue_frodo.cpp, into oracle/_ref/librefrodo976.so.
# NewHope is built for n = 1024 and n = 512 (NEWHOPE_N, NewHope_NIST_GPU/params.h:9-11); the
# n = 512 build adds oracle/ref_glue_newhope512.cpp for the one function the reference leaves
# undefined at that size.
#
# Usage: build_ref.sh [REFERENCE_TREE]   (or REFERENCE_TREE in $PQC_REFERENCE_DIR)
# Step 1, only when a reference tree is given: stage the source files into oracle/_ref/src
# (git-ignored).  The only transformation is mechanical: the kernel launches
# `K<<<g, b, ...>>>(args)` in the orchestration files become `host_launch(g, b, K, args)`, and
# FrodoKEM-976's CDF table line (frodo976.cu:21) is copied into a header of its own.
# Step 2: compile the staged copy.  The staged copy travels with the working tree, so step 2 also
# runs on a machine that has no reference tree.  Nothing from the reference is committed.
set -euo pipefail
REF="${1:-${PQC_REFERENCE_DIR:-}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
CXX="${CXX:-g++}"
CXXFLAGS="-std=c++17 -O2 -fPIC -w -I$HERE/ref_shim"
LAUNCH_SED='s/([A-Za-z_0-9]+) *<< *<\s*(dim3\([^)]*\)|[^,]+),\s*(dim3\([^)]*\)|[^,>]+)[^>]*>> *>\s*\(/host_launch(\2, \3, \1, /'

stage_one() {  # name srcdir "files" orchestration-file
  local name="$1" srcdir="$2" files="$3" orch="$4"
  local w="$OUT/src/$name"
  rm -rf "$w"; mkdir -p "$w"
  cp "$REF/$srcdir"/*.h "$w/"
  for f in $files; do cp "$REF/$srcdir/$f" "$w/${f%.cu}.cpp"; done
  sed -E -i "$LAUNCH_SED" "$w/${orch%.cu}.cpp"
}

build_one() {  # name "files" "driver files" defines
  local name="$1" files="$2" driver="$3" defs="$4"
  local w="$OUT/src/$name"
  local objs=() pids=()
  for f in $files; do
    "$CXX" $CXXFLAGS $defs -I"$w" -c "$w/${f%.cu}.cpp" -o "$w/${f%.cu}.o" &
    pids+=($!)
    objs+=("$w/${f%.cu}.o")
  done
  for p in "${pids[@]}"; do wait "$p"; done
  local drv=()
  for f in $driver; do drv+=("$HERE/$f"); done
  "$CXX" $CXXFLAGS $defs -I"$w" -shared -o "$OUT/lib$name.so" "${drv[@]}" "${objs[@]}"
}

stage_frodo() {
  local w="$OUT/src/refrodo976" f="$REF/FrodoKEM_GPU"
  rm -rf "$w"; mkdir -p "$w"
  cp "$f"/*.h "$w/"
  cp "$f/util.cu" "$w/util.cpp"; cp "$f/fips202.cu" "$w/fips202.cpp"
  cp "$f/noise.c" "$w/noise.cpp"; cp "$f/kem.c" "$w/kem.cpp"
  cp "$f/frodo_macrify_reference.cu" "$w/frodo_macrify_reference.cpp"
  sed -E -i "$LAUNCH_SED" "$w/frodo_macrify_reference.cpp"
  local line len
  line="$(grep -E '^__constant__ uint16_t CDF_TABLE\[[0-9]+\]' "$f/frodo976.cu")"
  len="$(echo "$line" | sed -E 's/.*CDF_TABLE\[([0-9]+)\].*/\1/')"
  echo "$line" > "$w/ref_cdf_table.h"
  printf 'extern uint16_t CDF_TABLE[%s];\n#define CDF_TABLE_LEN %s\n' "$len" "$len" > "$w/ref_cdf_decl.h"
}

build_frodo() {
  local w="$OUT/src/refrodo976"
  local fl="-std=c++20 -O2 -fPIC -w -pthread -I$HERE/ref_shim_sync -I$w -include stdint.h -include stddef.h -include cuda_runtime.h"
  local pids=()
  "$CXX" $fl -c "$w/util.cpp" -o "$w/util.o" & pids+=($!)
  "$CXX" $fl -c "$w/fips202.cpp" -o "$w/fips202.o" & pids+=($!)
  "$CXX" $fl -include "$w/ref_cdf_decl.h" -c "$w/noise.cpp" -o "$w/noise.o" & pids+=($!)
  "$CXX" $fl -include "$HERE/ref_glue_frodo.h" -c "$w/kem.cpp" -o "$w/kem.o" & pids+=($!)
  "$CXX" $fl -c "$w/frodo_macrify_reference.cpp" -o "$w/frodo_macrify_reference.o" & pids+=($!)
  for p in "${pids[@]}"; do wait "$p"; done
  "$CXX" $fl -shared -o "$OUT/librefrodo976.so" "$HERE/ref_glue_frodo.cpp" "$w"/*.o
}

KYBER_FILES="cbd.cu fips202.cu ntt.cu poly.cu polyvec.cu reduce.cu symmetric-fips202.cu indcpa.cu"
NEWHOPE_FILES="fips202.cu ntt.cu poly.cu precomp.cu reduce.cu cpapke.cu"

if [ -n "$REF" ]; then
  if [ ! -d "$REF/Kyber_GPU_Batched" ]; then
    echo "no Kyber_GPU_Batched under $REF" >&2
    exit 1
  fi
  for K in 2 3 4; do stage_one "refkyber$K" Kyber_GPU_Batched "$KYBER_FILES" indcpa.cu; done
  stage_one refnewhope NewHope_NIST_GPU "$NEWHOPE_FILES" cpapke.cu
  stage_one refnewhope512 NewHope_NIST_GPU "$NEWHOPE_FILES" cpapke.cu
  stage_frodo
fi
if [ ! -f "$OUT/src/refkyber3/indcpa.cpp" ]; then
  echo "reference sources not staged (give the reference tree as \$1 or PQC_REFERENCE_DIR); skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$OUT"
jobs_=()
for K in 2 3 4; do
  build_one "refkyber$K" "$KYBER_FILES" ref_driver_kyber.cpp "-DKYBER_K=$K" &
  jobs_+=($!)
done
build_one refnewhope "$NEWHOPE_FILES" ref_driver_newhope.cpp "" &
jobs_+=($!)
build_one refnewhope512 "$NEWHOPE_FILES" "ref_driver_newhope.cpp ref_glue_newhope512.cpp" "-DNEWHOPE_N=512" &
jobs_+=($!)
if [ -f "$OUT/src/refrodo976/kem.cpp" ]; then
  build_frodo &
  jobs_+=($!)
fi
for p in "${jobs_[@]}"; do wait "$p"; done
echo "built: $(ls "$OUT"/*.so | xargs -n1 basename | tr '\n' ' ')"
