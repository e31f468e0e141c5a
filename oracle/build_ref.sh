#!/usr/bin/env bash
# Recipe: compile the reference's own batched Kyber and NewHope device code for the host, via
# the CUDA shim in oracle/ref_shim, into oracle/_ref/*.so.  TEST INFRASTRUCTURE ONLY.
# NewHope is built for n = 1024 and n = 512 (NEWHOPE_N, NewHope_NIST_GPU/params.h:9-11); the
# n = 512 build adds oracle/ref_glue_newhope512.cpp for the one function the reference leaves
# undefined at that size.
#
# Reads the sources where they lie under the reference tree (default /root/reference, or $1).
# The only transformation is mechanical and lands in oracle/_ref/src (git-ignored): the kernel
# launches `K<<<g, b, ...>>>(args)` in the two orchestration files are rewritten into
# `host_launch(g, b, K, args)`.  Nothing from the reference is committed.
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/Kyber_GPU_Batched" ]; then
  echo "reference tree not found at $REF; skipping oracle/_ref" >&2
  exit 0
fi
CXX="${CXX:-g++}"
CXXFLAGS="-std=c++17 -O2 -fPIC -w -I$HERE/ref_shim"
LAUNCH_SED='s/([A-Za-z_0-9]+) *<< *<\s*([^,]+),\s*([^,>]+)[^>]*>> *>\s*\(/host_launch(\2, \3, \1, /'

build_one() {  # name srcdir "files" orchestration-file "driver files" kdefine
  local name="$1" srcdir="$2" files="$3" orch="$4" driver="$5" defs="$6"
  local w="$OUT/src/$name"
  rm -rf "$w"; mkdir -p "$w"
  cp "$REF/$srcdir"/*.h "$w/"
  for f in $files; do cp "$REF/$srcdir/$f" "$w/${f%.cu}.cpp"; done
  sed -E -i "$LAUNCH_SED" "$w/${orch%.cu}.cpp"
  local objs=()
  for f in $files; do
    "$CXX" $CXXFLAGS $defs -I"$w" -c "$w/${f%.cu}.cpp" -o "$w/${f%.cu}.o"
    objs+=("$w/${f%.cu}.o")
  done
  local drv=()
  for f in $driver; do drv+=("$HERE/$f"); done
  "$CXX" $CXXFLAGS $defs -I"$w" -shared -o "$OUT/lib$name.so" "${drv[@]}" "${objs[@]}"
}

mkdir -p "$OUT"
for K in 2 3 4; do
  build_one "refkyber$K" Kyber_GPU_Batched \
    "cbd.cu fips202.cu ntt.cu poly.cu polyvec.cu reduce.cu symmetric-fips202.cu indcpa.cu" \
    indcpa.cu ref_driver_kyber.cpp "-DKYBER_K=$K"
done
build_one refnewhope NewHope_NIST_GPU \
  "fips202.cu ntt.cu poly.cu precomp.cu reduce.cu cpapke.cu" \
  cpapke.cu ref_driver_newhope.cpp ""
build_one refnewhope512 NewHope_NIST_GPU \
  "fips202.cu ntt.cu poly.cu precomp.cu reduce.cu cpapke.cu" \
  cpapke.cu "ref_driver_newhope.cpp ref_glue_newhope512.cpp" "-DNEWHOPE_N=512"
echo "built: $(ls "$OUT"/*.so | xargs -n1 basename | tr '\n' ' ')"
