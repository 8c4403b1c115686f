#!/usr/bin/env bash
# Builds the reference's own OpenMP counting binaries (G2Miner, vendored in
# X-GMiner under codes/GraphMiner) from their unmodified sources into oracle/_ref/.
# Test infrastructure only: the tests use these binaries to pin the C restatement in
# oracle/oracle.c.  Needs the reference tree; exits 0 without building when it is
# absent (the GPU host has no copy of it).
#
#   tc_omp_base     <- src/common/{graph,VertexSet}.cc src/triangle/{main,omp_base}.cc
#   clique_omp_base <- src/common/{graph,VertexSet}.cc src/clique/{main,omp_base}.cc
#   count_omp_base  <- + src/common/{pattern,intersect}.cc src/count/{main,omp_base}.cc
#   motif_omp_formula <- src/common/{graph,VertexSet}.cc src/motif/{main,omp_formula}.cc
#   glumin_pattern_cpu <- GLUMIN's codes/GLUMIN/src/common/{graph,VertexSet}.cc
#                         src/pattern/{main,cpu_serials}.cc (the 5-vertex CPU plans)
#
# count's intersect.cc uses x86 AVX2 intrinsics and rectangle.h misses <array>
# under gcc 13, hence -mavx2 and -include array for that binary only; on hosts
# without AVX2 it is skipped.
set -u
REF="${XGM_REFERENCE_ROOT:-/root/reference}"
GM="$REF/codes/GraphMiner"
OUT="$(cd "$(dirname "$0")" && pwd)/_ref"
if [ ! -d "$GM/src" ]; then
  echo "build_ref: reference tree not found at $REF; skipping"
  exit 0
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS="-O3 -fopenmp -std=c++17 -w -I$GM/include"
COMMON="$GM/src/common/graph.cc $GM/src/common/VertexSet.cc"
rc=0
build() {  # name, extra args...
  local name="$1"; shift
  if [ -x "$OUT/$name" ] && [ "$OUT/$name" -nt "$0" ]; then return 0; fi
  "$CXX" ${BFLAGS:-$FLAGS} "$@" -o "$OUT/$name" || { echo "build_ref: $name failed"; rc=1; }
}
build tc_omp_base $COMMON "$GM/src/triangle/main.cc" "$GM/src/triangle/omp_base.cc" &
build clique_omp_base -I"$GM/src/clique/cpu_kernels" $COMMON "$GM/src/clique/main.cc" \
  "$GM/src/clique/omp_base.cc" &
build motif_omp_formula -I"$GM/src/motif/cpu_kernels" $COMMON "$GM/src/motif/main.cc" \
  "$GM/src/motif/omp_formula.cc" &
GL="$REF/codes/GLUMIN"
if [ -d "$GL/src/pattern" ]; then
  BFLAGS="-O3 -fopenmp -std=c++17 -w" build glumin_pattern_cpu -I"$GL/include" \
    -I"$GL/src/pattern/cpu_kernels" \
    "$GL/src/common/graph.cc" "$GL/src/common/VertexSet.cc" "$GL/src/pattern/cpu_serials.cc" \
    "$GL/src/pattern/main.cc" &
fi
if [ "$(uname -m)" = "x86_64" ]; then
  build count_omp_base -mavx2 -include array -I"$GM/src/count/cpu_kernels" $COMMON \
    "$GM/src/common/pattern.cc" "$GM/src/common/intersect.cc" "$GM/src/count/main.cc" \
    "$GM/src/count/omp_base.cc" &
fi
wait
exit $rc
