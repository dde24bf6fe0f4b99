#!/usr/bin/env bash
# Test infrastructure: compiles the reference's own EFIE/CFIE/MLFMA sources
# (xiangwei0909/EMFA) into oracle/_ref/emfa_ref_f32 and oracle/_ref/emfa_ref_f64,
# each linked with oracle/ref_harness.cpp, which drives the reference classes
# and dumps their matrices/vectors in binary.  Only tests, the golden-vector
# script and the CPU baseline run these binaries; the product never does.
#
# The reference is MSVC code; four mechanical patches make it build with g++
# on a scratch copy under oracle/_ref/src_<variant>/ (never committed):
#   P1 Result.h: include Mathdef.h (MSVC found it by accident)
#   P2 tools.cpp: <filesystem> -> <experimental/filesystem>
#   P3 Custom.h: Qumat = arma::umat (size_t != arma::uword on LP64 Linux)
#   P4 Custom.h: no ARMA_USE_LAPACK/BLAS (those libraries are not shipped)
# The f64 variant additionally sets value_t = double and strips the 'f'
# suffix of float literals, giving the FP64-promoted reference.
#
# The patched sources and the header libraries they include (Armadillo, Eigen,
# vendored by the reference) are staged under oracle/_ref/ (git-ignored), so
# `oracle/build_ref.sh --staged` rebuilds the binaries on a machine without the
# reference tree (the GPU host is another architecture).
#
# Usage: oracle/build_ref.sh [reference_root]   (default /root/reference)
#        oracle/build_ref.sh --staged
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
STAGED=0
if [ "${1:-}" = "--staged" ]; then
  STAGED=1
  if [ ! -d "$OUT/src_f32" ] || [ ! -d "$OUT/include" ]; then
    echo "build_ref: no staged reference under $OUT; skipping" >&2
    exit 0
  fi
  INC="$OUT/include"
else
  REF="${1:-${EMFA_REFERENCE:-/root/reference}}"
  if [ ! -d "$REF/EMSolver" ]; then
    echo "build_ref: reference sources not found at $REF; skipping" >&2
    exit 0
  fi
  mkdir -p "$OUT/include/Eigen"
  cp -r "$REF/include/armadillo" "$REF/include/armadillo_bits" "$OUT/include/"
  cp -r "$REF/include/Eigen/Eigen" "$REF/include/Eigen/unsupported" "$OUT/include/Eigen/"
  INC="$OUT/include"
fi

COMP_SRC="Mesh Triangle Tetrahedron CommonEdge ConfigLoader Quadrature Result ThreadPool tools MLFMA_Boundary"
SOLV_SRC="EM EFIE CFIE MLFMA Miscellaneous"

build_variant() {
  local v="$1"
  local S="$OUT/src_$v"
  if [ "$STAGED" = "0" ]; then
  rm -rf "$S"
  mkdir -p "$S"
  cp "$REF"/EMComponent/*.h "$S/"
  for f in $COMP_SRC; do cp "$REF/EMComponent/$f.cpp" "$S/"; done
  for f in $SOLV_SRC; do cp "$REF/EMSolver/$f.cpp" "$REF/EMSolver/$f.h" "$S/"; done
  cp "$REF/EMSolver/EMBase.h" "$S/"
  cp "$REF/EMIterative/iml.h" "$REF/EMIterative/iml.cpp" "$S/"
  # P1
  sed -i 's|#include "MyFWD.h"|#include "MyFWD.h"\n#include "Mathdef.h"|' "$S/Result.h"
  # P2
  sed -i 's|#include <filesystem>|#include <experimental/filesystem>|' "$S/tools.cpp"
  # P3
  sed -i 's|typedef arma::Mat<size_t>       Qumat;|typedef arma::umat Qumat;|' "$S/Custom.h"
  # P4
  sed -i -e 's|^#define ARMA_USE_LAPACK|// P4 removed ARMA_USE_LAPACK|' \
         -e 's|^#define ARMA_USE_BLAS|// P4 removed ARMA_USE_BLAS|' "$S/Custom.h"
  if [ "$v" = "f64" ]; then
    sed -i 's|typedef float                   value_t;|typedef double                  value_t;|' "$S/Custom.h"
    # strip the f suffix of float literals: 1.0f, .5f, 2e-7f, 1.f
    sed -i -E 's/([0-9]\.[0-9]*([eE][-+]?[0-9]+)?|\.[0-9]+([eE][-+]?[0-9]+)?|[0-9][eE][-+]?[0-9]+)[fF]\b/\1/g' \
        "$S"/*.cpp "$S"/*.h
  fi
  fi
  grep -q "typedef arma::umat Qumat" "$S/Custom.h" || { echo "P3 failed" >&2; exit 1; }
  local objs=()
  for f in "$S"/*.cpp "$HERE/ref_harness.cpp"; do
    local o="$S/$(basename "${f%.cpp}").o"
    objs+=("$o")
    g++ -std=c++14 -O2 -w -fpermissive -DARMA_DONT_USE_LAPACK -DARMA_DONT_USE_BLAS \
        -DARMA_DONT_USE_WRAPPER -I"$S" -I"$INC" -I"$INC/Eigen" \
        -c "$f" -o "$o" &
  done
  wait
  g++ -o "$OUT/emfa_ref_$v.tmp" "${objs[@]}" -lstdc++fs -lpthread
  mv -f "$OUT/emfa_ref_$v.tmp" "$OUT/emfa_ref_$v"
  rm -f "${objs[@]}"
  echo "build_ref: built $OUT/emfa_ref_$v"
}

build_variant f32 &
build_variant f64 &
wait
