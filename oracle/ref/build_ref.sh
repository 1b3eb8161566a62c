#!/usr/bin/env bash
# Builds the reference oracle (test infrastructure only) into oracle/_ref.
#
# The reference's density-based path is compiled from its own sources where
# they lie (MSTCFD_REF_SRC, required: the read-only reference checkout);
# nothing is copied.  Per variant, oracle/_ref/<variant>/src is a mirror of the
# reference tree made of symlinks, plus
#   * case-fixing symlinks for the includes the sources spell differently
#     from the file names (sparseSolverNUM.h, sparseSolver.h/.cpp, solverRoe.h),
#   * include/CONST.h = the reference CONST.h (linked as CONST_ref.h) followed
#     by the variant's overrides (RHO_P 0, ACCURACY, RHOSOLVER, threads),
#   * an empty pSolver/PSolver.h (the pressure solvers are not on this path and
#     need Eigen/Sparse plus a header the reference does not ship),
# and Eigen comes from the project's shim in oracle/ref/eigen_shim.
# -ffp-contract=off keeps gcc from fusing multiply-adds (aarch64 fuses by
# default), so the oracle rounds every operation like the parity kernels do.
set -euo pipefail
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=${MSTCFD_REF_OUT:-$HERE/../_ref}
REF=${MSTCFD_REF_SRC:?set MSTCFD_REF_SRC to the reference MST-CFD source directory}
THREADS=${MSTCFD_REF_THREADS:-$(nproc)}
CXX=${CXX:-g++}
CXXFLAGS="-std=c++20 -O2 -fopenmp -ffp-contract=off -w -I$HERE/eigen_shim"

if [ ! -f "$REF/rhoSolver/RhoSolver.cpp" ]; then
  echo "build_ref: reference sources not found at $REF" >&2
  exit 3
fi
mkdir -p "$OUT"
OUT=$(cd "$OUT" && pwd)

mirror() {  # variant-dir accuracy flux-class
  local V=$1 ACC=$2 FLUX=$3
  local S="$OUT/$V/src"
  rm -rf "$OUT/$V"
  mkdir -p "$S"
  for d in include mesh work data rhoSolver time lusolver pSolver; do
    mkdir -p "$S/$d"
  done
  for d in mesh work data rhoSolver time lusolver; do
    for f in "$REF/$d"/*; do ln -s "$f" "$S/$d/$(basename "$f")"; done
  done
  ln -s "$REF/lusolver/SparseSolverNUM.h" "$S/lusolver/sparseSolverNUM.h"
  ln -s "$REF/lusolver/SparseSolver.h" "$S/lusolver/sparseSolver.h"
  ln -s "$REF/lusolver/SparseSolver.cpp" "$S/lusolver/sparseSolver.cpp"
  ln -s "$REF/rhoSolver/SolverRoe.h" "$S/rhoSolver/solverRoe.h"
  ln -s "$REF/include/CONST.h" "$S/include/CONST_ref.h"
  printf '#pragma once\n' > "$S/pSolver/PSolver.h"
  cat > "$S/include/CONST.h" <<EOF
#pragma once
#include "CONST_ref.h"
#undef RHO_P
#define RHO_P 0
#undef ACCURACY
#define ACCURACY $ACC
#undef RHOSOLVER
#define RHOSOLVER $FLUX
#undef NUM_CPU_THREADS
#define NUM_CPU_THREADS $THREADS
EOF
}

SRCS="mesh/Cell.cpp mesh/Face.cpp mesh/Node.cpp mesh/FacesInf.cpp mesh/MshBlock.cpp
      work/FUNCTION.cpp data/AllData.cpp rhoSolver/RhoSolver.cpp
      rhoSolver/SolverRoe.cpp rhoSolver/SolverAusm.cpp time/Time.cpp"

build_variant() {  # variant-dir accuracy flux-class
  local V=$1
  mirror "$@"
  local S="$OUT/$V/src" O="$OUT/$V/obj"
  mkdir -p "$O"
  local objs=""
  for f in $SRCS; do
    local o="$O/$(echo "$f" | tr '/' '_').o"
    objs="$objs $o"
    $CXX $CXXFLAGS -I"$S" -c "$S/$f" -o "$o" &
  done
  $CXX $CXXFLAGS -I"$S" -c "$HERE/harness_rho.cpp" -o "$O/harness_rho.o" &
  wait
  $CXX $CXXFLAGS $objs "$O/harness_rho.o" -o "$OUT/ref_rho_$V"
}

build_variant ausm_o1 1 SolverAusm &
build_variant ausm_o2 2 SolverAusm &
build_variant roe_o1 1 solverRoe &
build_variant roe_o2 2 solverRoe &
wait

# lusolver: the scalar SparseSolverNUM and the block SparseSolver template.
S="$OUT/ausm_o1/src"
$CXX $CXXFLAGS -I"$S" "$S/lusolver/SparseSolverNUM.cpp" "$S/work/FUNCTION.cpp" \
  "$HERE/harness_lu.cpp" -o "$OUT/ref_lu"

# Result writer and checkpoint files: Work.cpp's own members
# (harness_io.cpp), linked with the first variant's objects.
O="$OUT/ausm_o1/obj"
$CXX $CXXFLAGS -I"$S" -c "$S/work/Work.cpp" -o "$O/work_Work.cpp.o"
$CXX $CXXFLAGS -I"$S" -c "$HERE/harness_io.cpp" -o "$O/harness_io.o"
objs=""
for f in $SRCS; do objs="$objs $O/$(echo "$f" | tr '/' '_').o"; done
$CXX $CXXFLAGS $objs "$O/work_Work.cpp.o" "$O/harness_io.o" -o "$OUT/ref_io"

# 3D reader: the mesh sources with DIM 3 (harness_mesh3d.cpp)
mirror mesh3d 1 SolverAusm
printf '#undef DIM\n#define DIM 3\n' >> "$OUT/mesh3d/src/include/CONST.h"
S3="$OUT/mesh3d/src"
O3="$OUT/mesh3d/obj"
mkdir -p "$O3"
objs3=""
for f in mesh/Cell.cpp mesh/Face.cpp mesh/Node.cpp mesh/FacesInf.cpp mesh/MshBlock.cpp work/FUNCTION.cpp; do
  o="$O3/$(echo "$f" | tr '/' '_').o"
  objs3="$objs3 $o"
  $CXX $CXXFLAGS -I"$S3" -c "$S3/$f" -o "$o" &
done
$CXX $CXXFLAGS -I"$S3" -c "$HERE/harness_mesh3d.cpp" -o "$O3/harness_mesh3d.o" &
wait
$CXX $CXXFLAGS $objs3 "$O3/harness_mesh3d.o" -o "$OUT/ref_mesh3d"

# Pressure-based SIMPLE path (harness_simple.cpp): the density-based sources
# plus pSolver/SolverSIMPLE.cpp, whose header only needs the (empty)
# PSolver.h overlay.  "simple" runs one thread: the reference's SIMPLE
# residual maximum is a data race across OpenMP threads
# (SolverSIMPLE.cpp:62-71); "simple_mt" uses every host thread and is the
# timed CPU baseline.
build_simple() {  # variant-dir threads
  local V=$1 T=$2
  mirror "$V" 1 SolverAusm
  local S="$OUT/$V/src" O="$OUT/$V/obj"
  printf '#undef NUM_CPU_THREADS\n#define NUM_CPU_THREADS %s\n' "$T" >> "$S/include/CONST.h"
  ln -s "$REF/pSolver/SolverSIMPLE.h" "$S/pSolver/SolverSIMPLE.h"
  ln -s "$REF/pSolver/SolverSIMPLE.cpp" "$S/pSolver/SolverSIMPLE.cpp"
  mkdir -p "$O"
  local objs=""
  for f in $SRCS lusolver/SparseSolverNUM.cpp pSolver/SolverSIMPLE.cpp; do
    local o="$O/$(echo "$f" | tr '/' '_').o"
    objs="$objs $o"
    $CXX $CXXFLAGS -I"$S" -c "$S/$f" -o "$o" &
  done
  $CXX $CXXFLAGS -I"$S" -c "$HERE/harness_simple.cpp" -o "$O/harness_simple.o" &
  wait
  $CXX $CXXFLAGS $objs "$O/harness_simple.o" -o "$OUT/ref_$V"
}
build_simple simple 1 &
build_simple simple_mt "$THREADS" &
wait

for v in ausm_o1 ausm_o2 roe_o1 roe_o2; do
  test -x "$OUT/ref_rho_$v"
done
test -x "$OUT/ref_simple"
test -x "$OUT/ref_simple_mt"
test -x "$OUT/ref_mesh3d"
test -x "$OUT/ref_lu"
test -x "$OUT/ref_io"
echo "build_ref: ok ($OUT)"
