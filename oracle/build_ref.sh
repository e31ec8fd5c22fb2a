#!/bin/sh
# Builds oracle/_ref/libgarmref.so: the reference's unmodified Source/Core sources, compiled
# where they lie under the reference tree, against the project's Eigen/yaml-cpp subset shim
# (oracle/refshim) and the harness oracle/ref_harness.cpp.  TEST INFRASTRUCTURE ONLY.
#
#   oracle/build_ref.sh [REFERENCE_ROOT]      (default /root/reference)
#
# Configuration: the reference-map + gradient-augmentation path with WENO5 reinitialisation
# and the plain restart, i.e. none of _ENABLE_NEWTON_, _ENABLE_FMM_, _ENABLE_MC_,
# _ENABLE_CORR_, _ENABLE_PARTICLE_, _USE_LERP_, _USE_BFECC_, _DISABLE_RM_, _DISABLE_GA_
# (xmake.lua:25-80).  Flags as the reference's release build under g++ in ISO mode: -O3,
# OpenMP, no FMA contraction (g++'s default for -std=c++23).  Nothing is written outside
# oracle/_ref.
set -e
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -f "$REF/Source/Core/LevelSetLiquid.cpp" ] || { echo "reference sources not found under $REF" >&2; exit 1; }
mkdir -p "$OUT/obj"
CXX=${CXX:-g++}
FLAGS="-std=c++23 -O3 -fopenmp -ffp-contract=off -fPIC -w -I $HERE/refshim -I $HERE/../include -I $REF/Common/Util -I $REF/Source/Core -include $HERE/refshim/gcc_compat.h"
SRCS="LevelSetLiquid Boundary Projector Grid StaggeredGrid LagrangeIntrpl Contourer SurfaceMesh FastMarching FMMExtrapolator MeshToSdf HybridNewton"
pids=""
for s in $SRCS; do
	$CXX $FLAGS -c "$REF/Source/Core/$s.cpp" -o "$OUT/obj/$s.o" &
	pids="$pids $!"
done
$CXX $FLAGS -c "$HERE/ref_harness.cpp" -o "$OUT/obj/ref_harness.o" &
pids="$pids $!"
for p in $pids; do wait $p; done
objs=""
for s in $SRCS ref_harness; do objs="$objs $OUT/obj/$s.o"; done
$CXX -shared -fopenmp -o "$OUT/libgarmref.so" $objs
rm -f $objs
rmdir "$OUT/obj"
echo "built $OUT/libgarmref.so"
