#!/usr/bin/env bash
# Compiles the reference's own code, in place, into oracle/_ref/:
#   libeolc_ref.so     the four translation units that include nothing but
#                      <cmath>/<math.h> (element math and the ray test);
#   libeolc_ref_cd.so  src/boxTriCollision.cpp (collision detection, with the
#                      ray test of src/raytri.cpp) against the minimal Eigen
#                      shim in oracle/eigen_shim/, and the CD2 wrapper
#                      oracle/ref_cd.cpp.
# The rest of the reference needs Eigen 3.3.4 (sparse matrices, solvers),
# Windows include paths and Mosek/Gurobi and is not built.
#
#   REF_SRC defaults to /root/reference/src (read-only; nothing is copied).
#   Output goes only to oracle/_ref/ (git-ignored).
#
# -ffp-contract=off keeps the reference's arithmetic free of fused
# multiply-adds on every host (GCC contracts by default on aarch64).
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
REF_SRC="${REF_SRC:-/root/reference/src}"
out="$here/_ref"
if [ ! -f "$REF_SRC/ComputeMembrane.cpp" ]; then
  echo "build_ref: reference sources not found at $REF_SRC; skipping" >&2
  exit 0
fi
mkdir -p "$out"
CXX="${CXX:-g++}"
FLAGS="-O2 -fPIC -ffp-contract=off -fno-fast-math -w"
objs=()
for f in ComputeMembrane ComputeBending ComputeInertial raytri; do
  "$CXX" $FLAGS -c "$REF_SRC/$f.cpp" -o "$out/$f.o" &
  objs+=("$out/$f.o")
done
"$CXX" $FLAGS -c "$here/ref_shim.cpp" -o "$out/ref_shim.o" &
# The reference's collision detection (boxTriCollision.cpp, unmodified)
# against the minimal Eigen shim, plus the CD2 wrapper ref_cd.cpp.
CDFLAGS="$FLAGS -std=c++14 -I$here/eigen_shim -I$REF_SRC"
"$CXX" $CDFLAGS -c "$REF_SRC/boxTriCollision.cpp" -o "$out/boxTriCollision.o" &
"$CXX" $CDFLAGS -c "$here/ref_cd.cpp" -o "$out/ref_cd.o" &
wait
"$CXX" -shared -o "$out/libeolc_ref.so" "${objs[@]}" "$out/ref_shim.o"
"$CXX" -shared -o "$out/libeolc_ref_cd.so" "$out/boxTriCollision.o" "$out/raytri.o" \
  "$out/ref_cd.o"
echo "build_ref: wrote $out/libeolc_ref.so and $out/libeolc_ref_cd.so"
