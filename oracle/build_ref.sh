#!/usr/bin/env bash
# Compiles the reference's own arithmetic cores, in place, into
# oracle/_ref/libeolc_ref.so.  Only the four translation units that include
# nothing but <cmath>/<math.h> are used; the rest of the reference needs
# Eigen 3.3.4, Windows include paths and Mosek/Gurobi and is not built.
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
wait
"$CXX" -shared -o "$out/libeolc_ref.so" "${objs[@]}" "$out/ref_shim.o"
echo "build_ref: wrote $out/libeolc_ref.so"
