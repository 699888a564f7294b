#!/usr/bin/env bash
# Compile the reference's own forward-solver (and octree regularisation) sources, unmodified and read in
# place from the reference tree, into a shared library that the tests use as
# a checker (oracle/_ref/libm3d_ref.so).  Three small shims stand in for what
# the reference tree lacks (p8est-backed OctreeMesh, the missing MT data
# header); they sit ahead of the reference include path.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
# Output goes to oracle/_ref/ only.  Skips silently when the tree is absent.
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/src/forward" ]; then
    echo "build_ref: reference tree not found at $REF; skipping" >&2
    exit 0
fi
mkdir -p "$OUT"
SRCS=(
  "$REF/src/octree/staggered_grid.cpp"
  "$REF/src/octree/operators.cpp"
  "$REF/src/forward/forward_solver_fv.cpp"
  "$REF/src/forward/bicgstab.cpp"
  "$REF/src/utils/logger.cpp"
  "$REF/src/model/conductivity_model.cpp"
  "$REF/src/inversion/regularization_octree.cpp"
  "$HERE/ref_driver.cpp"
)
CXXFLAGS=(-std=c++17 -O2 -fPIC -ffp-contract=off -DMAPLE3DMT_USE_OCTREE
          -I"$HERE/shim" -I"$HERE" -I"$REF/include" -w)
pids=()
objs=()
for s in "${SRCS[@]}"; do
    o="$OUT/$(basename "${s%.cpp}").o"
    objs+=("$o")
    g++ "${CXXFLAGS[@]}" -c "$s" -o "$o" &
    pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -o "$OUT/libm3d_ref.so" "${objs[@]}"
echo "build_ref: $OUT/libm3d_ref.so"
