#!/bin/sh
# Compile the reference's own scene generator (Source/SceneManager.cpp) and
# frame loop (Source/Simulator.cpp), read in place from a read-only reference
# tree, with the shim headers in ref_shim/ into oracle/_ref/libref_scenes.so
# and oracle/_ref/libref_sim.so.  The solver itself (Banana SPHSolver) is not
# part of the reference tree and cannot be built.  Test infrastructure only.
# Usage: build_ref.sh <reference root>   (or SF_REFERENCE_ROOT in the environment)
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-$SF_REFERENCE_ROOT}"
[ -n "$REF" ] || { echo "usage: build_ref.sh <reference root> (or set SF_REFERENCE_ROOT)" >&2; exit 2; }
[ -f "$REF/Source/SceneManager.cpp" ] || { echo "reference tree not present: $REF" >&2; exit 1; }
mkdir -p "$HERE/_ref"
${CXX:-g++} -std=c++17 -O2 -fPIC -shared -ffp-contract=off -fno-fast-math \
    -I "$HERE/ref_shim" "$REF/Source/SceneManager.cpp" "$HERE/ref_scenes_wrap.cpp" \
    -o "$HERE/_ref/libref_scenes.so"
${CXX:-g++} -std=c++17 -O2 -fPIC -shared -ffp-contract=off -fno-fast-math -pthread \
    -I "$HERE/ref_shim" "$REF/Source/Simulator.cpp" "$REF/Source/SceneManager.cpp" "$HERE/ref_sim_wrap.cpp" \
    -o "$HERE/_ref/libref_sim.so"
