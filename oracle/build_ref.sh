#!/bin/sh
# Compile the reference's own scene generator (Source/SceneManager.cpp, read in
# place from the read-only reference tree) with the shim headers in ref_shim/
# into oracle/_ref/libref_scenes.so.  The solver itself (Banana SPHSolver) is
# not part of the reference tree and cannot be built.  Test infrastructure only.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${SF_REFERENCE_ROOT:-/root/reference}"
[ -f "$REF/Source/SceneManager.cpp" ] || { echo "reference tree not present: $REF" >&2; exit 1; }
mkdir -p "$HERE/_ref"
${CXX:-g++} -std=c++17 -O2 -fPIC -shared -ffp-contract=off -fno-fast-math \
    -I "$HERE/ref_shim" "$REF/Source/SceneManager.cpp" "$HERE/ref_scenes_wrap.cpp" \
    -o "$HERE/_ref/libref_scenes.so"
