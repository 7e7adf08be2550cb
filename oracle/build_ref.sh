#!/bin/sh
# Compile the reference's own scene generator (Source/SceneManager.cpp), frame
# loop (Source/Simulator.cpp) and particle shaders (Shaders/particle.vs.glsl,
# particle.fs.glsl), read in place from a read-only reference tree, with the
# shim headers in ref_shim/ into oracle/_ref/libref_scenes.so,
# oracle/_ref/libref_sim.so and oracle/_ref/libref_shader.so.  The shaders'
# text is compiled as C++: the awk below drops the #version line and the
# storage qualifiers, and turns each uniform block into plain declarations
# (an instance-named block into an unnamed struct of that name); ref_shim/glsl.h
# supplies the GLSL types and built-ins.  The solver itself (Banana SPHSolver)
# is not part of the reference tree and cannot be built.  Test infrastructure
# only.
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

glsl_to_cpp() {
    awk '
        /^#version/ { next }
        /^layout\(std140\) uniform/ { blk = 1; buf = ""; next }
        blk && /^[[:space:]]*\{/ { next }
        blk && /^[[:space:]]*\}/ {
            if ($0 ~ /^[[:space:]]*\};/) printf "%s", buf
            else printf "struct {\n%s%s\n", buf, $0
            blk = 0; next
        }
        blk { buf = buf $0 "\n"; next }
        { sub(/^(uniform|in|out)[[:space:]]+/, ""); print }
    ' "$1" > "$2"
}
glsl_to_cpp "$REF/Shaders/particle.vs.glsl" "$HERE/_ref/particle_vs.inc"
glsl_to_cpp "$REF/Shaders/particle.fs.glsl" "$HERE/_ref/particle_fs.inc"
${CXX:-g++} -std=c++17 -O2 -fPIC -shared -ffp-contract=off -fno-fast-math -fsingle-precision-constant \
    -I "$HERE/ref_shim" -I "$HERE/_ref" "$HERE/ref_shader_wrap.cpp" -o "$HERE/_ref/libref_shader.so"
