#!/bin/sh
# Build the CPU oracle (test infrastructure) into oracle/_build/libsf_oracle.so.
# -ffp-contract=off: no implicit fused multiply-adds (the restatement writes its
# fma calls explicitly); no -march flags so x86-64 and aarch64 agree.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$HERE/_build"
${CXX:-g++} -std=c++17 -O3 -fPIC -shared -fopenmp -ffp-contract=off -fno-fast-math \
    "$HERE/sph_oracle.cpp" -o "$HERE/_build/libsf_oracle.so"
