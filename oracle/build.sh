#!/bin/sh
# Builds the oracle (CPU restatement; test infrastructure only).
#
#   oracle/_build/libw3o.so       parity checker: -ffp-contract=off keeps the
#                                 arithmetic order of the restated Fortran
#                                 (no fused multiply-add contraction)
#   oracle/_build/libw3o_fast.so  the timed CPU baseline: the same source
#                                 compiled the way WARP3D's own build treats
#                                 it (ifort -O3 -ip contracts multiply-adds
#                                 and inlines; src/Makefile.linux.inc), i.e.
#                                 with contraction, no errno from sqrt and
#                                 unrolling. Never used as a checker.
#
# Portable flags only: the same source builds on x86_64 and aarch64 hosts
# (no -march=native; on aarch64 the base ISA already has NEON and FMA).
set -e
here=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$here/_build"
${CXX:-g++} -O3 -fopenmp -ffp-contract=off -fPIC -shared -std=c++17 \
    -o "$here/_build/libw3o.so" "$here/w3o.cpp" "$here/w3o_mm10.cpp" "$here/w3o_umat.cpp" &
checker=$!
${CXX:-g++} -O3 -fopenmp -ffp-contract=fast -fno-math-errno -fno-trapping-math -funroll-loops -fPIC -shared \
    -std=c++17 -o "$here/_build/libw3o_fast.so" "$here/w3o.cpp" "$here/w3o_mm10.cpp" "$here/w3o_umat.cpp" &
timed=$!
wait $checker
wait $timed
