#!/bin/sh
# Builds the oracle (CPU restatement; test infrastructure only) into
# oracle/_build/libw3o.so. Portable flags only: the same source builds on
# x86_64 and aarch64 hosts. -ffp-contract=off keeps the arithmetic order
# of the restated Fortran (no fused multiply-add contraction).
set -e
here=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$here/_build"
${CXX:-g++} -O3 -fopenmp -ffp-contract=off -fPIC -shared -std=c++17 \
    -o "$here/_build/libw3o.so" "$here/w3o.cpp" "$here/w3o_mm10.cpp"
