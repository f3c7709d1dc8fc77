#!/bin/sh
# Builds oracle/_ref/ref_tables: the reference's own host-side B-spline table code
# (mesh/FunctionData.h, math/PPolynomial.h, math/Polynomial.h, mesh/BinaryNode.h,
# math/Factor.cpp) compiled in place from the reference tree, driven by
# oracle/ref_tables_main.cpp.  It is only used to pin the oracle's tables; nothing
# in the product links it.  Usage: sh oracle/build_ref.sh [reference_root]
set -e
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
CUDA_INC=${CUDA_HOME:-/usr/local/cuda}/include
mkdir -p "$HERE/_ref"
g++ -O1 -std=c++17 -w -include cfloat -include cstdio -I"$REF" -I"$CUDA_INC" \
    -o "$HERE/_ref/ref_tables" "$HERE/ref_tables_main.cpp" "$REF/math/Factor.cpp"
echo "built $HERE/_ref/ref_tables"
