#!/bin/sh
# Builds oracle/_ref/ref_tables: the reference's own host-side B-spline table code
# (mesh/FunctionData.h, math/PPolynomial.h, math/Polynomial.h, mesh/BinaryNode.h,
# math/Factor.cpp) compiled in place from the reference tree, driven by
# oracle/ref_tables_main.cpp.  It is only used to pin the oracle's tables; nothing
# in the product links it.  Usage: sh oracle/build_ref.sh REFERENCE_ROOT
# (or with PSR_REFERENCE_ROOT set)
set -e
REF=${1:-$PSR_REFERENCE_ROOT}
if [ -z "$REF" ]; then echo "usage: build_ref.sh REFERENCE_ROOT" >&2; exit 2; fi
HERE=$(cd "$(dirname "$0")" && pwd)
CUDA_INC=${CUDA_HOME:-/usr/local/cuda}/include
mkdir -p "$HERE/_ref"
g++ -O1 -std=c++17 -w -include cfloat -include cstdio -I"$REF" -I"$CUDA_INC" \
    -o "$HERE/_ref/ref_tables" "$HERE/ref_tables_main.cpp" "$REF/math/Factor.cpp"
echo "built $HERE/_ref/ref_tables"
