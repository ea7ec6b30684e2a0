#!/bin/sh
# Compiles the reference's own icbc.h (unmodified, read where it lies) in its
# scalar profile into oracle/_ref/libicbc_ref.so.  Test infrastructure only:
# the library pins the C restatement and generates tests/golden/.  Needs the
# reference checkout; exits 0 without building when it is absent.
set -e
REF=${ICBC_REFERENCE_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
if [ ! -f "$REF/icbc.h" ]; then
    echo "build_ref: no reference at $REF, skipping"
    exit 0
fi
mkdir -p "$HERE/_ref"
${CXX:-g++} -O2 -std=c++11 -DICBC_SIMD=0 -ffp-contract=off -fno-fast-math -fPIC -shared \
    -I"$REF" "$HERE/ref_shim.cpp" -o "$HERE/_ref/libicbc_ref.so"
echo "build_ref: built $HERE/_ref/libicbc_ref.so"
