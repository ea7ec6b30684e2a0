#!/bin/sh
# Compiles the reference's own icbc.h (unmodified, read where it lies) in its
# scalar profile into oracle/_ref/libicbc_ref.so.  Test infrastructure only:
# the library pins the C restatement and generates tests/golden/.  Needs the
# reference checkout; exits 0 without building when it is absent.  This
# recipe is the one place that names the checkout's location;
# ICBC_REFERENCE_DIR overrides it, and `build_ref.sh --where` prints it.
set -e
REF=${ICBC_REFERENCE_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
if [ "$1" = "--where" ]; then
    echo "$REF"
    exit 0
fi
if [ ! -f "$REF/icbc.h" ]; then
    echo "build_ref: no reference at $REF, skipping"
    exit 0
fi
mkdir -p "$HERE/_ref"
${CXX:-g++} -O2 -std=c++11 -DICBC_SIMD=0 -ffp-contract=off -fno-fast-math -fPIC -shared \
    -I"$REF" "$HERE/ref_shim.cpp" -o "$HERE/_ref/libicbc_ref.so"
echo "build_ref: built $HERE/_ref/libicbc_ref.so"
# The x86 SIMD builds of the same header (ICBC_SSE2 .. ICBC_AVX512,
# icbc.h:59-64), also without FP contraction: they pin the oracle's SIMD
# profiles.  Only where the compiler targets x86-64.
case "$(${CXX:-g++} -dumpmachine)" in
x86_64*)
    for v in "1:" "2:-msse4.1" "3:-mavx" "4:-mavx2 -mfma -mbmi2" \
             "5:-mavx512f -mavx512vl -mavx512bw -mavx512dq -mfma -mbmi2"; do
        n=${v%%:*}
        f=${v#*:}
        ${CXX:-g++} -O2 -std=c++11 -DICBC_SIMD=$n $f -ffp-contract=off -fno-fast-math -fPIC -shared \
            -I"$REF" "$HERE/ref_shim.cpp" -o "$HERE/_ref/libicbc_ref_simd$n.so"
    done
    echo "build_ref: built the SIMD builds 1..5"
    ;;
esac
