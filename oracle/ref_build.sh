#!/bin/sh
# Builds oracle/_ref/libref_pin.so from the reference's own headers (read in
# place, never copied) plus oracle/ref_pin.cpp. Needs the reference checkout,
# named by NANOFILLER_REF;
# only the golden-vector script runs it.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${NANOFILLER_REF:?set NANOFILLER_REF to the reference checkout}
CUDA_INC=${CUDA_INC:-/usr/local/cuda/include}
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++17 -fPIC -shared -ffp-contract=off -fno-fast-math -w \
    -I"$REF/inc" -I"$CUDA_INC" -o "$HERE/_ref/libref_pin.so" "$HERE/ref_pin.cpp"
echo "$HERE/_ref/libref_pin.so"
