#!/bin/sh
# Builds oracle/_ref/libref_pin.so from the reference's own headers (read in
# place, never copied) plus oracle/ref_pin.cpp, and oracle/_ref/libref_io.so
# from its own file writers (src/IO.cpp, src/stateSR.cpp, compiled in place)
# plus oracle/ref_io.cpp. Needs the reference checkout, named by
# NANOFILLER_REF; only the golden-vector scripts run them.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${NANOFILLER_REF:?set NANOFILLER_REF to the reference checkout}
CUDA_INC=${CUDA_INC:-/usr/local/cuda/include}
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++17 -fPIC -shared -ffp-contract=off -fno-fast-math -w \
    -I"$REF/inc" -I"$CUDA_INC" -o "$HERE/_ref/libref_pin.so" "$HERE/ref_pin.cpp"
g++ -O2 -std=c++17 -fPIC -shared -w -I"$REF/inc" -I"$REF/src" -I"$CUDA_INC" \
    -o "$HERE/_ref/libref_io.so" "$HERE/ref_io.cpp"
echo "$HERE/_ref/libref_pin.so $HERE/_ref/libref_io.so"
