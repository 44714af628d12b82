#!/usr/bin/env bash
# Compile the reference library from its own sources, where they lie, into
# oracle/_ref/.  Only runs where the reference tree is present; nothing is
# copied.  The reference's CMake cannot be used (it relies on the removed
# FindCUDA module and on pre-Turing architectures), so nvcc is called on its
# two .cu files directly.  cuFFT 12 removed three enum names that the
# reference's error-string helper (src/book.h:66,72,81) still uses; they are
# supplied with -D so that no source is edited.
set -euo pipefail
REF=${REF:-/root/reference}
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
# absent reference tree (a machine without the reference sources): nothing to build, not an error
[ -d "$REF/src" ] || { echo "reference sources not present: skipped" >&2; exit 0; }
mkdir -p "$OUT"
NVCC=${NVCC:-nvcc}
FLAGS=(-std=c++17 -O2 --use_fast_math -Xcompiler -fPIC -gencode arch=compute_103a,code=sm_103a
       -DCUFFT_INCOMPLETE_PARAMETER_LIST=1001 -DCUFFT_PARSE_ERROR=1002 -DCUFFT_LICENSE_ERROR=1003 -I "$REF/src")
"$NVCC" "${FLAGS[@]}" -c "$REF/src/convolution3Dfft.cu" -o "$OUT/convolution3Dfft.o" &
"$NVCC" "${FLAGS[@]}" -c "$REF/src/standardCUDAfunctions.cu" -o "$OUT/standardCUDAfunctions.o" &
wait
"$NVCC" -shared -gencode arch=compute_103a,code=sm_103a -o "$OUT/libFourierConvolutionCUDALib.so" \
  "$OUT/convolution3Dfft.o" "$OUT/standardCUDAfunctions.o" -lcufft -lcuda
echo "$OUT/libFourierConvolutionCUDALib.so"
