#!/usr/bin/env bash
# Compile the reference library (FourierConvolutionCUDALib) from its own,
# unmodified sources into oracle/_ref/libfc_reference.so, for the parity tests
# and the timing of the reference's GPU build on the same GPU; and, into
# oracle/_ref/libfc_reference_sub.so, the host driver oracle/ref_subsampled.cu
# of the reference's subsampled-kernel product, compiled together with the
# reference's convolution3Dfft.cu.
#
# The reference's CMake cannot be used (it relies on the removed FindCUDA
# module and on pre-Turing architectures), so nvcc is called on its two .cu
# files directly.  cuFFT 12 removed three enum names that the reference's
# error-string helper (src/book.h:66,72,81) still uses; they are supplied with
# -D so that no source is edited.
#
# Where the reference tree is present ($REF/src), the five files the library
# is built from are staged unchanged into oracle/_ref/src (git-ignored, never
# committed) and compiled from there.  The staged directory travels with the
# working tree to machines that lack the reference tree (a GPU host of another
# architecture, where a library built here would not load), and the library is
# rebuilt there from it.  Without either, nothing is built and the script
# exits 0.
#
# The output has its own file name and soname, so that a process can load it
# beside this project's libFourierConvolutionCUDALib.so without one shadowing
# the other.
set -euo pipefail
REF=${REF:-/root/reference}
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
SRC="$OUT/src"
FILES=(convolution3Dfft.cu standardCUDAfunctions.cu convolution3Dfft.h book.h traits.hpp)
if [ -d "$REF/src" ]; then
  mkdir -p "$SRC"
  for f in "${FILES[@]}"; do cmp -s "$REF/src/$f" "$SRC/$f" || cp "$REF/src/$f" "$SRC/$f"; done
fi
for f in "${FILES[@]}"; do
  [ -f "$SRC/$f" ] || { echo "reference sources not present: skipped" >&2; exit 0; }
done
LIB="$OUT/libfc_reference.so"
ARCHTAG="$OUT/.built_for"
# rebuild when a source is newer, or when the library was built on another host architecture
SUBLIB="$OUT/libfc_reference_sub.so"
if [ -f "$LIB" ] && [ -f "$SUBLIB" ] && [ -f "$ARCHTAG" ] && [ "$(cat "$ARCHTAG")" = "$(uname -m)" ] && \
   [ -z "$(find "$SRC" "$HERE/ref_subsampled.cu" -newer "$SUBLIB" -type f)" ] && \
   [ -z "$(find "$SRC" -newer "$LIB" -type f)" ]; then
  echo "$LIB"
  exit 0
fi
NVCC=${NVCC:-nvcc}
command -v "$NVCC" >/dev/null 2>&1 || NVCC=/usr/local/cuda/bin/nvcc
FLAGS=(-std=c++17 -O2 --use_fast_math -Xcompiler -fPIC -gencode arch=compute_103a,code=sm_103a
       -DCUFFT_INCOMPLETE_PARAMETER_LIST=1001 -DCUFFT_PARSE_ERROR=1002 -DCUFFT_LICENSE_ERROR=1003 -I "$SRC")
"$NVCC" "${FLAGS[@]}" -c "$SRC/convolution3Dfft.cu" -o "$OUT/convolution3Dfft.o" &
p1=$!
"$NVCC" "${FLAGS[@]}" -c "$SRC/standardCUDAfunctions.cu" -o "$OUT/standardCUDAfunctions.o" &
p2=$!
# the host driver of the reference's subsampled-kernel product (oracle/ref_subsampled.cu), which
# includes the reference's convolution3Dfft.cu, as a library of its own
"$NVCC" "${FLAGS[@]}" -c "$HERE/ref_subsampled.cu" -o "$OUT/ref_subsampled.o" &
p3=$!
wait $p1
wait $p2
wait $p3
"$NVCC" -shared -gencode arch=compute_103a,code=sm_103a -Xlinker -soname=libfc_reference_sub.so \
  -Xlinker -rpath=/usr/local/cuda/lib64 -o "$SUBLIB.tmp" "$OUT/ref_subsampled.o" -lcufft -lcuda
mv "$SUBLIB.tmp" "$SUBLIB"
"$NVCC" -shared -gencode arch=compute_103a,code=sm_103a -Xlinker -soname=libfc_reference.so -Xlinker -rpath=/usr/local/cuda/lib64 -o "$LIB.tmp" \
  "$OUT/convolution3Dfft.o" "$OUT/standardCUDAfunctions.o" -lcufft -lcuda
mv "$LIB.tmp" "$LIB"
uname -m > "$ARCHTAG"
echo "$LIB"
