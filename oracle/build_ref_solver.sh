#!/bin/sh
# Builds oracle/_ref/ref_solver: the unmodified reference sources in the
# directory given by FFCZ_REF (projection_algorithm.cu, fileIO.cpp and the
# headers they include, with cuFFT, CUB, Thrust and the system libzstd.so.1)
# plus the harness oracle/ref_solver.cu, for sm_103a, with the reference's
# own flags (-O3, C++17, separable compilation); and
# oracle/_ref/legacy_kernels_ref, the driver tests/legacy_kernels_driver.cu
# built against the reference's header and kernels.  Test infrastructure;
# the outputs go to oracle/_ref/ only.  The translation units compile in
# parallel.
set -e
if [ -z "$FFCZ_REF" ]; then
  echo "FFCZ_REF is not set: give the directory holding the reference sources" >&2
  exit 2
fi
HERE=$(cd "$(dirname "$0")" && pwd)
REF=$(cd "$FFCZ_REF" && pwd)
NVCC=${NVCC:-/usr/local/cuda/bin/nvcc}
ZLIB=$(ls /usr/lib/*-linux-gnu/libzstd.so.1 2>/dev/null | head -1)
OUT="$HERE/_ref"
mkdir -p "$OUT"
ARCH="-gencode arch=compute_103a,code=sm_103a"
FLAGS="-std=c++17 -O3 $ARCH -rdc=true -I$REF -I$HERE/ref_shim"
"$NVCC" $FLAGS -c "$REF/projection_algorithm.cu" -o "$OUT/rs_projection_algorithm.o" &
P1=$!
"$NVCC" $FLAGS -c "$HERE/ref_solver.cu" -o "$OUT/rs_harness.o" &
P2=$!
"$NVCC" $FLAGS -c "$HERE/../tests/legacy_kernels_driver.cu" -o "$OUT/rs_legacy_driver.o" &
P3=$!
g++ -std=c++17 -O3 -I"$REF" -c "$REF/fileIO.cpp" -o "$OUT/rs_fileIO.o"
wait $P1
wait $P2
wait $P3
"$NVCC" $ARCH -rdc=true "$OUT/rs_projection_algorithm.o" "$OUT/rs_harness.o" "$OUT/rs_fileIO.o" \
  -o "$OUT/ref_solver" -lcufft -Xlinker "$ZLIB"
"$NVCC" $ARCH -rdc=true "$OUT/rs_projection_algorithm.o" "$OUT/rs_legacy_driver.o" \
  -o "$OUT/legacy_kernels_ref" -lcufft
echo "$OUT/ref_solver"
