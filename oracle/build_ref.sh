#!/bin/sh
# Builds oracle/_ref/ref_harness from the reference sources in the
# directory FFCZ_REF names: HuffmanZSTDCoder.cuh with thrust on its CPP
# backend (host only, no GPU) and fileIO.cpp, against the system
# libzstd.so.1.  Test infrastructure; outputs go to oracle/_ref/ only.
set -e
if [ -z "$FFCZ_REF" ]; then
  echo "FFCZ_REF is not set: give the directory holding the reference sources" >&2
  exit 2
fi
HERE=$(cd "$(dirname "$0")" && pwd)
REF=$FFCZ_REF
NVCC=${NVCC:-/usr/local/cuda/bin/nvcc}
ZLIB=$(ls /usr/lib/*-linux-gnu/libzstd.so.1 2>/dev/null | head -1)
mkdir -p "$HERE/_ref"
"$NVCC" -std=c++17 -O2 -DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP \
  -I"$REF" -I"$HERE/ref_shim" "$HERE/ref_harness.cu" "$REF/fileIO.cpp" \
  -o "$HERE/_ref/ref_harness" -Xlinker "$ZLIB"
echo "$HERE/_ref/ref_harness"
