#!/bin/sh
# Builds libgwgb_peaks.so (the throughput probes bench.py reports as roofline
# denominators) for sm_103a.  Measurement code, built beside the engine.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
NVCC=${NVCC:-nvcc}
$NVCC -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo -std=c++17 -Xcompiler -fPIC -shared \
  -o "$HERE/libgwgb_peaks.so" "$HERE/peaks.cu" -lcudart_static -lrt -lpthread -ldl
echo "built $HERE/libgwgb_peaks.so"
