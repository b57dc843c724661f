#!/bin/sh
# Builds libgwgb.so for sm_103a (the GB300 engine).  Translation units are
# compiled in parallel; the shared library links the CUDA runtime statically.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=${1:-$HERE/libgwgb.so}
BUILD=$HERE/_build
mkdir -p "$BUILD"
NVCC=${NVCC:-nvcc}
FLAGS="-gencode arch=compute_103a,code=sm_103a -O3 -lineinfo -std=c++17 -Xcompiler -fPIC -Xcompiler -Wall"
pids=""
for src in "$HERE"/*.cu; do
  obj="$BUILD/$(basename "$src" .cu).o"
  $NVCC $FLAGS -c "$src" -o "$obj" &
  pids="$pids $!"
done
for p in $pids; do wait $p; done
$NVCC -gencode arch=compute_103a,code=sm_103a -shared -o "$OUT" "$BUILD"/*.o -lcudart_static -lrt -lpthread -ldl
echo "built $OUT"
