#!/bin/sh
# Build recipe for the oracle (test infrastructure only).
#   oracle/liborc.so    - the C restatement + Dot2 ground truth (any host).
#   oracle/_ref/*.so    - the reference library itself, compiled straight from its
#                         sources when they are present (x86-64 only: its kernels
#                         are x86-64 AVX2 assembly).  Output goes to oracle/_ref/ only.
# Usage: oracle/build.sh [reference-source-dir]
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
cc=${CC:-gcc}
$cc -O3 -fopenmp -ffp-contract=off -fno-math-errno -fPIC -shared -fvisibility=hidden \
    -o "$HERE/liborc.so" "$HERE/oracle.c" -lm
REF=${1:-}
if [ -n "$REF" ] && [ -f "$REF/src/gemm_driver.c" ] && [ "$(uname -m)" = "x86_64" ]; then
  mkdir -p "$HERE/_ref"
  # Same flags as the reference's own Makefile (Makefile:2,14-18), run on its
  # sources in place; nothing is copied.
  $cc -DDOUBLE -fopenmp --shared -fPIC -march=haswell -O2 \
      "$REF/src/kernel/gemm_kernel.S" "$REF/src/gemm_driver.c" -o "$HERE/_ref/DGEMM.so" 2>/dev/null
  $cc -fopenmp --shared -fPIC -march=haswell -O2 \
      "$REF/src/kernel/gemm_kernel.S" "$REF/src/gemm_driver.c" -o "$HERE/_ref/SGEMM.so" 2>/dev/null
fi
