#!/bin/sh
# Build recipe for the oracle (test infrastructure only).
#   oracle/liborc.so    - the C restatement + Dot2 ground truth (any host).
#   oracle/_ref/*.so    - the reference library itself, compiled straight from its
#                         sources when they are present (x86-64 only: its kernels
#                         are x86-64 AVX2 assembly).  Output goes to oracle/_ref/ only.
#   oracle/_ref/libcplx.so - the reference's OpenBLAS-style complex and 3M kernels
#                         (four conjugation variants each) behind oracle/ref_cplx.c.
# Usage: oracle/build.sh [reference-source-dir]
#   (default: $GB300_REFERENCE_SOURCES, else /root/reference, the read-only
#   checkout of the reference in the build container; absent on GPU hosts)
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
cc=${CC:-gcc}
$cc -O3 -fopenmp -ffp-contract=off -fno-math-errno -fPIC -shared -fvisibility=hidden \
    -o "$HERE/liborc.so" "$HERE/oracle.c" -lm
REF=${1:-${GB300_REFERENCE_SOURCES:-/root/reference}}
if [ -n "$REF" ] && [ -f "$REF/src/gemm_driver.c" ] && [ "$(uname -m)" = "x86_64" ]; then
  mkdir -p "$HERE/_ref"
  # Same flags as the reference's own Makefile (Makefile:2,14-18), run on its
  # sources in place; nothing is copied.
  $cc -DDOUBLE -fopenmp --shared -fPIC -march=haswell -O2 \
      "$REF/src/kernel/gemm_kernel.S" "$REF/src/gemm_driver.c" -o "$HERE/_ref/DGEMM.so" 2>/dev/null
  $cc -fopenmp --shared -fPIC -march=haswell -O2 \
      "$REF/src/kernel/gemm_kernel.S" "$REF/src/gemm_driver.c" -o "$HERE/_ref/SGEMM.so" 2>/dev/null
fi
CK="$REF/OpenBLAS-like_implementation"
if [ -n "$REF" ] && [ -f "$CK/zgemm_kernel_4x2_haswell.c" ] && [ "$(uname -m)" = "x86_64" ]; then
  # The kernels include OpenBLAS's common.h for BLASLONG only; a two-line
  # stand-in under oracle/_ref/ provides it.  Variants by the kernels' own
  # macros (zgemm_kernel_4x2_haswell.c:6-21).
  mkdir -p "$HERE/_ref/include" "$HERE/_ref/obj"
  printf '#include <stdint.h>\ntypedef long BLASLONG;\n' > "$HERE/_ref/include/common.h"
  for v in NN RN NR RR; do
    lc=$(echo "$v" | tr 'A-Z' 'a-z')
    $cc -O2 -march=haswell -fPIC -c -D"$v" -DCNAME=ref_zgemm_kernel_"$lc" -I "$HERE/_ref/include" \
        "$CK/zgemm_kernel_4x2_haswell.c" -o "$HERE/_ref/obj/z_$lc.o"
    $cc -O2 -march=haswell -fPIC -c -D"$v" -DCNAME=ref_cgemm_kernel_"$lc" -I "$HERE/_ref/include" \
        "$CK/cgemm_kernel_8x2_haswell.c" -o "$HERE/_ref/obj/c_$lc.o"
  done
  $cc -O2 -march=haswell -fPIC -c -DCNAME=ref_zgemm3m_kernel -I "$HERE/_ref/include" \
      "$CK/zgemm3m_kernel_4x4_haswell.c" -o "$HERE/_ref/obj/z3m.o"
  $cc -O2 -march=haswell -fPIC -c -DCNAME=ref_cgemm3m_kernel -I "$HERE/_ref/include" \
      "$CK/cgemm3m_kernel_8x4_haswell.c" -o "$HERE/_ref/obj/c3m.o"
  $cc -O2 -fopenmp -fPIC -shared -fvisibility=hidden -o "$HERE/_ref/libcplx.so" "$HERE/ref_cplx.c" \
      "$HERE"/_ref/obj/z_*.o "$HERE"/_ref/obj/c_*.o "$HERE/_ref/obj/z3m.o" "$HERE/_ref/obj/c3m.o"
fi
if [ -n "$REF" ] && [ -f "$CK/TRSM_KERNEL_LN_simplified.c" ] && [ "$(uname -m)" = "x86_64" ]; then
  # The reference's TRSM and TRMM kernels behind oracle/ref_blas3.c.  The
  # stand-in common.h gives BLASLONG and, for the TRSM kernels, a prototype of
  # the GEMM kernel they call (GEMM_KERNEL_N, set per precision below).
  B3="$HERE/_ref/include3"
  mkdir -p "$B3" "$HERE/_ref/obj3"
  printf '%s\n' '#include <stdint.h>' 'typedef long BLASLONG;' \
      '#if defined(GEMM_KERNEL_N) && defined(FLOAT)' \
      'int GEMM_KERNEL_N(BLASLONG, BLASLONG, BLASLONG, FLOAT, FLOAT *, FLOAT *, FLOAT *, BLASLONG);' \
      '#endif' > "$B3/common.h"
  O3="$HERE/_ref/obj3"
  OPT="-O2 -march=haswell -fPIC -fvisibility=hidden -c -I $B3"
  # dgemm_kernel_4x4_haswell.c names its kernel KERNELFUNC (its own #define CNAME)
  $cc $OPT -DKERNELFUNC=ref_dgemm_kernel_4x4 "$CK/dgemm_kernel_4x4_haswell.c" -o "$O3/dgemm44.o"
  $cc $OPT -DCNAME=ref_sgemm_kernel_8x4 "$CK/sgemm_kernel_8x4_haswell.c" -o "$O3/sgemm84.o"
  for v in LN LT RN RT; do
    lc=$(echo "$v" | tr 'A-Z' 'a-z')
    $cc $OPT -DFLOAT=double -DGEMM_UNROLL_M=4 -DGEMM_UNROLL_N=4 \
        -DGEMM_KERNEL_N=ref_dgemm_kernel_long -DCNAME=ref_dtrsm_kernel_"$lc" \
        "$CK/TRSM_KERNEL_${v}_simplified.c" -o "$O3/dtrsm_$lc.o"
    $cc $OPT -DFLOAT=float -DGEMM_KERNEL_N=ref_sgemm_kernel_8x4 -DCNAME=ref_strsm_kernel_"$lc" \
        "$CK/strsm_kernel_8x4_haswell_$v.c" -o "$O3/strsm_$lc.o"
  done
  # TRMM variants by the kernel's LEFT / TRANSA macros (trmm_kernel_4x8_simplified.c:4-29)
  for v in ln:-DLEFT lt:-DLEFT:-DTRANSA rn: rt:-DTRANSA; do
    lc=${v%%:*}
    fl=$(echo "${v#*:}" | tr ':' ' ')
    for p in d:double s:float; do
      $cc $OPT -DFLOAT="${p#*:}" $fl -DCNAME=ref_"${p%%:*}"trmm_kernel_"$lc" \
          "$CK/trmm_kernel_4x8_simplified.c" -o "$O3/${p%%:*}trmm_$lc.o"
    done
  done
  $cc -O2 -fPIC -shared -fvisibility=hidden -o "$HERE/_ref/libblas3.so" "$HERE/ref_blas3.c" \
      "$O3"/*.o
fi
