/*
 * ref_blas3.c -- harness around the reference's OpenBLAS-style TRSM and TRMM
 * kernels, compiled from their sources by oracle/build.sh into
 * oracle/_ref/libblas3.so (x86-64 only: the GEMM kernels the TRSM kernels call
 * are AVX2 assembly).
 *
 * TEST INFRASTRUCTURE ONLY: the tests use it to pin oracle/blas3.py (which
 * triangle each side/uplo/trans/diag variant references, where alpha applies)
 * to the reference's own kernels, and tests/golden/make_golden_blas3.py uses
 * it to write the fixtures the GPU tests compare against.
 *
 * Kernels (OpenBLAS-like_implementation/ in the reference):
 *   - DTRSM: TRSM_KERNEL_{LN,LT,RN,RT}_simplified.c with FLOAT = double,
 *     GEMM_UNROLL_M = GEMM_UNROLL_N = 4 and GEMM_KERNEL_N = the reference's
 *     dgemm_kernel_4x4_haswell.c (B in 4-column panels, r12 = k << 5 bytes);
 *   - STRSM: strsm_kernel_8x4_haswell_{LN,LT,RN,RT}.c (8 x 4 register tiles)
 *     with GEMM_KERNEL_N = sgemm_kernel_8x4_haswell.c;
 *   - D/STRMM: trmm_kernel_4x8_simplified.c, four variants by its LEFT and
 *     TRANSA macros (trmm_kernel_4x8_simplified.c:4-29).
 *
 * What each kernel variant solves / multiplies by (read from their loops):
 *   TRSM LN: backward substitution, op(A) upper (TRSM_KERNEL_LN_simplified.c:15-27)
 *   TRSM LT: forward substitution, op(A) lower (TRSM_KERNEL_LT_simplified.c:6-18)
 *   TRSM RN: X op(A) = B, op(A) upper, columns left to right
 *   TRSM RT: X op(A) = B, op(A) lower, columns right to left
 *   TRMM LN / RN (TRANSA unset): op(A) upper; LT / RT: op(A) lower.
 * The triangular operand is packed as OpenBLAS's trsm/trmm copy routines do:
 * the effective triangle of op(A) with the other triangle zero, the diagonal
 * as 1 / a_ii for TRSM (1 for a unit diagonal), in row panels (left side:
 * UNROLL_M rows, then the remainder in descending powers of two; for each k
 * the panel's rows) or column panels (right side: for each k the panel's
 * columns).  The other operand is packed in the complementary layout.  Each
 * call is one block covering the whole problem (offset 0), after the
 * driver-level scaling of B by alpha (TRSM; TRMM applies alpha in the kernel).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef long BLASLONG;

#define TRSM_KDECL(name, T) \
  int name(BLASLONG m, BLASLONG n, BLASLONG k, T d, T *a, T *b, T *c, BLASLONG ldc, BLASLONG off);
TRSM_KDECL(ref_dtrsm_kernel_ln, double)
TRSM_KDECL(ref_dtrsm_kernel_lt, double)
TRSM_KDECL(ref_dtrsm_kernel_rn, double)
TRSM_KDECL(ref_dtrsm_kernel_rt, double)
TRSM_KDECL(ref_strsm_kernel_ln, float)
TRSM_KDECL(ref_strsm_kernel_lt, float)
TRSM_KDECL(ref_strsm_kernel_rn, float)
TRSM_KDECL(ref_strsm_kernel_rt, float)
TRSM_KDECL(ref_dtrmm_kernel_ln, double)
TRSM_KDECL(ref_dtrmm_kernel_lt, double)
TRSM_KDECL(ref_dtrmm_kernel_rn, double)
TRSM_KDECL(ref_dtrmm_kernel_rt, double)
TRSM_KDECL(ref_strmm_kernel_ln, float)
TRSM_KDECL(ref_strmm_kernel_lt, float)
TRSM_KDECL(ref_strmm_kernel_rn, float)
TRSM_KDECL(ref_strmm_kernel_rt, float)

/* dgemm_kernel_4x4_haswell.c declares its kernel with int sizes
 * (`#define BLASLONG int` in that file); the TRSM kernels call GEMM_KERNEL_N
 * with BLASLONG, so they go through this adapter. */
int ref_dgemm_kernel_4x4(int m, int n, int k, double alpha, double *A, double *B, double *C,
                         int ldc);
int ref_dgemm_kernel_long(BLASLONG m, BLASLONG n, BLASLONG k, double alpha, double *A, double *B,
                          double *C, BLASLONG ldc) {
  return ref_dgemm_kernel_4x4((int)m, (int)n, (int)k, alpha, A, B, C, (int)ldc);
}

#define EXPORT __attribute__((visibility("default")))

static int upper_of(char uplo, char transa) {
  const int up = (uplo == 'U' || uplo == 'u');
  const int tr = !(transa == 'N' || transa == 'n');
  return up != tr;
}

#define HARNESS(T, P)                                                                          \
  /* effective triangle of op(A) (na x na, column-major, ld na) */                           \
  static T *tri_##P(const T *A, long lda, long na, char uplo, char transa, char diag,        \
                    int upper, int invert) {                                                 \
    T *t = (T *)calloc((size_t)(na * na > 0 ? na * na : 1), sizeof(T));                      \
    const int tr = !(transa == 'N' || transa == 'n');                                        \
    const int unit = (diag == 'U' || diag == 'u');                                           \
    for (long j = 0; j < na; j++)                                                            \
      for (long i = 0; i < na; i++) {                                                        \
        if (upper ? i > j : i < j) continue;                                                 \
        T v = tr ? A[j + i * lda] : A[i + j * lda];                                          \
        if (i == j) v = unit ? (T)1 : (invert ? (T)1 / v : v);                               \
        t[i + j * na] = v;                                                                   \
      }                                                                                      \
    (void)uplo;                                                                              \
    return t;                                                                                \
  }                                                                                          \
  /* row panels of X (R x K, ld): unroll rows, then descending powers of two */              \
  static T *pack_rows_##P(const T *X, long ld, long R, long K, int unroll) {                 \
    T *o = (T *)malloc((size_t)(R * K > 0 ? R * K : 1) * sizeof(T));                         \
    long r0 = 0, pos = 0;                                                                    \
    int w = unroll;                                                                          \
    while (r0 < R) {                                                                         \
      while (w > R - r0) w >>= 1;                                                            \
      for (long kk = 0; kk < K; kk++)                                                        \
        for (int r = 0; r < w; r++) o[pos++] = X[(r0 + r) + kk * ld];                        \
      r0 += w;                                                                               \
    }                                                                                        \
    return o;                                                                                \
  }                                                                                          \
  /* column panels of X (K x N, ld): unroll columns, then descending powers of two */       \
  static T *pack_cols_##P(const T *X, long ld, long K, long N, int unroll) {                 \
    T *o = (T *)malloc((size_t)(K * N > 0 ? K * N : 1) * sizeof(T));                         \
    long c0 = 0, pos = 0;                                                                    \
    int w = unroll;                                                                          \
    while (c0 < N) {                                                                         \
      while (w > N - c0) w >>= 1;                                                            \
      for (long kk = 0; kk < K; kk++)                                                        \
        for (int c = 0; c < w; c++) o[pos++] = X[kk + (c0 + c) * ld];                        \
      c0 += w;                                                                               \
    }                                                                                        \
    return o;                                                                                \
  }

HARNESS(double, d)
HARNESS(float, s)

/* B := alpha * inv(op(A)) * B (side 'L') or alpha * B * inv(op(A)) (side 'R'). */
#define TRSM_DRIVER(T, P, UM, UN)                                                              \
  EXPORT int ref_trsm_##P(char side, char uplo, char transa, char diag, long m, long n,        \
                          T alpha, const T *A, long lda, T *B, long ldb) {                     \
    if (m <= 0 || n <= 0) return 0;                                                            \
    for (long j = 0; j < n; j++)                                                               \
      for (long i = 0; i < m; i++) B[i + j * ldb] = alpha == (T)0 ? (T)0 : B[i + j * ldb] * alpha; \
    if (alpha == (T)0) return 0;                                                               \
    const int left = (side == 'L' || side == 'l');                                             \
    const int up = upper_of(uplo, transa);                                                     \
    const long na = left ? m : n;                                                              \
    T *t = tri_##P(A, lda, na, uplo, transa, diag, up, 1);                                     \
    T *scratch = (T *)calloc((size_t)(m * n), sizeof(T));                                      \
    T *pk;                                                                                     \
    int rc;                                                                                    \
    if (left) {                                                                                \
      pk = pack_rows_##P(t, na, m, m, UM);                                                     \
      rc = (up ? ref_##P##trsm_kernel_ln : ref_##P##trsm_kernel_lt)(m, n, m, (T)0, pk, scratch, \
                                                                    B, ldb, 0);                \
    } else {                                                                                   \
      pk = pack_cols_##P(t, na, n, n, UN);                                                     \
      rc = (up ? ref_##P##trsm_kernel_rn : ref_##P##trsm_kernel_rt)(m, n, n, (T)0, scratch, pk, \
                                                                    B, ldb, 0);                \
    }                                                                                          \
    free(pk);                                                                                  \
    free(scratch);                                                                             \
    free(t);                                                                                   \
    return rc;                                                                                 \
  }

TRSM_DRIVER(double, d, 4, 4)
TRSM_DRIVER(float, s, 8, 4)

/* B := alpha * op(A) * B (side 'L') or alpha * B * op(A) (side 'R'); the TRMM
 * kernel works on 4-row and 8-column panels (trmm_kernel_4x8_simplified.c). */
#define TRMM_DRIVER(T, P)                                                                      \
  EXPORT int ref_trmm_##P(char side, char uplo, char transa, char diag, long m, long n,        \
                          T alpha, const T *A, long lda, T *B, long ldb) {                     \
    if (m <= 0 || n <= 0) return 0;                                                            \
    const int left = (side == 'L' || side == 'l');                                             \
    const int up = upper_of(uplo, transa);                                                     \
    const long na = left ? m : n;                                                              \
    T *t = tri_##P(A, lda, na, uplo, transa, diag, up, 0);                                     \
    T *pa, *pb;                                                                                \
    int rc;                                                                                    \
    if (left) {                                                                                \
      pa = pack_rows_##P(t, na, m, m, 4);                                                      \
      pb = pack_cols_##P(B, ldb, m, n, 8);                                                     \
      rc = (up ? ref_##P##trmm_kernel_ln : ref_##P##trmm_kernel_lt)(m, n, m, alpha, pa, pb, B,  \
                                                                    ldb, 0);                   \
    } else {                                                                                   \
      pa = pack_rows_##P(B, ldb, m, n, 4);                                                     \
      pb = pack_cols_##P(t, na, n, n, 8);                                                      \
      rc = (up ? ref_##P##trmm_kernel_rn : ref_##P##trmm_kernel_rt)(m, n, n, alpha, pa, pb, B,  \
                                                                    ldb, 0);                   \
    }                                                                                          \
    free(pa);                                                                                  \
    free(pb);                                                                                  \
    free(t);                                                                                   \
    return rc;                                                                                 \
  }

TRMM_DRIVER(double, d)
TRMM_DRIVER(float, s)
