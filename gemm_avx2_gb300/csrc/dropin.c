/* dropin.c -- the drop-in BLAS symbol of DGEMM.so (built with -DDOUBLE) or
 * SGEMM.so.  It is the only symbol each library exports, exactly as the
 * reference's libraries (Makefile:14-18, src/gemm_driver.c:8-14,118), and it
 * forwards to the GB300 host-pointer path in libgemm_gb300.so.  Like the
 * reference it returns nothing; invalid arguments leave C untouched.
 *
 * Built with -DZCOMPLEX / -DCCOMPLEX it is ZGEMM.so / CGEMM.so instead: the
 * complex BLAS symbols zgemm_ and zgemm3m_ (cgemm_, cgemm3m_), complex scalars
 * and matrices as interleaved (re, im) pairs, trans 'N', 'T', 'C' or 'R'.  The
 * reference has complex GEMM only as OpenBLAS-style kernels
 * (OpenBLAS-like_implementation/zgemm_kernel_4x2_haswell.c,
 * zgemm3m_kernel_4x4_haswell.c and their c counterparts) that an OpenBLAS
 * driver reaches through these same BLAS names.
 *
 * GB300_DROPIN_FORM=split in the environment (read once per process) makes
 * dgemm_, sgemm_, zgemm_ and cgemm_ run the tensor-core forms with their tuned
 * parameters (the CRT form for FP64, 6xBF16 for FP32: at most the plain
 * kernels' error on finite data, see gemm_gb300.h) for problems of at least
 * 512^3 multiply-adds, where they are many times faster; smaller problems
 * keep the plain kernels.  A row of op(A) or column of op(B) holding Inf or
 * NaN then makes the whole row / column of the product NaN. */
#include <stdlib.h>
#include <string.h>

#include "../../include/gemm_gb300.h"

#define EXPORT __attribute__((visibility("default")))

static int split_form(int m, int n, int k) {
  static int mode = -1;  /* the same value in every thread: a benign race */
  if (mode < 0) {
    const char *e = getenv("GB300_DROPIN_FORM");
    mode = (e && strcmp(e, "split") == 0) ? 1 : 0;
  }
  return mode && (double)m * n * k >= 134217728.0;
}

#if defined(ZCOMPLEX)
EXPORT void zgemm_(const char *transa, const char *transb, const int *m, const int *n,
                   const int *k, const double *alpha, const double *a, const int *lda,
                   const double *b, const int *ldb, const double *beta, double *c,
                   const int *ldc) {
  (void)gb300_host_zgemm(*transa, *transb, *m, *n, *k, alpha, a, *lda, b, *ldb, beta, c, *ldc,
                         split_form(*m, *n, *k) ? GB300_CPLX_CRT : GB300_CPLX_4M, 0);
}
EXPORT void zgemm3m_(const char *transa, const char *transb, const int *m, const int *n,
                     const int *k, const double *alpha, const double *a, const int *lda,
                     const double *b, const int *ldb, const double *beta, double *c,
                     const int *ldc) {
  (void)gb300_host_zgemm(*transa, *transb, *m, *n, *k, alpha, a, *lda, b, *ldb, beta, c, *ldc,
                         GB300_CPLX_3M, 0);
}
#elif defined(CCOMPLEX)
EXPORT void cgemm_(const char *transa, const char *transb, const int *m, const int *n,
                   const int *k, const float *alpha, const float *a, const int *lda,
                   const float *b, const int *ldb, const float *beta, float *c, const int *ldc) {
  (void)gb300_host_cgemm(*transa, *transb, *m, *n, *k, alpha, a, *lda, b, *ldb, beta, c, *ldc,
                         split_form(*m, *n, *k) ? GB300_CPLX_SPLIT : GB300_CPLX_4M, 0);
}
EXPORT void cgemm3m_(const char *transa, const char *transb, const int *m, const int *n,
                     const int *k, const float *alpha, const float *a, const int *lda,
                     const float *b, const int *ldb, const float *beta, float *c,
                     const int *ldc) {
  (void)gb300_host_cgemm(*transa, *transb, *m, *n, *k, alpha, a, *lda, b, *ldb, beta, c, *ldc,
                         GB300_CPLX_3M, 0);
}
#elif defined(DOUBLE)
EXPORT void dgemm_(const char *transa, const char *transb, const int *m, const int *n,
                   const int *k, const double *alpha, const double *a, const int *lda,
                   const double *b, const int *ldb, const double *beta, double *c,
                   const int *ldc) {
  if (split_form(*m, *n, *k))
    (void)gb300_host_dgemm_ozaki2(*transa, *transb, *m, *n, *k, *alpha, a, *lda, b, *ldb, *beta,
                                  c, *ldc, 0);
  else
    (void)gb300_host_dgemm(*transa, *transb, *m, *n, *k, *alpha, a, *lda, b, *ldb, *beta, c,
                           *ldc);
}
#else
EXPORT void sgemm_(const char *transa, const char *transb, const int *m, const int *n,
                   const int *k, const float *alpha, const float *a, const int *lda,
                   const float *b, const int *ldb, const float *beta, float *c, const int *ldc) {
  if (split_form(*m, *n, *k))
    (void)gb300_host_sgemm_bf16x(*transa, *transb, *m, *n, *k, *alpha, a, *lda, b, *ldb, *beta,
                                 c, *ldc, 0);
  else
    (void)gb300_host_sgemm(*transa, *transb, *m, *n, *k, *alpha, a, *lda, b, *ldb, *beta, c,
                           *ldc);
}
#endif
