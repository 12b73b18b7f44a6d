/* dropin.c -- the drop-in BLAS symbol of DGEMM.so (built with -DDOUBLE) or
 * SGEMM.so.  It is the only symbol each library exports, exactly as the
 * reference's libraries (Makefile:14-18, src/gemm_driver.c:8-14,118), and it
 * forwards to the GB300 host-pointer path in libgemm_gb300.so.  Like the
 * reference it returns nothing; invalid arguments leave C untouched. */
#include "../../include/gemm_gb300.h"

#define EXPORT __attribute__((visibility("default")))

#ifdef DOUBLE
EXPORT void dgemm_(const char *transa, const char *transb, const int *m, const int *n,
                   const int *k, const double *alpha, const double *a, const int *lda,
                   const double *b, const int *ldb, const double *beta, double *c,
                   const int *ldc) {
  (void)gb300_host_dgemm(*transa, *transb, *m, *n, *k, *alpha, a, *lda, b, *ldb, *beta, c, *ldc);
}
#else
EXPORT void sgemm_(const char *transa, const char *transb, const int *m, const int *n,
                   const int *k, const float *alpha, const float *a, const int *lda,
                   const float *b, const int *ldb, const float *beta, float *c, const int *ldc) {
  (void)gb300_host_sgemm(*transa, *transb, *m, *n, *k, *alpha, a, *lda, b, *ldb, *beta, c, *ldc);
}
#endif
