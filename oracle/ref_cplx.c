/*
 * ref_cplx.c -- harness around the reference's OpenBLAS-style complex GEMM
 * kernels, compiled from their sources by oracle/build.sh into
 * oracle/_ref/libcplx.so (x86-64 only: the kernels are AVX2 assembly).
 *
 * TEST INFRASTRUCTURE ONLY: the tests use it to pin the complex oracle's
 * conventions (conjugation variants, where alpha applies, what the 3M kernel
 * adds) to the reference's own code.
 *
 * The kernels take packed panels (the layout their loops walk):
 *   - A: row panels of UNROLL_M rows, then one panel each of UNROLL_M/2, ...,
 *     1 rows for the remainder; inside a panel, for each k the panel's rows
 *     (zgemm_kernel_4x2_haswell.c:223-238 COMPUTE, m loop 4/2/1;
 *      cgemm_kernel_8x2_haswell.c:263-280, m loop 8/4/2/1);
 *   - B: column panels of UNROLL_N columns, then one panel of the remainder's
 *     powers of two; inside a panel, for each k the panel's columns.  The
 *     complex kernels step through 2-column panels (r12 = k*2 elements,
 *     zgemm_kernel_4x2_haswell.c:48-58), the 3M kernels through 4-column
 *     panels (zgemm3m_kernel_4x4_haswell.c:185-222).
 * The driver is OpenBLAS's level-3 blocking in its simplest form, with each
 * kernel file's recommended block sizes (zgemm_kernel_4x2_haswell.c:4
 * GEMM_P = GEMM_Q = 192, cgemm_kernel_8x2_haswell.c:4 256,
 * zgemm3m_kernel_4x4_haswell.c:7 256, cgemm3m_kernel_8x4_haswell.c:7 320):
 * columns of C are split over the OpenMP team; per thread, for each K block of
 * Q, the thread's B columns are packed once and every P x Q block of A is packed
 * and multiplied.  So C += alpha * conj_a(A) * conj_b(B) (complex kernels) or
 * C += alpha * (A * B) (3M kernels, real A and B, complex C and alpha).
 */
#include <stdint.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef long BLASLONG;

#define KDECL(name, T)                                                                   \
  int name(BLASLONG m, BLASLONG n, BLASLONG k, T ar, T ai, T *A, T *B, T *C, BLASLONG ldc);
KDECL(ref_zgemm_kernel_nn, double)
KDECL(ref_zgemm_kernel_rn, double)
KDECL(ref_zgemm_kernel_nr, double)
KDECL(ref_zgemm_kernel_rr, double)
KDECL(ref_cgemm_kernel_nn, float)
KDECL(ref_cgemm_kernel_rn, float)
KDECL(ref_cgemm_kernel_nr, float)
KDECL(ref_cgemm_kernel_rr, float)
KDECL(ref_zgemm3m_kernel, double)
KDECL(ref_cgemm3m_kernel, float)

#define EXPORT __attribute__((visibility("default")))

/* Row panels of X (m x k, ld in elements of `cw` scalars each: 2 complex, 1
 * real), widths unroll, then powers of two below it. */
#define PACK_ROWS(T)                                                                       \
  static void pack_rows_##T(const T *X, long ld, long m, long k, int unroll, int cw, T *o) { \
    long i0 = 0;                                                                           \
    int w = unroll;                                                                        \
    while (i0 < m) {                                                                       \
      while (w > m - i0) w >>= 1;                                                          \
      for (long l = 0; l < k; l++)                                                         \
        for (int ii = 0; ii < w; ii++)                                                     \
          for (int c = 0; c < cw; c++) *o++ = X[cw * (i0 + ii + l * ld) + c];              \
      i0 += w;                                                                             \
    }                                                                                      \
  }                                                                                        \
  static void pack_cols_##T(const T *X, long ld, long k, long n, int unroll, int cw, T *o) { \
    long j0 = 0;                                                                           \
    int w = unroll;                                                                        \
    while (j0 < n) {                                                                       \
      while (w > n - j0) w >>= 1;                                                          \
      for (long l = 0; l < k; l++)                                                         \
        for (int jj = 0; jj < w; jj++)                                                     \
          for (int c = 0; c < cw; c++) *o++ = X[cw * (l + (j0 + jj) * ld) + c];            \
      j0 += w;                                                                             \
    }                                                                                      \
  }
PACK_ROWS(double)
PACK_ROWS(float)

typedef int (*zkern)(BLASLONG, BLASLONG, BLASLONG, double, double, double *, double *, double *,
                     BLASLONG);
typedef int (*ckern)(BLASLONG, BLASLONG, BLASLONG, float, float, float *, float *, float *,
                     BLASLONG);

/* Column chunk [j0, j1) of thread t out of nt: multiples of the B panel width. */
static void chunk(long n, int unroll, int t, int nt, long *j0, long *j1) {
  long panels = (n + unroll - 1) / unroll, per = (panels + nt - 1) / nt;
  *j0 = t * per * unroll;
  *j1 = (t + 1) * per * unroll;
  if (*j0 > n) *j0 = n;
  if (*j1 > n) *j1 = n;
}

#define CPLX_DRIVER(NAME, T, KS, MU, NU, CW, P, Q)                                          \
  EXPORT int NAME(int conj_a, int conj_b, long m, long n, long k, T ar, T ai, const T *A,   \
                  long lda, const T *B, long ldb, T *C, long ldc) {                         \
    int bad = 0;                                                                           \
    _Pragma("omp parallel reduction(|: bad)")                                              \
    {                                                                                      \
      int t = 0, nt = 1;                                                                   \
      THREAD_IDS(t, nt);                                                                   \
      long j0, j1;                                                                         \
      chunk(n, NU, t, nt, &j0, &j1);                                                       \
      const long nj = j1 - j0;                                                             \
      T *pb = nj > 0 ? malloc(sizeof(T) * CW * (Q * nj + 1)) : NULL;                       \
      T *pa = nj > 0 ? malloc(sizeof(T) * CW * (P * Q + 1)) : NULL;                        \
      if (nj > 0 && (!pa || !pb)) bad = 1;                                                 \
      for (long kk = 0; nj > 0 && !bad && kk < k; kk += Q) {                               \
        const long kq = k - kk < Q ? k - kk : Q;                                           \
        pack_cols_##T(B + CW * (kk + j0 * ldb), ldb, kq, nj, NU, CW, pb);                  \
        for (long mm = 0; mm < m; mm += P) {                                               \
          const long mp = m - mm < P ? m - mm : P;                                         \
          pack_rows_##T(A + CW * (mm + kk * lda), lda, mp, kq, MU, CW, pa);                \
          KS(conj_a, conj_b, mp, nj, kq, ar, ai, pa, pb, C + 2 * (mm + j0 * ldc), ldc);    \
        }                                                                                  \
      }                                                                                    \
      free(pa);                                                                            \
      free(pb);                                                                            \
    }                                                                                      \
    return bad ? -1 : 0;                                                                   \
  }

#ifdef _OPENMP
#define THREAD_IDS(t, nt) (t = omp_get_thread_num(), nt = omp_get_num_threads())
#else
#define THREAD_IDS(t, nt) (void)0
#endif

static const zkern zk[4] = {ref_zgemm_kernel_nn, ref_zgemm_kernel_rn, ref_zgemm_kernel_nr,
                            ref_zgemm_kernel_rr};
static const ckern ck[4] = {ref_cgemm_kernel_nn, ref_cgemm_kernel_rn, ref_cgemm_kernel_nr,
                            ref_cgemm_kernel_rr};
#define ZSEL(ca, cb, ...) zk[((ca) ? 1 : 0) + ((cb) ? 2 : 0)](__VA_ARGS__)
#define CSEL(ca, cb, ...) ck[((ca) ? 1 : 0) + ((cb) ? 2 : 0)](__VA_ARGS__)
#define Z3M(ca, cb, ...) ((void)(ca), (void)(cb), ref_zgemm3m_kernel(__VA_ARGS__))
#define C3M(ca, cb, ...) ((void)(ca), (void)(cb), ref_cgemm3m_kernel(__VA_ARGS__))

/* C (m x n complex, ldc) += alpha * conj_a(A) * conj_b(B); A m x k, B k x n
 * complex column-major.  Returns -1 on allocation failure. */
CPLX_DRIVER(ref_zgemm_conj, double, ZSEL, 4, 2, 2, 192, 192)
CPLX_DRIVER(ref_cgemm_conj, float, CSEL, 8, 2, 2, 256, 256)
/* C (complex) += alpha * (A * B) with real A (m x k) and B (k x n); conj_a and
 * conj_b are ignored. */
CPLX_DRIVER(ref_zgemm3m_conj, double, Z3M, 4, 4, 1, 256, 256)
CPLX_DRIVER(ref_cgemm3m_conj, float, C3M, 8, 4, 1, 320, 320)
