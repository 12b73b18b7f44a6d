/*
 * oracle.c -- CPU oracle for the sgemm_/dgemm_ path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this file; only the tests, the smoke check and the CPU-baseline leg of
 * the benchmark use it, and only as the checker.
 *
 * It holds four things:
 *
 *  1. A portable, counter-based input generator (splitmix64, Vigna 2014) that
 *     produces bit-identical FP64/FP32 uniform inputs on x86-64 and aarch64.
 *
 *  2. orc_refgemm_{d,s}: a restatement of the reference's GEMM algorithm
 *     (wjc404/GEMM_AVX2, src/gemm_driver.c:118-197) that reproduces its
 *     floating-point operation sequence element by element, so that it agrees
 *     with the reference library bit for bit:
 *       - C *= beta first when beta != 1            (src/gemm_driver.c:106-116,133)
 *       - nothing else when alpha == 0              (src/gemm_driver.c:134)
 *       - B is packed pre-multiplied by alpha        (src/gemm_copy.c:65,115,134)
 *       - columns are split over T OpenMP threads as n*t/T (src/gemm_driver.c:138)
 *       - per thread: the K-edge block (first K-(NK-1)*BDK columns of op(A))
 *         first, then the full K blocks            (src/gemm_driver.c:156-190)
 *       - each K block contributes C += acc, where acc is a fused-multiply-add
 *         chain started from zero                   (src/edge_kernel/gemm_edge_kernel_unroll6.h:46-52)
 *       - edge kernels (K-edge block, last N block of a thread) sum k in
 *         increasing order                          (src/edge_kernel/gemm_edge_kernel.c:39-117)
 *       - the full-block micro-kernel (every N block of a thread except its
 *         last, full K blocks) runs a 6-column skewed window: the K block is cut
 *         into UNROLL_N chunks of BDK/UNROLL_N, outer iteration `it` uses chunk
 *         it mod UNROLL_N, column j is live during iterations j-5..j, and the
 *         first UNROLL_N-1 columns of the block are stored twice, once after
 *         chunks 0..j and once (at the end, FIN_C) after chunks j+1..5
 *         (src/kernel/gemm_kernel.S:118-194,197-238; gemm_kernel_unroll6.S:70-229).
 *     Block constants come from the shipped tune headers (dgemm_tune.h:6-10,
 *     sgemm_tune.h:7-11) through src/gemm_set_parameters.h:55-61.
 *     The restatement works on whole columns rather than 8/16-row panels; rows
 *     are independent in the reference (one SIMD lane per row), so the per-element
 *     operation sequence is unchanged.
 *
 *  3. orc_dot2gemm_{d,s}: a compensated FP64 ground truth for
 *     alpha*op(A)*op(B) + beta*C (Ogita, Rump & Oishi, "Accurate sum and dot
 *     product", SIAM J. Sci. Comput. 26(6), 2005: Dot2 with TwoSum/TwoProduct;
 *     TwoProduct via fma).  Full-matrix and sampled-entry variants.
 *
 *  4. The exponent-spread generator a = (u - 0.5) * exp(phi * g), g ~ N(0,1)
 *     by Box-Muller from the same counter stream.
 *
 *  5. orc_{z,c}gemm_dot2: the complex ground truth (trans N/T/C/R, complex
 *     alpha and beta), full and sampled.
 *
 *  6. orc_{z,c}gemm_port: the arithmetic of the reference's complex kernels
 *     in portable C (the CPU baseline where those x86-64 kernels cannot run).
 *
 * Build with -ffp-contract=off (the recipe in oracle/build.sh does): every
 * rounding here is written out explicitly.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_API __attribute__((visibility("default")))

/* ------------------------------------------------------------------ */
/* 1. generator                                                        */
/* ------------------------------------------------------------------ */
static inline uint64_t sm64_mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
/* Stream key for (seed, stream); element idx of the stream is
 * sm64_mix(key + (idx+1) * golden). */
static inline uint64_t stream_key(uint64_t seed, uint64_t stream) {
  return sm64_mix(seed * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL * (stream + 1));
}
static inline uint64_t draw(uint64_t key, uint64_t idx) {
  return sm64_mix(key + (idx + 1) * 0x9E3779B97F4A7C15ULL);
}

ORC_API uint64_t orc_draw(uint64_t seed, uint64_t stream, uint64_t idx) {
  return draw(stream_key(seed, stream), idx);
}

/* x[i] = U[-1,1) on the 2^-52 grid, i = 0..n-1 */
ORC_API void orc_fill_uniform_d(double *x, int64_t n, uint64_t seed, uint64_t stream) {
  const uint64_t key = stream_key(seed, stream);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    uint64_t u = draw(key, (uint64_t)i);
    x[i] = (double)(int64_t)(u >> 11) * 0x1p-52 - 1.0;
  }
}
/* x[i] = U[-1,1) on the 2^-23 grid */
ORC_API void orc_fill_uniform_s(float *x, int64_t n, uint64_t seed, uint64_t stream) {
  const uint64_t key = stream_key(seed, stream);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    uint64_t u = draw(key, (uint64_t)i);
    x[i] = (float)(int32_t)(u >> 40) * 0x1p-23f - 1.0f;
  }
}
/* x[i] = (u - 0.5) * exp(phi * g): u ~ U[0,1), g ~ N(0,1) (Box-Muller).
 * Three draws per element: 3i (u), 3i+1 and 3i+2 (g). */
ORC_API void orc_fill_spread_d(double *x, int64_t n, uint64_t seed, uint64_t stream, double phi) {
  const uint64_t key = stream_key(seed, stream);
  const double two_pi = 6.283185307179586476925286766559;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    double u = (double)(draw(key, 3 * (uint64_t)i) >> 11) * 0x1p-53;
    double u1 = 1.0 - (double)(draw(key, 3 * (uint64_t)i + 1) >> 11) * 0x1p-53; /* (0,1] */
    double u2 = (double)(draw(key, 3 * (uint64_t)i + 2) >> 11) * 0x1p-53;
    double g = sqrt(-2.0 * log(u1)) * cos(two_pi * u2);
    x[i] = (u - 0.5) * exp(phi * g);
  }
}

/* ------------------------------------------------------------------ */
/* 2. reference-algorithm restatement                                  */
/* ------------------------------------------------------------------ */
/* Block geometry of the reference build (tune headers as shipped). */
typedef struct {
  int unroll_n; /* GEMM_UNROLL_N                               */
  int bdn;      /* GEMM_BLOCK_DIM_N = LOOP_TIMES_N * UNROLL_N   */
  int bdk;      /* GEMM_BLOCK_DIM_K = LOOP_TIMES_K * 8 * UNROLL_N */
} orc_geom;
static const orc_geom GEOM_D = {6, 16 * 6, 6 * 8 * 6};  /* dgemm_tune.h:6-8  */
static const orc_geom GEOM_S = {6, 32 * 6, 7 * 8 * 6};  /* sgemm_tune.h:7-9  */

ORC_API void orc_geometry(int is_double, int *unroll_n, int *bdn, int *bdk) {
  const orc_geom *g = is_double ? &GEOM_D : &GEOM_S;
  *unroll_n = g->unroll_n; *bdn = g->bdn; *bdk = g->bdk;
}

static inline int notrans(char t) { return t == 'N' || t == 'n'; } /* src/gemm_driver.c:17-18 */

/* The restatement is written once as a macro body over the element type. */
#define ORC_REFGEMM_BODY(FT, FMA, GEOM)                                                    \
  const int M = m, N = n, K = k;                                                           \
  const orc_geom G = GEOM;                                                                 \
  if (M <= 0 || N <= 0) return;                                                            \
  if (beta != (FT)1) { /* C_MULT_BETA, src/gemm_driver.c:106-116 */                        \
    for (int j = 0; j < N; j++)                                                            \
      for (int i = 0; i < M; i++) c[i + (int64_t)j * ldc] *= beta;                         \
  }                                                                                        \
  if (alpha == (FT)0) return;                                                              \
  if (T < 1) T = 1;                                                                        \
  const int BNK = (K - 1) / G.bdk + 1;            /* C truncation, K=0 -> 1 block */       \
  const int EDK = K - (BNK - 1) * G.bdk;                                                   \
  const int CH = G.bdk / G.unroll_n;              /* chunk of the skewed window */         \
  const int UN = G.unroll_n;                                                               \
  /* op(A) packed column by column for the whole K range: ap[i + p*M] = op(A)(i,p) */      \
  FT *ap = (FT *)malloc(sizeof(FT) * ((size_t)M * (size_t)(K > 0 ? K : 1)));               \
  for (int p = 0; p < K; p++)                                                              \
    for (int i = 0; i < M; i++)                                                            \
      ap[i + (int64_t)p * M] = notrans(ta) ? a[i + (int64_t)p * lda] : a[p + (int64_t)i * lda]; \
  _Pragma("omp parallel")                                                                  \
  {                                                                                        \
    FT *acc = (FT *)malloc(sizeof(FT) * (size_t)M);                                        \
    FT *acc2 = (FT *)malloc(sizeof(FT) * (size_t)M);                                       \
    FT *bcol = (FT *)malloc(sizeof(FT) * (size_t)(K > 0 ? K : 1));                         \
    _Pragma("omp for schedule(dynamic, 4)")                                                \
    for (int j = 0; j < N; j++) {                                                          \
      /* owning reference thread and position inside its column chunk */                   \
      int t = 0;                                                                           \
      while ((int64_t)N * (t + 1) / T <= j) t++;                                           \
      const int c0 = (int)((int64_t)N * t / T), c1 = (int)((int64_t)N * (t + 1) / T);      \
      const int Nt = c1 - c0, jl = j - c0;                                                 \
      const int BNN = (Nt - 1) / G.bdn + 1;                                                \
      const int nb = jl / G.bdn, jj = jl % G.bdn;                                          \
      const int full_n = nb < BNN - 1; /* the last N block of a thread is an edge block */ \
      FT *cc = c + (int64_t)j * ldc;                                                       \
      /* alpha-scaled column of op(B), src/gemm_copy.c:65 */                               \
      for (int p = 0; p < K; p++) {                                                        \
        FT bv = notrans(tb) ? b[p + (int64_t)j * ldb] : b[j + (int64_t)p * ldb];           \
        bcol[p] = bv * alpha;                                                              \
      }                                                                                    \
      /* K-edge block: k in [0, EDK), sequential (edge kernels) */                         \
      for (int i = 0; i < M; i++) acc[i] = (FT)0;                                          \
      for (int p = 0; p < EDK; p++) {                                                      \
        const FT bv = bcol[p]; const FT *ac = ap + (int64_t)p * M;                         \
        for (int i = 0; i < M; i++) acc[i] = FMA(ac[i], bv, acc[i]);                       \
      }                                                                                    \
      for (int i = 0; i < M; i++) cc[i] = cc[i] + acc[i];                                  \
      /* full K blocks */                                                                  \
      for (int kb = 0; kb < BNK - 1; kb++) {                                               \
        const int k0 = EDK + kb * G.bdk;                                                   \
        if (!full_n) { /* gemmblkirregnccc / gemmblkirregccc: sequential */                \
          for (int i = 0; i < M; i++) acc[i] = (FT)0;                                      \
          for (int p = k0; p < k0 + G.bdk; p++) {                                          \
            const FT bv = bcol[p]; const FT *ac = ap + (int64_t)p * M;                     \
            for (int i = 0; i < M; i++) acc[i] = FMA(ac[i], bv, acc[i]);                   \
          }                                                                                \
          for (int i = 0; i < M; i++) cc[i] = cc[i] + acc[i];                              \
        } else if (jj >= UN - 1) { /* one window pass: chunks (jj-UN+1..jj) mod UN */      \
          for (int i = 0; i < M; i++) acc[i] = (FT)0;                                      \
          for (int q = 0; q < UN; q++) {                                                   \
            const int ch = (jj - (UN - 1) + q) % UN;                                       \
            for (int p = k0 + ch * CH; p < k0 + (ch + 1) * CH; p++) {                      \
              const FT bv = bcol[p]; const FT *ac = ap + (int64_t)p * M;                   \
              for (int i = 0; i < M; i++) acc[i] = FMA(ac[i], bv, acc[i]);                 \
            }                                                                              \
          }                                                                                \
          for (int i = 0; i < M; i++) cc[i] = cc[i] + acc[i];                              \
        } else { /* wrapped column: chunks 0..jj stored first, jj+1..UN-1 at FIN_C */      \
          for (int i = 0; i < M; i++) { acc[i] = (FT)0; acc2[i] = (FT)0; }                 \
          for (int p = k0; p < k0 + (jj + 1) * CH; p++) {                                  \
            const FT bv = bcol[p]; const FT *ac = ap + (int64_t)p * M;                     \
            for (int i = 0; i < M; i++) acc[i] = FMA(ac[i], bv, acc[i]);                   \
          }                                                                                \
          for (int p = k0 + (jj + 1) * CH; p < k0 + G.bdk; p++) {                          \
            const FT bv = bcol[p]; const FT *ac = ap + (int64_t)p * M;                     \
            for (int i = 0; i < M; i++) acc2[i] = FMA(ac[i], bv, acc2[i]);                 \
          }                                                                                \
          for (int i = 0; i < M; i++) cc[i] = cc[i] + acc[i];                              \
          for (int i = 0; i < M; i++) cc[i] = cc[i] + acc2[i];                             \
        }                                                                                  \
      }                                                                                    \
    }                                                                                      \
    free(acc); free(acc2); free(bcol);                                                     \
  }                                                                                        \
  free(ap);

/* T = the reference's OpenMP team size (omp_get_max_threads() there). */
ORC_API void orc_refgemm_d(char ta, char tb, int m, int n, int k, double alpha, const double *a,
                           int lda, const double *b, int ldb, double beta, double *c, int ldc,
                           int T) {
  ORC_REFGEMM_BODY(double, fma, GEOM_D)
}
ORC_API void orc_refgemm_s(char ta, char tb, int m, int n, int k, float alpha, const float *a,
                           int lda, const float *b, int ldb, float beta, float *c, int ldc,
                           int T) {
  ORC_REFGEMM_BODY(float, fmaf, GEOM_S)
}

/* ------------------------------------------------------------------ */
/* 3. compensated FP64 ground truth (Dot2)                             */
/* ------------------------------------------------------------------ */
static inline void two_sum(double x, double y, double *s, double *e) {
  double z = x + y, t = z - x;
  *s = z;
  *e = (x - (z - t)) + (y - t);
}
static inline void two_prod(double x, double y, double *p, double *e) {
  double z = x * y;
  *p = z;
  *e = fma(x, y, -z);
}
/* alpha * dot + beta * c0 with the dot in double-double, rounded once at the end. */
static inline double dot2_finish(double s, double err, double alpha, double beta, double c0) {
  double ph, pl, qh, ql, rh, rl;
  two_prod(alpha, s, &ph, &pl);
  pl += alpha * err;
  two_prod(beta, c0, &qh, &ql);
  two_sum(ph, qh, &rh, &rl);
  rl += pl + ql;
  return rh + rl;
}

#define ORC_DOT2_ELEM(AT, BT)                                                              \
  double s = 0.0, err = 0.0;                                                               \
  for (int p = 0; p < k; p++) {                                                            \
    double av = notrans(ta) ? (double)a[i + (int64_t)p * lda] : (double)a[p + (int64_t)i * lda]; \
    double bv = notrans(tb) ? (double)b[p + (int64_t)j * ldb] : (double)b[j + (int64_t)p * ldb]; \
    double ph, pe, q;                                                                      \
    two_prod(av, bv, &ph, &pe);                                                            \
    two_sum(s, ph, &s, &q);                                                                \
    err += q + pe;                                                                         \
  }

/* out[i + j*ldo] = alpha*op(A)op(B) + beta*C evaluated with Dot2 (C read from c). */
ORC_API void orc_dot2gemm_d(char ta, char tb, int m, int n, int k, double alpha, const double *a,
                            int lda, const double *b, int ldb, double beta, const double *c,
                            int ldc, double *out, int ldo) {
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
  for (int j = 0; j < n; j++)
    for (int i = 0; i < m; i++) {
      ORC_DOT2_ELEM(double, double)
      out[i + (int64_t)j * ldo] = dot2_finish(s, err, alpha, beta, c[i + (int64_t)j * ldc]);
    }
}
ORC_API void orc_dot2gemm_s(char ta, char tb, int m, int n, int k, double alpha, const float *a,
                            int lda, const float *b, int ldb, double beta, const float *c, int ldc,
                            double *out, int ldo) {
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
  for (int j = 0; j < n; j++)
    for (int i = 0; i < m; i++) {
      ORC_DOT2_ELEM(float, float)
      out[i + (int64_t)j * ldo] =
          dot2_finish(s, err, alpha, beta, c ? (double)c[i + (int64_t)j * ldc] : 0.0);
    }
}
/* Sampled entries: out[q] for (rows[q], cols[q]), q = 0..count-1. */
ORC_API void orc_dot2gemm_sampled_d(char ta, char tb, int m, int n, int k, double alpha,
                                    const double *a, int lda, const double *b, int ldb,
                                    double beta, const double *c, int ldc, const int64_t *rows,
                                    const int64_t *cols, int64_t count, double *out) {
  (void)m; (void)n;
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t q = 0; q < count; q++) {
    const int64_t i = rows[q], j = cols[q];
    ORC_DOT2_ELEM(double, double)
    out[q] = dot2_finish(s, err, alpha, beta, c ? c[i + j * ldc] : 0.0);
  }
}
ORC_API void orc_dot2gemm_sampled_s(char ta, char tb, int m, int n, int k, double alpha,
                                    const float *a, int lda, const float *b, int ldb, double beta,
                                    const float *c, int ldc, const int64_t *rows,
                                    const int64_t *cols, int64_t count, double *out) {
  (void)m; (void)n;
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t q = 0; q < count; q++) {
    const int64_t i = rows[q], j = cols[q];
    ORC_DOT2_ELEM(float, float)
    out[q] = dot2_finish(s, err, alpha, beta, c ? (double)c[i + j * ldc] : 0.0);
  }
}

/* ------------------------------------------------------------------ */
/* 5. complex ground truth                                             */
/* ------------------------------------------------------------------ */
/* Complex GEMM C = alpha*op(A)*op(B) + beta*C on interleaved (re, im) storage,
 * the semantics of the reference's OpenBLAS-style complex kernels
 * (OpenBLAS-like_implementation/zgemm_kernel_4x2_haswell.c:6-21: A_CONJ/B_CONJ
 * per variant; :224-243 CNAME adds alpha*A*B to C) extended with the BLAS
 * trans codes: 'N' op(X) = X, 'T' X^T, 'C' conj(X)^T, 'R' conj(X); any other
 * character is a transpose, like the real path.  Real and imaginary parts are
 * Dot2 sums of 2k exact products; alpha and beta are applied in double-double
 * and rounded once. */
static inline int ctrans(char t) { return !(t == 'N' || t == 'n' || t == 'R' || t == 'r'); }
static inline int cconj(char t) { return t == 'C' || t == 'c' || t == 'R' || t == 'r'; }
static inline void dd_acc(double *h, double *l, double x, double y) {
  double p, e, q;
  two_prod(x, y, &p, &e);
  two_sum(*h, p, h, &q);
  *l += q + e;
}

#define ORC_ZDOT2_ELEM(T)                                                                  \
  double sr = 0.0, er = 0.0, si = 0.0, ei = 0.0;                                           \
  for (int p = 0; p < k; p++) {                                                            \
    const T *ap = ctrans(ta) ? a + 2 * (p + (int64_t)i * lda) : a + 2 * (i + (int64_t)p * lda); \
    const T *bp = ctrans(tb) ? b + 2 * (j + (int64_t)p * ldb) : b + 2 * (p + (int64_t)j * ldb); \
    const double ar = ap[0], ai = cconj(ta) ? -(double)ap[1] : (double)ap[1];            \
    const double br = bp[0], bi = cconj(tb) ? -(double)bp[1] : (double)bp[1];            \
    dd_acc(&sr, &er, ar, br);                                                              \
    dd_acc(&sr, &er, -ai, bi);                                                             \
    dd_acc(&si, &ei, ar, bi);                                                              \
    dd_acc(&si, &ei, ai, br);                                                              \
  }

static inline void zdot2_finish(double sr, double er, double si, double ei, const double *alpha,
                                const double *beta, double cr, double ci, double *out) {
  double h = 0.0, l = 0.0;
  dd_acc(&h, &l, alpha[0], sr);
  l += alpha[0] * er;
  dd_acc(&h, &l, -alpha[1], si);
  l -= alpha[1] * ei;
  dd_acc(&h, &l, beta[0], cr);
  dd_acc(&h, &l, -beta[1], ci);
  out[0] = h + l;
  h = 0.0; l = 0.0;
  dd_acc(&h, &l, alpha[0], si);
  l += alpha[0] * ei;
  dd_acc(&h, &l, alpha[1], sr);
  l += alpha[1] * er;
  dd_acc(&h, &l, beta[0], ci);
  dd_acc(&h, &l, beta[1], cr);
  out[1] = h + l;
}

/* out (complex, ld ldo) = alpha*op(A)op(B) + beta*C; c may be NULL (C = 0). */
ORC_API void orc_zgemm_dot2(char ta, char tb, int m, int n, int k, const double *alpha,
                            const double *a, int lda, const double *b, int ldb,
                            const double *beta, const double *c, int ldc, double *out, int ldo) {
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
  for (int j = 0; j < n; j++)
    for (int i = 0; i < m; i++) {
      ORC_ZDOT2_ELEM(double)
      const double *cp = c ? c + 2 * (i + (int64_t)j * ldc) : NULL;
      zdot2_finish(sr, er, si, ei, alpha, beta, cp ? cp[0] : 0.0, cp ? cp[1] : 0.0,
                   out + 2 * (i + (int64_t)j * ldo));
    }
}
ORC_API void orc_cgemm_dot2(char ta, char tb, int m, int n, int k, const double *alpha,
                            const float *a, int lda, const float *b, int ldb, const double *beta,
                            const float *c, int ldc, double *out, int ldo) {
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
  for (int j = 0; j < n; j++)
    for (int i = 0; i < m; i++) {
      ORC_ZDOT2_ELEM(float)
      const float *cp = c ? c + 2 * (i + (int64_t)j * ldc) : NULL;
      zdot2_finish(sr, er, si, ei, alpha, beta, cp ? cp[0] : 0.0, cp ? cp[1] : 0.0,
                   out + 2 * (i + (int64_t)j * ldo));
    }
}
/* Sampled entries (rows[q], cols[q]) of the complex result, out[2q], out[2q+1]. */
ORC_API void orc_zgemm_dot2_sampled(char ta, char tb, int k, const double *alpha, const double *a,
                                    int lda, const double *b, int ldb, const double *beta,
                                    const double *c, int ldc, const int64_t *rows,
                                    const int64_t *cols, int64_t count, double *out) {
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t q = 0; q < count; q++) {
    const int64_t i = rows[q], j = cols[q];
    ORC_ZDOT2_ELEM(double)
    const double *cp = c + 2 * (i + j * ldc);
    zdot2_finish(sr, er, si, ei, alpha, beta, cp[0], cp[1], out + 2 * q);
  }
}
ORC_API void orc_cgemm_dot2_sampled(char ta, char tb, int k, const double *alpha, const float *a,
                                    int lda, const float *b, int ldb, const double *beta,
                                    const float *c, int ldc, const int64_t *rows,
                                    const int64_t *cols, int64_t count, double *out) {
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t q = 0; q < count; q++) {
    const int64_t i = rows[q], j = cols[q];
    ORC_ZDOT2_ELEM(float)
    const float *cp = c + 2 * (i + j * ldc);
    zdot2_finish(sr, er, si, ei, alpha, beta, cp[0], cp[1], out + 2 * q);
  }
}

/* ------------------------------------------------------------------ */
/* 6. complex kernel arithmetic, portable (CPU baseline)               */
/* ------------------------------------------------------------------ */
/* The operation sequence of the reference's complex kernels in their
 * expanded-accumulator form (OpenBLAS-like_implementation/
 * zgemm_kernel_4x2_haswell.c:26-33 acc_m2n1_exp, :66-71 cont_expacc, :72-80
 * save): per element four FMA chains over k, s1 = sum ar*br, s2 = sum ai*bi,
 * s3 = sum ar*bi, s4 = sum ai*br (conjugation flips the sign of the imaginary
 * part it applies to), combined as (s1 - s2, s3 + s4), then C += alpha * that.
 * A is m x k, B k x n, complex column-major.  Used as the CPU baseline on hosts
 * where the kernels themselves (x86-64 AVX2) cannot run; columns of C are
 * split over the OpenMP team, rows are the vector dimension. */
#define ORC_ZPORT(NAME, T, FMA)                                                            \
  ORC_API void NAME(int conj_a, int conj_b, int m, int n, int k, const T *alpha, const T *a, \
                    int lda, const T *b, int ldb, T *c, int ldc) {                         \
    _Pragma("omp parallel")                                                                \
    {                                                                                      \
      T *acc = (T *)malloc(sizeof(T) * 4 * (size_t)(m > 0 ? m : 1));                      \
      T *s1 = acc, *s2 = acc + m, *s3 = acc + 2 * m, *s4 = acc + 3 * m;                    \
      const T sa = conj_a ? (T)-1 : (T)1, sb = conj_b ? (T)-1 : (T)1;                      \
      _Pragma("omp for schedule(static)")                                                  \
      for (int j = 0; j < n; j++) {                                                        \
        for (int i = 0; i < m; i++) s1[i] = s2[i] = s3[i] = s4[i] = (T)0;                 \
        for (int p = 0; p < k; p++) {                                                      \
          const T br = b[2 * (p + (int64_t)j * ldb)];                                      \
          const T bi = sb * b[2 * (p + (int64_t)j * ldb) + 1];                             \
          const T *ap = a + 2 * (int64_t)p * lda;                                          \
          for (int i = 0; i < m; i++) {                                                    \
            const T ar = ap[2 * i], ai = sa * ap[2 * i + 1];                               \
            s1[i] = FMA(ar, br, s1[i]);                                                    \
            s2[i] = FMA(ai, bi, s2[i]);                                                    \
            s3[i] = FMA(ar, bi, s3[i]);                                                    \
            s4[i] = FMA(ai, br, s4[i]);                                                    \
          }                                                                                \
        }                                                                                  \
        T *cp = c + 2 * (int64_t)j * ldc;                                                  \
        for (int i = 0; i < m; i++) {                                                      \
          const T re = s1[i] - s2[i], im = s3[i] + s4[i];                                  \
          cp[2 * i] = FMA(alpha[0], re, FMA(-alpha[1], im, cp[2 * i]));                    \
          cp[2 * i + 1] = FMA(alpha[0], im, FMA(alpha[1], re, cp[2 * i + 1]));             \
        }                                                                                  \
      }                                                                                    \
      free(acc);                                                                           \
    }                                                                                      \
  }
ORC_ZPORT(orc_zgemm_port, double, fma)
ORC_ZPORT(orc_cgemm_port, float, fmaf)

ORC_API int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
