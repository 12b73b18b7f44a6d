/*
 * gemm_gb300.h -- C ABI of the GB300 (sm_103a) GEMM library.
 *
 * Two layers:
 *
 *  1. The drop-in BLAS symbols.  DGEMM.so exports exactly `dgemm_`, SGEMM.so
 *     exactly `sgemm_`, with the reference's Fortran-style signature and
 *     semantics (wjc404/GEMM_AVX2 src/gemm_driver.c:118, README.md:10).  They
 *     take HOST pointers, stage the operands through HBM, run the plain
 *     FP64/FP32 kernels and return when C has been written back.  ZGEMM.so and
 *     CGEMM.so export the complex BLAS symbols `zgemm_`/`zgemm3m_` and
 *     `cgemm_`/`cgemm3m_` the same way (complex arguments as interleaved
 *     (re, im) pairs).
 *
 *  2. Device-pointer entry points in libgemm_gb300.so (prefix gb300_).  All
 *     matrices are column-major device buffers; every call is stream-ordered
 *     and asynchronous (the stream is a cudaStream_t passed as void*, NULL =
 *     legacy default stream).  They return a gb300_status.  Operand
 *     semantics are the reference's (see `dgemm_` below).
 *
 * Semantics shared by every entry point (src/gemm_driver.c:17-18,118-197):
 *   - op(X) = X when trans is 'N' or 'n'; ANY other character means transpose.
 *   - C = beta*C first (when beta != 1; beta == 0 still multiplies, so NaN/Inf
 *     already in C propagate), then C += alpha*op(A)*op(B) when alpha != 0.
 *     alpha == 0 therefore never reads A or B.
 *   - m, n or k == 0 is valid.  Only the m x n window of C is written.
 *   - Invalid arguments (negative sizes, lda/ldb/ldc smaller than the stored
 *     rows, at least 1): the drop-in symbols return without touching C (the
 *     reference has no argument checks; this is the safe reading of its
 *     undefined behaviour); the gb300_ calls return GB300_ERR_ARG.
 */
#ifndef GEMM_GB300_H
#define GEMM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GB300_OK = 0,
  GB300_ERR_ARG = 1,         /* invalid size / leading dimension / option   */
  GB300_ERR_CUDA = 2,        /* a CUDA runtime call failed                    */
  GB300_ERR_TIMEOUT = 3,     /* a kernel's bounded wait expired (device error word set) */
  GB300_ERR_NOMEM = 4,       /* device workspace could not be allocated       */
  GB300_ERR_UNSUPPORTED = 5, /* option this library does not implement       */
  GB300_ERR_WORKSPACE = 6,   /* caller-provided workspace too small           */
  GB300_ERR_NOALLOC_LIMIT = 7 /* problem needs more scratch than gb300_sgemm_bf16x_noalloc's fixed array */
} gb300_status;

/* ------------------------------------------------------------------------
 * 1. Drop-in symbols (DGEMM.so / SGEMM.so).
 *    Replace: src/gemm_driver.c:118 (GEMM_DRIVER = dgemm_ / sgemm_, :8-14).
 *    Synchronous; host pointers; 32-bit int sizes (LP64, no ILP64).
 * ---------------------------------------------------------------------- */
void dgemm_(const char *transa, const char *transb, const int *m, const int *n, const int *k,
            const double *alpha, const double *a, const int *lda, const double *b,
            const int *ldb, const double *beta, double *c, const int *ldc);
void sgemm_(const char *transa, const char *transb, const int *m, const int *n, const int *k,
            const float *alpha, const float *a, const int *lda, const float *b, const int *ldb,
            const float *beta, float *c, const int *ldc);

/* Host-pointer forms of the drop-in symbols with a status return
 * (libgemm_gb300.so).  dgemm_/sgemm_ call these and drop the status.
 * Replace: src/gemm_driver.c:118. */
int gb300_host_dgemm(char transa, char transb, int m, int n, int k, double alpha, const double *a,
                     int lda, const double *b, int ldb, double beta, double *c, int ldc);
int gb300_host_sgemm(char transa, char transb, int m, int n, int k, float alpha, const float *a,
                     int lda, const float *b, int ldb, float beta, float *c, int ldc);

/* ------------------------------------------------------------------------
 * 2. Device-pointer entry points (libgemm_gb300.so).
 * ---------------------------------------------------------------------- */

/* Plain native-precision forms: the same computation as dgemm_/sgemm_
 * (src/gemm_driver.c:118-197) on device buffers.  FP64 runs on the FP64
 * tensor path (DMMA), FP32 on the FFMA pipe. */
int gb300_dgemm(char transa, char transb, int m, int n, int k, double alpha, const double *A,
                int lda, const double *B, int ldb, double beta, double *C, int ldc,
                void *stream);
int gb300_sgemm(char transa, char transb, int m, int n, int k, float alpha, const float *A,
                int lda, const float *B, int ldb, float beta, float *C, int ldc, void *stream);

/* Split-precision SGEMM on the BF16 tensor cores (tcgen05, FP32 accumulation
 * in TMEM).  No reference counterpart: a tensor-core form of sgemm_
 * (src/gemm_driver.c:118) with the same operand semantics.
 *   products = 3: A = Ah + Al, B = Bh + Bl (BF16 hi + BF16 lo of the residual),
 *                 C += Ah*Bh + Ah*Bl + Al*Bh                  ("3xBF16")
 *   products = 6: three BF16 terms per operand, all cross products whose
 *                 order sum is <= 2                              ("6xBF16")
 *   products = GB300_SPLIT_FP16X3: rows of op(A) and columns of op(B) scaled
 *                 by powers of two into (-2^15, 2^15), then FP16 hi + FP16 lo
 *                 (the residual times 2^11) on the FP16 tensor cores,
 *                 C += 2^(e_i + f_j) (Ah*Bh + (Ah*Bl + Al*Bh) * 2^-11)
 *                 ("3xFP16", the lo*lo product dropped).  Each operand keeps
 *                 about 22 bits; values below 2^-50 of their row's (column's)
 *                 max |.| are lost, so accuracy is normwise per row/column,
 *                 like the Ozaki form.  A row or column holding Inf/NaN gives
 *                 a NaN row/column of the product (as the BF16 forms).
 *   products = 0: the autotuned choice for the shape class (gb300_autotune),
 *                 else 6
 * Uses a device workspace of gb300_split_workspace_bytes() bytes, allocated
 * and cached by the library (the _ws variant takes the caller's instead). */
enum { GB300_SPLIT_FP16X3 = 0x103 };
int gb300_sgemm_bf16x(char transa, char transb, int m, int n, int k, float alpha, const float *A,
                      int lda, const float *B, int ldb, float beta, float *C, int ldc,
                      int products, void *stream);
int gb300_sgemm_bf16x_ws(char transa, char transb, int m, int n, int k, float alpha,
                         const float *A, int lda, const float *B, int ldb, float beta, float *C,
                         int ldc, int products, void *workspace, size_t workspace_bytes,
                         void *stream);

/* Ozaki-scheme DGEMM on the tensor cores.  No reference counterpart: a
 * tensor-core form of dgemm_ (src/gemm_driver.c:118).  Rows of op(A) and
 * columns of op(B) are scaled by powers of two and cut into `slices`
 * signed 7-bit integer slices (int8 range, |v| <= 127); the slice products
 * with i + j <= slices + 1 are accumulated exactly (integer-valued FP32 in
 * TMEM over K chunks of 1024, whose sums stay below 2^24, flushed into 32-bit
 * integers) and recombined
 * in FP64 with the fused alpha/beta epilogue.  slices in [2, 12]; 0 picks the
 * autotuned default for the shape class. */
int gb300_dgemm_ozaki(char transa, char transb, int m, int n, int k, double alpha,
                      const double *A, int lda, const double *B, int ldb, double beta, double *C,
                      int ldc, int slices, void *stream);
int gb300_dgemm_ozaki_ws(char transa, char transb, int m, int n, int k, double alpha,
                         const double *A, int lda, const double *B, int ldb, double beta,
                         double *C, int ldc, int slices, void *workspace, size_t workspace_bytes,
                         void *stream);

/* BF16xP split SGEMM that allocates nothing.  No counterpart in the reference.
 * For callers that may not call cudaMalloc/cudaFree: code running under a
 * framework that owns all device memory (a pool or a fixed budget that must
 * not be bypassed) and code on a latency-critical path.  Same arguments and
 * result as gb300_sgemm_bf16x (products 3, 6 or GB300_SPLIT_FP16X3), but the scratch is a fixed
 * 32 MiB array that is part of the library's device image (each GPU that loads
 * the library holds it until exit); the call allocates and frees nothing.
 *   - Problems whose scratch (gb300_split_workspace_bytes(0, m, n, k,
 *     products)) exceeds 32 MiB are rejected with GB300_ERR_NOALLOC_LIMIT
 *     (3xBF16 and FP16X3: up to about m = n = k = 1980; 6xBF16: about 1600).
 *   - The first call on a device looks up the array's device address (set-up,
 *     once per device); make that first call before any stream capture.
 *   - Every call uses the same array: calls whose execution overlaps on the
 *     GPU (different streams, or different host threads) race on it; order
 *     them on one stream.  Each call writes all the scratch it reads, so no
 *     state carries over from the previous call.
 *   - products may also be GB300_SPLIT_FP16X3 (the scaled FP16 form); its
 *     scratch includes the row / column scale exponents and is sized by the
 *     same gb300_split_workspace_bytes(0, m, n, k, GB300_SPLIT_FP16X3).
 *   - The GEMM runs pair MMAs on 2-CTA clusters when op(A) has more than
 *     128 rows (the default cluster mode; GB300_TUNE_PAIR_MMA = 2 makes it
 *     one CTA per tile); every load lands in the issuing CTA's own memory.
 *   - Kernel time-outs are recorded in an error word of this entry point
 *     (a static device variable, so no allocation either);
 *     gb300_device_error reports it after a stream synchronisation. */
int gb300_sgemm_bf16x_noalloc(char transa, char transb, int m, int n, int k, float alpha,
                              const float *A, int lda, const float *B, int ldb, float beta,
                              float *C, int ldc, int products, void *stream);

/* Two-phase forms of the split GEMMs (no reference counterpart; the split of
 * the reference's pack-then-compute structure, src/gemm_driver.c:157-188):
 * _prepare writes the split/sliced operands of op(A), op(B) into the
 * workspace; _run computes C = alpha*op(A)op(B) + beta*C from a workspace
 * prepared for the same m, n, k and products/slices.  One prepared operand
 * set can serve several _run calls (e.g. different alpha/beta/C). */
int gb300_sgemm_bf16x_prepare(char transa, char transb, int m, int n, int k, const float *A,
                              int lda, const float *B, int ldb, int products, void *workspace,
                              size_t workspace_bytes, void *stream);
int gb300_sgemm_bf16x_run(int m, int n, int k, float alpha, float beta, float *C, int ldc,
                          int products, const void *workspace, size_t workspace_bytes,
                          void *stream);
int gb300_dgemm_ozaki_prepare(char transa, char transb, int m, int n, int k, const double *A,
                              int lda, const double *B, int ldb, int slices, void *workspace,
                              size_t workspace_bytes, void *stream);
int gb300_dgemm_ozaki_run(int m, int n, int k, double alpha, double beta, double *C, int ldc,
                          int slices, const void *workspace, size_t workspace_bytes,
                          void *stream);

/* Host-pointer (synchronous, staged through HBM) forms of the split GEMMs,
 * with the drop-in's argument conventions (src/gemm_driver.c:118). */
int gb300_host_sgemm_bf16x(char transa, char transb, int m, int n, int k, float alpha,
                           const float *a, int lda, const float *b, int ldb, float beta, float *c,
                           int ldc, int products);
int gb300_host_dgemm_ozaki(char transa, char transb, int m, int n, int k, double alpha,
                           const double *a, int lda, const double *b, int ldb, double beta,
                           double *c, int ldc, int slices);

/* ------------------------------------------------------------------------
 * Grouped GEMMs (no reference counterpart: the reference computes one problem
 * per call, src/gemm_driver.c:118).  Many independent problems of any sizes,
 * FP64 ('d') or FP32 ('s'), any transposes and leading dimensions, each with
 * the semantics of dgemm_/sgemm_ above, on device buffers.
 * ---------------------------------------------------------------------- */
typedef struct {
  char transa, transb;
  char precision; /* 'd': A, B, C are double; 's': float */
  int m, n, k;
  double alpha, beta; /* rounded to float for 's' problems */
  const void *A;
  int lda;
  const void *B;
  int ldb;
  void *C;
  int ldc;
} gb300_gemm_problem;

/* Plain (native precision) forms of all problems in ONE persistent launch:
 * the 128x128 tiles of all problems are ordered longest-work-first and CTAs
 * take them from a device-side atomic counter.  Problems must not overlap
 * in C.  Returns GB300_ERR_ARG (and launches nothing) if any problem is
 * invalid.  The _ws form takes a caller workspace of
 * gb300_grouped_workspace_bytes(count) bytes (metadata: tensor maps, tile
 * table); the other uses a library-owned one. */
size_t gb300_grouped_workspace_bytes(int count);
int gb300_gemm_grouped(const gb300_gemm_problem *problems, int count, void *stream);
int gb300_gemm_grouped_ws(const gb300_gemm_problem *problems, int count, void *workspace,
                          size_t workspace_bytes, void *stream);

/* A fixed batch captured once into a CUDA graph and replayed.  The problem
 * table, tensor maps and all workspace are built at creation (which may
 * allocate and synchronise); each launch replays the graph on `stream` with
 * no host-side work: the operand pointers are fixed, their contents may
 * change between launches.
 *   form 0: plain forms, one persistent launch (as gb300_gemm_grouped);
 *   form 1: split forms (FP32: 6xBF16, FP64: the CRT form with the tuned /
 *           default moduli count): the operands of every problem are
 *           prepared in parallel branches (GB300_TUNE_GRAPH_BRANCHES), then
 *           ONE persistent launch runs the residue GEMMs of all FP64
 *           problems and ONE the 6xBF16 GEMMs of all FP32 problems (128 x 128
 *           tiles of all problems, costliest first), then the FP64 problems'
 *           reconstructions run in branches.  Each problem has its own
 *           workspace (the graph holds the sum of the per-problem workspace
 *           sizes).  Results are bit-identical to gb300_dgemm_ozaki2 /
 *           gb300_sgemm_bf16x(products = 6) called on each problem.
 * gb300_grouped_graph_stats: the graph's kernel nodes and, of those, its
 * GEMM launches (1 for form 0; at most 2 for form 1). */
typedef struct gb300_grouped_graph_s *gb300_grouped_graph;
int gb300_grouped_graph_create(const gb300_gemm_problem *problems, int count, int form,
                               gb300_grouped_graph *out);
int gb300_grouped_graph_launch(gb300_grouped_graph graph, void *stream);
int gb300_grouped_graph_stats(gb300_grouped_graph graph, int *kernel_nodes, int *gemm_launches);
int gb300_grouped_graph_destroy(gb300_grouped_graph graph);

/* ------------------------------------------------------------------------
 * Triangular solve / multiply on top of the GEMM (BLAS semantics; the
 * reference has these only as OpenBLAS-style packed-panel kernels,
 * OpenBLAS-like_implementation/TRSM_KERNEL_*_simplified.c and
 * trmm_kernel_4x8_simplified.c, outside its built library).
 *   TRSM: side 'L': op(A) X = alpha B;  'R': X op(A) = alpha B;  X overwrites B
 *   TRMM: side 'L': B = alpha op(A) B;  'R': B = alpha B op(A)
 * A is m x m ('L') or n x n ('R'), triangle uplo 'U'/'L', diag 'U' (unit) or
 * 'N'; op(A) = A for transa 'N', A^T for 'T'/'C'.  alpha == 0 sets B to zero.
 * form 0: off-diagonal updates with the plain GEMM; form 1: with the split
 * forms (Ozaki slices for FP64, 6xBF16 for FP32; library-owned workspace);
 * form 2: the CRT form for FP64 (as gb300_dgemm_ozaki2; 6xBF16 for FP32).  The
 * diagonal 64x64 blocks are solved / multiplied by a small CUDA kernel.
 * Device pointers, stream-ordered; GB300_ERR_ARG for invalid characters,
 * sizes or leading dimensions.
 * ---------------------------------------------------------------------- */
int gb300_dtrsm(char side, char uplo, char transa, char diag, int m, int n, double alpha,
                const double *A, int lda, double *B, int ldb, int form, void *stream);
int gb300_strsm(char side, char uplo, char transa, char diag, int m, int n, float alpha,
                const float *A, int lda, float *B, int ldb, int form, void *stream);
int gb300_dtrmm(char side, char uplo, char transa, char diag, int m, int n, double alpha,
                const double *A, int lda, double *B, int ldb, int form, void *stream);
int gb300_strmm(char side, char uplo, char transa, char diag, int m, int n, float alpha,
                const float *A, int lda, float *B, int ldb, int form, void *stream);

/* ------------------------------------------------------------------------
 * Complex GEMM: C = alpha*op(A)*op(B) + beta*C on interleaved (re, im)
 * storage, column-major, leading dimensions in complex elements.  alpha and
 * beta point to (re, im) pairs in host memory.  trans: 'N' op(X) = X, 'R'
 * conj(X), 'T' X^T, 'C' conj(X)^T; any other character is a transpose (as in
 * the real path).  The reference has complex GEMM only as OpenBLAS-style
 * packed-panel kernels outside its built library; their four conjugation
 * variants (OpenBLAS-like_implementation/zgemm_kernel_4x2_haswell.c:6-21,
 * cgemm_kernel_8x2_haswell.c:6-21: C += alpha * conj_a(A) * conj_b(B)) are the
 * 'N'/'R' combinations here, and their 3M kernels
 * (zgemm3m_kernel_4x4_haswell.c, cgemm3m_kernel_8x4_haswell.c) the 3M method.
 *   method GB300_CPLX_4M    one real GEMM on the embedded 2m x n x 2k problem,
 *                           plain FP64 (DMMA) / FP32 (FFMA) kernels;
 *   method GB300_CPLX_3M    three real GEMMs (25% fewer flops, the imaginary
 *                           part's error scales with |Re A + Im A| |Re B + Im B|);
 *   method GB300_CPLX_SPLIT the embedded problem on the tensor-core split forms:
 *                           6xBF16/3xBF16 for CGEMM (param = products, 0 =
 *                           tuned), Ozaki for ZGEMM (param = slices, 0 = tuned);
 *   method GB300_CPLX_CRT   ZGEMM only: the embedded problem on the CRT form
 *                           of gb300_dgemm_ozaki2 (param = moduli, 0 = tuned).
 * Same semantics as the real path otherwise: beta*C first (beta == 0 still
 * multiplies), alpha == 0 or k == 0 reads neither A nor B.  A complex alpha is
 * folded into op(A) (one rounding per element), a complex beta scales C first.
 * workspace NULL: a library-owned buffer per stream; otherwise at least
 * gb300_complex_workspace_bytes(...) bytes of device memory.
 * ---------------------------------------------------------------------- */
enum { GB300_CPLX_4M = 0, GB300_CPLX_3M = 1, GB300_CPLX_SPLIT = 2, GB300_CPLX_CRT = 3 };
size_t gb300_complex_workspace_bytes(int is_double, int method, char transb, int m, int n,
                                     int k, int param);
int gb300_cgemm(char transa, char transb, int m, int n, int k, const float *alpha,
                const float *A, int lda, const float *B, int ldb, const float *beta, float *C,
                int ldc, int method, int param, void *workspace, size_t workspace_bytes,
                void *stream);
int gb300_zgemm(char transa, char transb, int m, int n, int k, const double *alpha,
                const double *A, int lda, const double *B, int ldb, const double *beta,
                double *C, int ldc, int method, int param, void *workspace,
                size_t workspace_bytes, void *stream);
/* Host-pointer forms (synchronous, like the drop-in symbols): the split method
 * runs directly on host memory where the device can read it (coherent CPU-GPU
 * systems), everything else stages through HBM. */
int gb300_host_cgemm(char transa, char transb, int m, int n, int k, const float *alpha,
                     const float *a, int lda, const float *b, int ldb, const float *beta,
                     float *c, int ldc, int method, int param);
int gb300_host_zgemm(char transa, char transb, int m, int n, int k, const double *alpha,
                     const double *a, int lda, const double *b, int ldb, const double *beta,
                     double *c, int ldc, int method, int param);

/* FP64 GEMM by the CRT (modular-integer) form on the BF16 tensor pipe, after
 * Ozaki scheme II: rows of op(A) and columns of op(B) are scaled by powers of
 * two to integers of b bits, their product is computed exactly as residues
 * modulo `moduli` pairwise coprime odd moduli <= 255 (one tensor-core GEMM per
 * modulus) and rebuilt by the Chinese remainder theorem in 192-bit integer
 * arithmetic, then rounded once to FP64.  b is the largest integer with
 * 2 k (2^b - 1)^2 < M (M the product of the moduli): 16 moduli give 56 bits at
 * k = 4096, the accuracy of 8 slices for 16 instead of 36 GEMMs.  moduli 0 =
 * 16, else 2..24; GB300_ERR_ARG when k is too large for any b at that count.
 * workspace NULL: a library-owned buffer per stream; otherwise at least
 * gb300_split_workspace_bytes(2, m, n, k, moduli) bytes. */
int gb300_dgemm_ozaki2(char transa, char transb, int m, int n, int k, double alpha,
                       const double *A, int lda, const double *B, int ldb, double beta, double *C,
                       int ldc, int moduli, void *workspace, size_t workspace_bytes,
                       void *stream);
int gb300_host_dgemm_ozaki2(char transa, char transb, int m, int n, int k, double alpha,
                            const double *a, int lda, const double *b, int ldb, double beta,
                            double *c, int ldc, int moduli);
/* Two phases of gb300_dgemm_ozaki2 on a caller workspace: prepare writes the
 * scale exponents and the residue operands of op(A) and op(B); run performs
 * the per-modulus GEMMs, the reconstruction and C = alpha*AB + beta*C (same m,
 * n, k, moduli; run may repeat with other alpha, beta, C). */
int gb300_dgemm_ozaki2_prepare(char transa, char transb, int m, int n, int k, const double *A,
                               int lda, const double *B, int ldb, int moduli, void *workspace,
                               size_t workspace_bytes, void *stream);
int gb300_dgemm_ozaki2_run(int m, int n, int k, double alpha, double beta, double *C, int ldc,
                           int moduli, const void *workspace, size_t workspace_bytes,
                           void *stream);

/* Workspace needed by the split forms for one call of the given shape.
 * kind = 0: sgemm_bf16x with `param` = products; kind = 1: dgemm_ozaki with
 * `param` = slices; kind = 2: dgemm_ozaki2 with `param` = moduli. */
size_t gb300_split_workspace_bytes(int kind, int m, int n, int k, int param);

/* After a stream synchronisation: the first error code any kernel of this
 * library recorded on the current device since the last clear (0 = none),
 * including calls of gb300_sgemm_bf16x_noalloc (which keeps its own word;
 * when both are set the library-wide word's code is returned).  Bounded
 * waits that expired record codes 0x10-0x14.  clear != 0 resets both words.
 * Allocates nothing, so callers of the no-allocation entry point can use it. */
unsigned gb300_device_error(int clear);

/* Failure-detection self-test (no reference counterpart; the reference has no
 * error detection at all, src/gemm_driver.c:23-33 spins without a limit):
 * launches one CTA that waits on an mbarrier nothing arrives on, with a poll
 * limit of `poll_limit`.  Expected result: GB300_ERR_TIMEOUT, with the error
 * word set to 0x10 (clear it with gb300_device_error(1)) and the CUDA context
 * still usable.  Faults, traps and hangs are never used to test this. */
int gb300_selftest_wait_timeout(unsigned poll_limit);

/* Autotuner (replaces the reference's compile-time tune headers dgemm_tune.h /
 * sgemm_tune.h, src/gemm_set_parameters.h:1-61).  kind 0 = BF16xP SGEMM
 * (chooses products 3/6 and the hi*hi chunk length), kind 1 = Ozaki DGEMM
 * (chooses the slice count 4..12), kind 2 = CRT DGEMM (gb300_dgemm_ozaki2;
 * chooses the moduli count 11..24), then for these three the output tile
 * width and the cluster mode; kind 3 / 4 = the plain DGEMM / SGEMM kernels
 * (gb300_dgemm / gb300_sgemm and the drop-ins: chooses the split-K factor
 * 1..32 and the ring depth 4 / 6 -- the reference's BDK / LOOP_TIMES_K
 * blocking, dgemm_tune.h:6-10, sgemm_tune.h:7-11).  gb300_autotune runs the
 * candidates on the given device operands (FP32 for kinds 0 and 4, FP64 for
 * kinds 1, 2, 3).  For kinds 0-2 it keeps the fastest whose max and Frobenius
 * relative errors against a near-exact FP64 reference (the Ozaki form with 12
 * slices) do not exceed the plain kernel's; for kinds 3, 4 the fastest (every
 * split sums the same products in K order).  The result is cached for the
 * shape class (floor(log2) of m, n, k) and used whenever a split entry point
 * gets products = 0 / slices = 0 / moduli = 0, and by every plain call of the
 * class.  It allocates temporary device memory and synchronises `stream`.
 * gb300_tune_lookup: the parameters products/slices = 0 resolve to for a
 * shape (GB300_OK if a tuned entry exists, GB300_ERR_UNSUPPORTED if the
 * defaults apply: 6 products, chunk 4, 8 slices, 16 moduli).
 * Cache file: gb300_tune_cache_save/_load (path NULL: $GB300_TUNE_CACHE, else
 * $HOME/.gemm_gb300_tune.json); loading skips malformed or out-of-range
 * entries and returns GB300_ERR_ARG for an unreadable file, keeping the cache. */
int gb300_autotune(int kind, char transa, char transb, int m, int n, int k, const void *A,
                   int lda, const void *B, int ldb, void *stream, int *chosen);
int gb300_tune_lookup(int kind, int m, int n, int k, int *param, int *chunk);
/* The output tile width (128 / 256) and the cluster mode (1 = pair MMAs on
 * 2-CTA clusters, 2 = one CTA per tile) the split GEMMs use for this shape
 * (knob, tuned entry or default, in that order; a problem with a single
 * 128-row tile always runs one CTA per tile); GB300_ERR_UNSUPPORTED when the
 * shape class has no tuned entry. */
int gb300_tune_layout(int kind, int m, int n, int k, int *tile_n, int *pair_mma);
/* The split-K factor and ring depth the plain kernels use for this shape
 * (knob, tuned entry of the shape class, else by shape / 4 stages; without
 * room for the slices -- no cached workspace -- a call runs unsplit);
 * GB300_ERR_UNSUPPORTED when the shape class has no tuned entry. */
int gb300_plain_layout(int is_double, int m, int n, int k, int *split_k, int *stages);
int gb300_tune_cache_save(const char *path);
int gb300_tune_cache_load(const char *path, int *loaded);
void gb300_tune_cache_clear(void);

/* Process-wide tuning knobs (the role of the reference's compile-time tune
 * headers, dgemm_tune.h / sgemm_tune.h via src/gemm_set_parameters.h:1-61).
 *   GB300_TUNE_BF16X_CHUNK: K extent (in 64-wide blocks) of one TMEM
 *   accumulation chunk of the BF16xP SGEMM's hi*hi product; products of
 *   order 1 use 4x that (32x with the scaled FP16 terms), order-2 products
 *   are not chunked.  0 restores the default (4).
 *   GB300_TUNE_GRAPH_BRANCHES: parallel branches (1..64) of the CUDA graph
 *   that gb300_grouped_graph_create captures for the split form (form 1);
 *   read at creation.  0 restores the default.
 *   GB300_TUNE_TILE_N: output tile width (128 or 256) of the tensor-core
 *   GEMMs of all split forms; 0 restores the choice by shape (the tuned
 *   width of the shape class, else 128 for outputs at most 128 columns wide
 *   and 256 otherwise).
 *   GB300_TUNE_PAIR_MMA: how the tensor-core GEMMs of all split forms run
 *   problems with two or more 128-row tiles: 1 = pair MMAs (tcgen05
 *   cta_group::2: two CTAs of a cluster compute a 256-row tile, each loading
 *   its A rows and half of the B tile into its own shared memory), 2 = one
 *   CTA per tile, loading its whole A and B tiles; 0 restores the default
 *   (the tuned mode of the shape class, else pair MMAs).  Both give the same
 *   results bit for bit.
 *   GB300_TUNE_HOST_PARTS: operand parts (1..8) of the pipelined host-pointer
 *   path of the FP32 split form and the FP64 CRT form (gb300_host_sgemm_bf16x,
 *   gb300_host_dgemm_ozaki2, the drop-ins with GB300_DROPIN_FORM=split):
 *   op(A) in that many row parts and op(B) in that
 *   many column parts, copied to HBM on a copy stream while the compute
 *   stream prepares the parts that have arrived and multiplies the C blocks
 *   whose parts are ready, and C blocks go back as they finish.  1 turns
 *   the pipeline off; 0 restores the choice by shape (page-locked buffers: 4
 *   parts per dimension of 4096 or more, 2 from 2048 for the FP64 CRT form,
 *   when k >= 1024; pageable: off).  The
 *   results are the same bit for bit.
 *   GB300_TUNE_MODULUS_SPLIT: work units of the CRT form's GEMM
 *   (gb300_dgemm_ozaki2): 1 = whole output tiles, each CTA running all
 *   moduli of its tile; 2 = one modulus of one tile (the moduli are
 *   independent GEMMs, so small outputs still fill the GPU); 0 restores the
 *   choice by shape (2 when the tiles alone fill fewer than four waves).
 *   Same results bit for bit.
 *   GB300_TUNE_SPLIT_K: K slices of the plain kernels (gb300_dgemm,
 *   gb300_sgemm, the drop-ins; the role of the reference's K blocking,
 *   src/gemm_driver.c:156-190): 1 = none, S = 2..65535 (at most one slice per
 *   k-tile); each slice's sums go to library-owned scratch and a second
 *   kernel adds them to beta*C in K order.  0 restores the choice by shape
 *   (tuned, else the factor 1..32 that a model of waves of 128 x 128 tiles
 *   and ring fill finds fastest, at least 8 k-tiles a slice).  Results
 *   differ from the unsplit call only in the grouping of the K sum.
 *   GB300_TUNE_PLAIN_STAGES: ring depth of the plain kernels, 4 or 6; 0
 *   restores the default (tuned, else 4). */
enum {
  GB300_TUNE_BF16X_CHUNK = 1,
  GB300_TUNE_GRAPH_BRANCHES = 2,
  GB300_TUNE_TILE_N = 3,
  GB300_TUNE_PAIR_MMA = 4,
  GB300_TUNE_HOST_PARTS = 5,
  GB300_TUNE_MODULUS_SPLIT = 6,
  GB300_TUNE_SPLIT_K = 7,
  GB300_TUNE_PLAIN_STAGES = 8
};
int gb300_tune_param(int param, int value);

/* Library version string. */
const char *gb300_version(void);

#ifdef __cplusplus
}
#endif
#endif /* GEMM_GB300_H */
