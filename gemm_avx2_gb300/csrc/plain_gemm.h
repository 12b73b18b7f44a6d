// plain_gemm.h -- internal host-side declarations shared by the library's
// translation units (not part of the public ABI; see include/gemm_gb300.h).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <vector>

#include "../../include/gemm_gb300.h"

namespace gb300 {

// 'N'/'n' = no transpose; any other character = transpose (src/gemm_driver.c:17-18).
inline bool notrans(char t) { return t == 'N' || t == 'n'; }

// Argument checks of every entry point (host only, no CUDA call):
// GB300_ERR_ARG for negative sizes or leading dimensions below the stored rows
// (at least 1); -1 for a valid call with nothing to compute (m or n == 0);
// GB300_OK otherwise.
inline int check_args(char ta, char tb, int m, int n, int k, int lda, int ldb, int ldc) {
  const int arows = notrans(ta) ? m : k, brows = notrans(tb) ? k : n;
  if (m < 0 || n < 0 || k < 0 || lda < (arows > 1 ? arows : 1) ||
      ldb < (brows > 1 ? brows : 1) || ldc < (m > 1 ? m : 1))
    return GB300_ERR_ARG;
  return (m == 0 || n == 0) ? -1 : GB300_OK;
}

// TMA requires a 16-byte aligned base and a leading dimension whose byte
// stride is a multiple of 16.
inline bool tma_ok(const void *p, int ld, size_t elem) {
  return (reinterpret_cast<uintptr_t>(p) % 16 == 0) && ((size_t)ld * elem) % 16 == 0;
}

// 3-D map of d0 x d1 x d2 elements (d0 contiguous; strides ld1 and ld2 of
// dimensions 1 and 2, in elements), box box0 x box1 x box2, 128-byte swizzle;
// reads past an extent return zeros.
bool encode_3d(CUtensorMap *map, const void *base, size_t elem_bytes, int64_t d0, int64_t d1,
               int64_t d2, int64_t ld1, int64_t ld2, int box0, int box1, int box2);
// Encode a 2-D tiled tensor map over a column-major matrix of rows x cols
// (rows contiguous, leading dimension ld elements).  box = (box_rows, box_cols).
// elem_bytes 2 -> BF16, 4 -> FP32, 8 -> FP64.  Returns false if the driver
// rejects it (the caller then falls back to non-TMA loads).
bool encode_2d(CUtensorMap *map, const void *base, size_t elem_bytes, int64_t rows, int64_t cols,
               int64_t ld, int box_rows, int box_cols, bool swizzle128);

// dst (dpitch bytes between columns) = src (spitch) over `cols` columns of
// `width` bytes each, by SM loads and stores.  Either side may be host memory
// the device can dereference: on a coherent CPU-GPU link that includes
// pageable memory, which the SMs read at the link's rate (measured about
// 200 GB/s host to device, as the copy engines on pinned memory) without the
// driver's staging.
int copy_2d(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, int cols,
            cudaStream_t st);

// ws / ws_bytes: room for the split-K slices (plain_workspace_bytes); without
// it (or too little) the call runs as one K slice.
int plain_dgemm(char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
                const double *B, int ldb, double beta, double *C, int ldc, cudaStream_t st,
                unsigned *err, void *ws = nullptr, size_t ws_bytes = 0);
int plain_sgemm(char ta, char tb, int m, int n, int k, float alpha, const float *A, int lda,
                const float *B, int ldb, float beta, float *C, int ldc, cudaStream_t st,
                unsigned *err, void *ws = nullptr, size_t ws_bytes = 0);
// Split-K of the plain kernels: the factor a call of this shape uses (knob,
// tuned value of the shape class, else by a model of waves and ring fill) and
// the workspace its slices need (0: none).
// The slices' sums are combined in K order by a second kernel.
int plain_split_k(int is_double, int m, int n, int k);
size_t plain_workspace_bytes(int is_double, int m, int n, int k);
void set_plain_split_k(int v);
void set_plain_stages(int v);
int plain_split_override();
int plain_stages_override();
// Tuned split-K factor and ring depth of the plain kernels for a shape class
// (kind 3: FP64, 4: FP32; 0 = not tuned).
int tune_plain_split(int kind, int m, int n, int k);
int tune_plain_stages(int kind, int m, int n, int k);

// Grouped plain GEMMs (grouped.cu).
size_t grouped_workspace_bytes(int count);
size_t grouped_blob_bytes(int count_used);
int grouped_build(const gb300_gemm_problem *P, int count, void *dev_base,
                  std::vector<uint8_t> &blob, int &count_used, int &total_tiles);
int grouped_launch_blob(void *dev_blob, int count_used, int total_tiles, cudaStream_t st,
                        unsigned *err);
int grouped_plain(const gb300_gemm_problem *P, int count, void *ws, size_t ws_bytes,
                  cudaStream_t st, unsigned *err);

// Blocked TRSM / TRMM (trsm.cu): solve = 1 TRSM, 0 TRMM; form 0 plain GEMM
// updates, 1 split-form updates (workspace of tr_workspace_bytes bytes).
size_t tr_workspace_bytes(int is_double, int form, int m, int n);
int tr_check(char side, char uplo, char transa, char diag, int m, int n, int lda, int ldb);
int trsm_d(int solve, char side, char uplo, char ta, char diag, int m, int n, double alpha,
           const double *A, int lda, double *B, int ldb, int form, void *ws, size_t wsb,
           cudaStream_t st, unsigned *err);
int trsm_s(int solve, char side, char uplo, char ta, char diag, int m, int n, float alpha,
           const float *A, int lda, float *B, int ldb, int form, void *ws, size_t wsb,
           cudaStream_t st, unsigned *err);

// Complex GEMM (cplx.cu): method GB300_CPLX_4M / _3M / _SPLIT, complex
// numbers interleaved, alpha and beta as (re, im) pairs in host memory.
size_t complex_workspace_bytes(int is_double, int method, char tb, int m, int n, int k,
                               int param);
int complex_check(char ta, char tb, int m, int n, int k, int lda, int ldb, int ldc, int method);
int complex_gemm_d(char ta, char tb, int m, int n, int k, const double *alpha, const double *A,
                   int lda, const double *B, int ldb, const double *beta, double *C, int ldc,
                   int method, int param, void *ws, size_t ws_bytes, cudaStream_t st,
                   unsigned *err);
int complex_gemm_s(char ta, char tb, int m, int n, int k, const float *alpha, const float *A,
                   int lda, const float *B, int ldb, const float *beta, float *C, int ldc,
                   int method, int param, void *ws, size_t ws_bytes, cudaStream_t st,
                   unsigned *err);

}  // namespace gb300
