// trsm.cu -- triangular solve (TRSM) and triangular multiply (TRMM)
// built on this library's GEMM, the BLAS-3 routines that spend most of their
// time in GEMM updates.  The reference ships TRSM/TRMM only as OpenBLAS-style
// packed-panel kernels (OpenBLAS-like_implementation/TRSM_KERNEL_*_simplified.c,
// trmm_kernel_4x8_simplified.c), outside its built library; this file gives them
// the BLAS interface and semantics:
//
//   TRSM: side 'L': op(A) X = alpha B,  side 'R': X op(A) = alpha B   (X -> B)
//   TRMM: side 'L': B = alpha op(A) B,  side 'R': B = alpha B op(A)
//
// A is triangular (uplo 'U'/'L', diag 'U' unit / 'N'), op(A) = A or A^T.  Both
// halve the "effective" triangle of op(A) (lower when uplo == 'L' xor op
// transposes) recursively: one half, one GEMM for the off-diagonal block
// between the halves, the other half; a range of at most 64 is one small
// kernel (the 64 x 64 block in shared memory, each right-hand side on a few
// lanes of a warp).  The GEMMs are the plain kernel (form 0), the tensor-core
// split form (form 1: Ozaki slices for FP64, 6xBF16 for FP32) or the CRT form
// (form 2, FP64; FP32 as form 1).
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"
#include "plain_gemm.h"
#include "split_gemm.h"

namespace gb300 {

constexpr int kTrNb = 64;     // diagonal block size
// right-hand sides per CTA of the diagonal kernels (tr_lanes<T>() lanes each)
constexpr int kTrCols = 32;

// op(A)(r, c) of the diagonal block starting at (d0, d0).
template <typename T>
__device__ __forceinline__ T opA_at(const T *A, int lda, bool trans, int d0, int r, int c) {
  return trans ? A[(int64_t)(d0 + r) * lda + d0 + c] : A[(int64_t)(d0 + c) * lda + d0 + r];
}

// The nb x nb diagonal block of op(A) at (d0, d0) into shared memory as
// Ms[c][r] = M(r, c), column by column: M = op(A)'s block for the left side,
// its transpose for the right side (X op(A) = B is op(A)^T X^T = B^T).  Only
// the effective triangle is read; the unit diagonal is written as 1 and
// everything else, up to 64 x 64, as 0.  Then Inv[c] = 1 / M(c, c) (0 past nb):
// the solves multiply by it, one division per entry of the block instead of
// one per step and lane (the FP64 divisions had held much of the FP64 pipe).
template <typename T>
__device__ void load_block(const T *A, int lda, bool trans, bool lower, bool unit, bool right,
                           int d0, int nb, T *Ms, T *Inv) {
  for (int e = threadIdx.x; e < kTrNb * kTrNb; e += blockDim.x) {
    const int c = e / kTrNb, r = e % kTrNb;     // M(r, c)
    const int ar = right ? c : r, ac = right ? r : c;  // the entry of op(A)'s block
    T v = T(0);
    if (r < nb && c < nb) {
      const bool in = lower ? (ac <= ar) : (ac >= ar);
      if (ar == ac && unit) v = T(1);
      else if (in) v = opA_at(A, lda, trans, d0, ar, ac);
    }
    Ms[e] = v;
  }
  __syncthreads();
  for (int c = threadIdx.x; c < kTrNb; c += blockDim.x)
    Inv[c] = c < nb ? T(1) / Ms[c * kTrNb + c] : T(0);
}

// x <- M^-1 x (solve) or M x (multiply) for one right-hand side spread over
// kLanes lanes of a warp: lane part p holds x[kRows p ..] in registers, M
// triangular (LOWER: below the diagonal) in Ms[c][r].  A solve takes the
// columns in order: a shuffle hands x_c to the group, which multiplies it by
// 1 / M(c, c) (the lane holding x_c keeps it), and each lane updates its rows
// still to solve (x_r -= M(r, c) x_c); a multiply sums M(r, c) x_c over the
// shuffled x_c into separate accumulators.  Rows and columns from nb on are
// zero in Ms and x and stay so.  (One thread per right-hand side, 2016
// multiply-adds in a chain through shared memory, took 42.5 us a block for
// 8192 FP32 columns.  Lanes per right-hand side, STRSM / DTRSM 8192^2: 4 ->
// 64.9 / 18.0 TFLOP/s, 8 -> 74.3 / 17.9, 16 -> 82.4 / 17.4; the FP64 block
// solves are FP64-pipe-bound.)
template <typename T>
__host__ __device__ constexpr int tr_lanes() { return sizeof(T) == 4 ? 16 : 8; }
template <typename T, bool LOWER, bool SOLVE, int kLanes = tr_lanes<T>(),
          int kRows = kTrNb / tr_lanes<T>()>
__device__ __forceinline__ void tri_apply(T (&x)[kRows], const T *Ms, const T *Inv, int nb,
                                          bool unit, int part) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  auto m_at = [&](int r, int c) { return Ms[c * kTrNb + r]; };
  if constexpr (SOLVE) {
#pragma unroll
    for (int q = 0; q < kTrNb; ++q) {
      const int c = LOWER ? q : kTrNb - 1 - q;
      const int owner = c / kRows, ic = c % kRows;
      // every lane of the group scales the shuffled x_c (nothing divergent
      // before the next shuffle); its owner keeps the result
      T xc = __shfl_sync(full, x[ic], (lane & ~(kLanes - 1)) | owner);
      if (!unit) xc *= Inv[c];
      x[ic] = part == owner ? xc : x[ic];
#pragma unroll
      for (int j = 0; j < kRows; ++j) {
        const int r = part * kRows + j;
        if (LOWER ? (r > c) : (r < c)) x[j] -= m_at(r, c) * xc;
      }
    }
  } else {
    T acc[kRows];
#pragma unroll
    for (int j = 0; j < kRows; ++j) acc[j] = T(0);
#pragma unroll
    for (int c = 0; c < kTrNb; ++c) {
      const int owner = c / kRows, ic = c % kRows;
      const T xc = __shfl_sync(full, x[ic], (lane & ~(kLanes - 1)) | owner);
#pragma unroll
      for (int j = 0; j < kRows; ++j) {
        const int r = part * kRows + j;
        if (LOWER ? (c <= r) : (c >= r)) acc[j] += m_at(r, c) * xc;
      }
    }
#pragma unroll
    for (int j = 0; j < kRows; ++j) x[j] = acc[j];
  }
}

// Left side: rows [d0, d0+nb) of B, tr_lanes<T>() lanes per column (kTrCols
// columns a CTA): SOLVE: X = op(A)_blk^-1 B_blk;  else X = op(A)_blk B_blk.
// LOWER: op(A)'s effective triangle.
template <typename T, bool LOWER, bool SOLVE>
__global__ void __launch_bounds__(kTrCols * tr_lanes<T>()) diag_left_kernel(
    const T *__restrict__ A, int lda, int trans, int unit, int d0, int nb, T *B, int ldb, int n) {
  constexpr int kLanes = tr_lanes<T>(), kRows = kTrNb / kLanes;
  extern __shared__ uint8_t sm[];
  T *Ms = reinterpret_cast<T *>(sm);  // [kTrNb][kTrNb], column-major
  T *Inv = Ms + kTrNb * kTrNb;        // [kTrNb]
  load_block<T>(A, lda, trans != 0, LOWER, unit != 0, false, d0, nb, Ms, Inv);
  __syncthreads();
  const int j = blockIdx.x * kTrCols + (int)threadIdx.x / kLanes;
  const int part = (int)threadIdx.x % kLanes;
  const bool live = j < n;  // a dead column's lanes still take part in the shuffles
  T *col = B + (int64_t)(live ? j : 0) * ldb + d0 + part * kRows;
  T x[kRows];
#pragma unroll
  for (int i = 0; i < kRows; ++i) x[i] = (live && part * kRows + i < nb) ? col[i] : T(0);
  tri_apply<T, LOWER, SOLVE>(x, Ms, Inv, nb, unit != 0, part);
#pragma unroll
  for (int i = 0; i < kRows; ++i)
    if (live && part * kRows + i < nb) col[i] = x[i];
}

// Right side: columns [d0, d0+nb) of B, tr_lanes<T>() lanes per row:
//   SOLVE: X = B_blk op(A)_blk^-1;  else X = B_blk op(A)_blk
// (the row vector times the block is the block's transpose times the column)
template <typename T, bool LOWER, bool SOLVE>
__global__ void __launch_bounds__(kTrCols * tr_lanes<T>()) diag_right_kernel(
    const T *__restrict__ A, int lda, int trans, int unit, int d0, int nb, T *B, int ldb, int m) {
  constexpr int kLanes = tr_lanes<T>(), kRows = kTrNb / kLanes;
  extern __shared__ uint8_t sm[];
  T *Ms = reinterpret_cast<T *>(sm);
  T *Inv = Ms + kTrNb * kTrNb;
  load_block<T>(A, lda, trans != 0, LOWER, unit != 0, true, d0, nb, Ms, Inv);
  __syncthreads();
  const int i = blockIdx.x * kTrCols + (int)threadIdx.x / kLanes;
  const int part = (int)threadIdx.x % kLanes;
  const bool live = i < m;
  T *row = B + (int64_t)(d0 + part * kRows) * ldb + (live ? i : 0);
  T x[kRows];
#pragma unroll
  for (int c = 0; c < kRows; ++c)
    x[c] = (live && part * kRows + c < nb) ? row[(int64_t)c * ldb] : T(0);
  tri_apply<T, !LOWER, SOLVE>(x, Ms, Inv, nb, unit != 0, part);  // op(A)^T: the other triangle
#pragma unroll
  for (int c = 0; c < kRows; ++c)
    if (live && part * kRows + c < nb) row[(int64_t)c * ldb] = x[c];
}

// B(m x n window) *= s, or = 0 exactly when s == 0 (BLAS: alpha = 0 sets B to zero).
template <typename T>
__global__ void scale_b_kernel(int m, int n, T s, T *B, int ldb) {
  const int64_t total = (int64_t)m * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    T *p = B + (e / m) * (int64_t)ldb + (e % m);
    *p = (s == T(0)) ? T(0) : *p * s;
  }
}

// ---------------------------------------------------------------- host driver
static int in_set(char c, const char *set) {
  for (; *set; ++set)
    if (c == *set) return 1;
  return 0;
}

// Off-diagonal update: C(mm x nn) -= op1(X) op2(Y) (solve) or += (multiply)
// through the library's GEMM.
template <typename T>
static int tr_gemm(int form, char t1, char t2, int mm, int nn, int kk, const T *X, int ldx,
                   const T *Y, int ldy, T *C, int ldc, void *ws, size_t ws_bytes, cudaStream_t st,
                   unsigned *err, bool add = false) {
  if (mm <= 0 || nn <= 0 || kk <= 0) return GB300_OK;
  const T a = add ? T(1) : T(-1);
  if constexpr (sizeof(T) == 8) {
    if (form == 1)
      return ozaki_dgemm(t1, t2, mm, nn, kk, a, X, ldx, Y, ldy, 1.0, C, ldc, 0, ws, ws_bytes, st,
                         err);
    if (form == 2)  // the CRT form, its moduli by shape class (16 untuned)
      return crt_dgemm(t1, t2, mm, nn, kk, a, X, ldx, Y, ldy, 1.0, C, ldc, 0, ws, ws_bytes, st,
                       err);
    return plain_dgemm(t1, t2, mm, nn, kk, a, X, ldx, Y, ldy, 1.0, C, ldc, st, err);
  } else {
    if (form == 1 || form == 2)
      return split_sgemm(t1, t2, mm, nn, kk, a, X, ldx, Y, ldy, 1.0f, C, ldc, 6, ws, ws_bytes, st,
                         err);
    return plain_sgemm(t1, t2, mm, nn, kk, a, X, ldx, Y, ldy, 1.0f, C, ldc, st, err);
  }
}

size_t tr_workspace_bytes(int is_double, int form, int m, int n) {
  if ((form != 1 && form != 2) || m <= 0 || n <= 0) return 0;
  // The off-diagonal updates are at most (m x n x half) for TRSM (half: the
  // first half of the triangle, a multiple of 64) and (64 x n x m) / (m x 64 x
  // n) for TRMM (left / right): size for the largest.
  const int na = m > n ? m : n;
  const int half = ((na + 1) / 2 + kTrNb - 1) / kTrNb * kTrNb;
  const int shapes[4][3] = {{m, n, half}, {kTrNb, n, m}, {m, kTrNb, n}, {m, n, half}};
  size_t need = 0;
  for (const auto &sh : shapes) {
    const size_t w = !is_double  ? split_workspace_bytes(0, sh[0], sh[1], sh[2], 6)
                     : form == 2 ? crt_workspace_bytes(sh[0], sh[1], sh[2], 0)
                                 : split_workspace_bytes(1, sh[0], sh[1], sh[2], 0);
    if (w > need) need = w;
  }
  return need;
}

int tr_check(char side, char uplo, char transa, char diag, int m, int n, int lda, int ldb) {
  if (!in_set(side, "LlRr") || !in_set(uplo, "UuLl") || !in_set(transa, "NnTtCc") ||
      !in_set(diag, "UuNn"))
    return GB300_ERR_ARG;
  const int na = (side == 'L' || side == 'l') ? m : n;
  if (m < 0 || n < 0 || lda < (na > 1 ? na : 1) || ldb < (m > 1 ? m : 1)) return GB300_ERR_ARG;
  return (m == 0 || n == 0) ? -1 : GB300_OK;
}

// solve = 1: TRSM, 0: TRMM.
template <typename T>
int tr_driver(int solve, char side, char uplo, char transa, char diag, int m, int n, T alpha,
              const T *A, int lda, T *B, int ldb, int form, void *ws, size_t ws_bytes,
              cudaStream_t st, unsigned *err) {
  const int ck = tr_check(side, uplo, transa, diag, m, n, lda, ldb);
  if (ck != GB300_OK) return ck < 0 ? GB300_OK : ck;
  if (form < 0 || form > 2) return GB300_ERR_ARG;
  if (form != 0 && (!ws || ws_bytes < tr_workspace_bytes(sizeof(T) == 8, form, m, n)))
    return GB300_ERR_WORKSPACE;
  const bool left = side == 'L' || side == 'l';
  const bool trans = !(transa == 'N' || transa == 'n');
  const bool lower = (uplo == 'L' || uplo == 'l') != trans;  // effective triangle of op(A)
  const bool unit = diag == 'U' || diag == 'u';
  const char tA = trans ? 'T' : 'N';
  auto scale = [&](T s) {
    const int64_t total = (int64_t)m * n;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    scale_b_kernel<T><<<blocks, 256, 0, st>>>(m, n, s, B, ldb);
  };
  if (alpha == T(0)) {
    scale(T(0));
    return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
  }
  // op(A)(r0.., c0..) as a GEMM operand: pointer and transpose flag
  auto opA = [&](int r0, int c0) -> const T * {
    return trans ? A + (int64_t)r0 * lda + c0 : A + (int64_t)c0 * lda + r0;
  };
  const int smem = (kTrNb * kTrNb + kTrNb) * (int)sizeof(T);  // the block and 1 / diagonal
  // the diagonal block [d0, d0 + nb): solve (1) or multiply (0) in place
  auto diag_block = [&](int d0, int nb, bool sv) {
    const int rhs = left ? n : m;
    const dim3 grid((rhs + kTrCols - 1) / kTrCols);
    const int tr = trans ? 1 : 0, un = unit ? 1 : 0;
    if (left) {
      if (lower)
        (sv ? diag_left_kernel<T, true, true> : diag_left_kernel<T, true, false>)
            <<<grid, kTrCols * tr_lanes<T>(), smem, st>>>(A, lda, tr, un, d0, nb, B, ldb, n);
      else
        (sv ? diag_left_kernel<T, false, true> : diag_left_kernel<T, false, false>)
            <<<grid, kTrCols * tr_lanes<T>(), smem, st>>>(A, lda, tr, un, d0, nb, B, ldb, n);
    } else {
      if (lower)
        (sv ? diag_right_kernel<T, true, true> : diag_right_kernel<T, true, false>)
            <<<grid, kTrCols * tr_lanes<T>(), smem, st>>>(A, lda, tr, un, d0, nb, B, ldb, m);
      else
        (sv ? diag_right_kernel<T, false, true> : diag_right_kernel<T, false, false>)
            <<<grid, kTrCols * tr_lanes<T>(), smem, st>>>(A, lda, tr, un, d0, nb, B, ldb, m);
    }
  };
  const int na = left ? m : n;
  // TRSM scales first (X = op(A)^-1 (alpha B)); TRMM scales last.
  if (solve && alpha != T(1)) scale(alpha);
  // Block order: a solve walks the triangle from its first row (lower-left /
  // upper-right as seen by the side); a multiply in place walks the other way
  // so that every block still reads unmodified rows / columns of B.
  const bool forward = left ? (solve ? lower : !lower) : (solve ? !lower : lower);
  int rc = GB300_OK;
  // The rows (left) / columns (right) [r0, r1) of B take the contribution of
  // [c0, c1): B(r, :) -= op(A)(r, c) B(c, :), or B(:, r) -= B(:, c) op(A)(c, r)
  // (TRSM: the solved block updates the ones still to solve); += for TRMM
  auto block_update = [&](int r0, int r1, int c0, int c1, bool add) -> int {
    if (r1 <= r0 || c1 <= c0) return GB300_OK;
    if (left)
      return tr_gemm<T>(form, tA, 'N', r1 - r0, n, c1 - c0, opA(r0, c0), lda, B + c0, ldb, B + r0,
                        ldb, ws, ws_bytes, st, err, add);
    return tr_gemm<T>(form, 'N', tA, m, r1 - r0, c1 - c0, B + (int64_t)c0 * ldb, ldb, opA(c0, r0),
                      lda, B + (int64_t)r0 * ldb, ldb, ws, ws_bytes, st, err, add);
  };
  // TRSM by recursive halving of the triangle: solve the first half, update
  // the second half with it (one GEMM with k = the half), solve the second
  // half; ranges of at most 64 go to the diagonal kernel.  The halves split at
  // multiples of 64, so the diagonal blocks are those of a 64-blocked walk.
  // Against a rank-64 update per diagonal block, the updates' C traffic (and
  // the CRT form's reconstructions) fall from m^2 n / 128 elements to about
  // n m log2(m / 64) / 2, and most of the flops run at long K.
  auto solve_range = [&](auto &self, int D0, int D1) -> int {
    if (D1 - D0 <= kTrNb) {
      diag_block(D0, D1 - D0, true);
      return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
    }
    const int Dm = D0 + ((D1 - D0) / 2 + kTrNb - 1) / kTrNb * kTrNb;  // D0 < Dm < D1
    // forward: the rows / columns still to solve follow the solved ones
    int r = self(self, forward ? D0 : Dm, forward ? Dm : D1);
    if (r == GB300_OK)
      r = forward ? block_update(Dm, D1, D0, Dm, false) : block_update(D0, Dm, Dm, D1, false);
    if (r == GB300_OK) r = self(self, forward ? Dm : D0, forward ? D1 : Dm);
    return r;
  };
  if (solve) rc = solve_range(solve_range, 0, na);
  // TRMM in place by the same halving: the half whose new value needs the
  // other half's old one goes first (forward: the first half, as for the
  // upper triangle on the left), then it takes that half's contribution, then
  // the other half; ranges of at most 64 go to the diagonal kernel.  (Per
  // 64-wide block the updates were 64 rows tall: few tiles for the GEMMs.)
  auto mul_range = [&](auto &self, int D0, int D1) -> int {
    if (D1 - D0 <= kTrNb) {
      diag_block(D0, D1 - D0, false);
      return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
    }
    const int Dm = D0 + ((D1 - D0) / 2 + kTrNb - 1) / kTrNb * kTrNb;  // D0 < Dm < D1
    int r = self(self, forward ? D0 : Dm, forward ? Dm : D1);
    if (r == GB300_OK)
      r = forward ? block_update(D0, Dm, Dm, D1, true) : block_update(Dm, D1, D0, Dm, true);
    if (r == GB300_OK) r = self(self, forward ? Dm : D0, forward ? D1 : Dm);
    return r;
  };
  if (!solve) rc = mul_range(mul_range, 0, na);
  if (rc == GB300_OK && !solve && alpha != T(1)) scale(alpha);
  if (rc == GB300_OK && cudaGetLastError() != cudaSuccess) rc = GB300_ERR_CUDA;
  return rc;
}

int trsm_d(int solve, char side, char uplo, char ta, char diag, int m, int n, double alpha,
           const double *A, int lda, double *B, int ldb, int form, void *ws, size_t wsb,
           cudaStream_t st, unsigned *err) {
  return tr_driver<double>(solve, side, uplo, ta, diag, m, n, alpha, A, lda, B, ldb, form, ws,
                           wsb, st, err);
}
int trsm_s(int solve, char side, char uplo, char ta, char diag, int m, int n, float alpha,
           const float *A, int lda, float *B, int ldb, int form, void *ws, size_t wsb,
           cudaStream_t st, unsigned *err) {
  return tr_driver<float>(solve, side, uplo, ta, diag, m, n, alpha, A, lda, B, ldb, form, ws, wsb,
                          st, err);
}

}  // namespace gb300
