// cplx.cu -- complex GEMM (CGEMM / ZGEMM) on the library's real kernels.
//
// C = alpha * op(A) * op(B) + beta * C.  Complex storage is interleaved
// (re, im), column-major, leading dimensions in complex elements.  Trans codes:
// 'N' op(X) = X, 'R' conj(X), 'T' X^T, 'C' conj(X)^T; any other character is a
// transpose, as in the real path.  'N'/'R' on either side are the four
// conjugation variants of the reference's OpenBLAS-style kernels
// (OpenBLAS-like_implementation/zgemm_kernel_4x2_haswell.c:6-21,
// cgemm_kernel_8x2_haswell.c:6-21), which add alpha * conj_a(A) * conj_b(B) to
// C (zgemm_kernel_4x2_haswell.c:224-243); 'T'/'C' are the transposes BLAS adds.
//
// Methods:
//  4M    one real GEMM on an embedded problem.  op(A) becomes the real 2m x 2k
//        matrix Ahat whose 2x2 block (i, l) is [[ar, -ai], [ai, ar]]: complex
//        column l of op(A) followed by i times it.  op(B) becomes the real
//        2k x n matrix Bhat of its interleaved columns (B itself when tb is
//        'N').  The real 2m x n product, column j holding (re, im) pairs, is C's
//        own storage with ld 2*ldc.  8mnk flops on the plain FP64 (DMMA) or FP32
//        (FFMA) kernel; for FP32 Bhat is stored transposed (n x 2k) so that the
//        FFMA kernel gets B MN-major.
//  3M    three real GEMMs T1 = Ar Br, T2 = Ai Bi, T3 = (Ar + Ai)(Br + Bi), then
//        re = T1 - T2, im = T3 - T1 - T2: 6mnk flops (the reference's 3M
//        kernels, OpenBLAS-like_implementation/zgemm3m_kernel_4x4_haswell.c:
//        209-224 and cgemm3m_kernel_8x4_haswell.c:263-279, add alpha times such
//        real products to complex C).
//  SPLIT the 4M embedding on the tensor-core split forms: BF16xP for CGEMM
//        (param = products), Ozaki slices for ZGEMM (param = slices).
//  CRT   (ZGEMM only) the 4M embedding on the CRT form (param = moduli).
// A complex alpha (nonzero imaginary part) is folded into Ahat, one complex
// rounding per element of op(A); a complex beta scales C first.  Real alpha and
// beta reach the real kernel's epilogue unchanged.
#include <cuda_runtime.h>

#include <cstdint>

#include "plain_gemm.h"
#include "split_gemm.h"

namespace gb300 {

namespace {

inline bool cx_trans(char t) { return !(t == 'N' || t == 'n' || t == 'R' || t == 'r'); }
inline bool cx_conj(char t) { return t == 'C' || t == 'c' || t == 'R' || t == 'r'; }
inline int64_t rup(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

template <typename T>
struct Cx;
template <>
struct Cx<float> {
  using v = float2;
};
template <>
struct Cx<double> {
  using v = double2;
};

constexpr int kPackDense = 0;   // out(r, c) = v, complex, ld in complex elements
constexpr int kPackEmbed = 1;   // out(r, 2c) = v, out(r, 2c + 1) = i v
constexpr int kPackPlanar = 2;  // three real planes: re, im, re + im
constexpr int kPackCols = 3;    // reals: out(r, 2c) = re v, out(r, 2c + 1) = im v

// op(X) is the R x K complex view: (r, c) at X[r + c*ld], or X[c + r*ld] when
// trans; conjugated when conj; times s when scale.  32 x 32 tiles through
// shared memory keep both the read and the write coalesced.
template <typename T, int MODE>
__global__ void __launch_bounds__(256)
    cx_pack_kernel(const T *__restrict__ X, int64_t ld, int R, int K, int trans, int conj,
                   int scale, T sr, T si, T *__restrict__ out, int64_t ldo, int64_t plane) {
  using V = typename Cx<T>::v;
  __shared__ V tile[32][33];  // [c][r]
  const V *Xv = reinterpret_cast<const V *>(X);
  const int c0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int r0 = blockIdx.y * 32; r0 < R; r0 += gridDim.y * 32) {  // grid.y strides over rows
#pragma unroll
    for (int q = ty; q < 32; q += 8) {
      V v;
      v.x = T(0);
      v.y = T(0);
      if (!trans) {
        const int r = r0 + tx, c = c0 + q;
        if (r < R && c < K) v = Xv[r + (int64_t)c * ld];
        tile[q][tx] = v;
      } else {
        const int r = r0 + q, c = c0 + tx;
        if (r < R && c < K) v = Xv[c + (int64_t)r * ld];
        tile[tx][q] = v;
      }
    }
    __syncthreads();
#pragma unroll
    for (int q = ty; q < 32; q += 8) {
      const int r = r0 + tx, c = c0 + q;
      if (r >= R || c >= K) continue;
      V v = tile[q][tx];
      if (conj) v.y = -v.y;
      if (scale) {
        const T x = sr * v.x - si * v.y, y = sr * v.y + si * v.x;
        v.x = x;
        v.y = y;
      }
      if constexpr (MODE == kPackDense) {
        reinterpret_cast<V *>(out)[r + (int64_t)c * ldo] = v;
      } else if constexpr (MODE == kPackEmbed) {
        V *o = reinterpret_cast<V *>(out);
        V w;
        w.x = -v.y;
        w.y = v.x;
        o[r + (int64_t)(2 * c) * ldo] = v;
        o[r + (int64_t)(2 * c + 1) * ldo] = w;
      } else if constexpr (MODE == kPackPlanar) {
        const int64_t at = r + (int64_t)c * ldo;
        out[at] = v.x;
        out[plane + at] = v.y;
        out[2 * plane + at] = v.x + v.y;
      } else {
        out[r + (int64_t)(2 * c) * ldo] = v.x;
        out[r + (int64_t)(2 * c + 1) * ldo] = v.y;
      }
    }
    __syncthreads();  // the tile is refilled for the next row block
  }
}

// C = beta * C over the m x n window (complex multiply: beta == 0 still
// multiplies, so NaN/Inf in C propagate as in the real path).
template <typename T>
__global__ void __launch_bounds__(256)
    cx_scale_kernel(T *__restrict__ C, int64_t ldc, int m, int n, T br, T bi) {
  using V = typename Cx<T>::v;
  V *Cv = reinterpret_cast<V *>(C);
  const int64_t total = (int64_t)m * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = idx / m, i = idx - j * m;
    const V v = Cv[i + j * ldc];
    V w;
    w.x = br * v.x - bi * v.y;
    w.y = br * v.y + bi * v.x;
    Cv[i + j * ldc] = w;
  }
}

// 3M combine: P = (T1 - T2) + i (T3 - T1 - T2); C = alpha * P + beta * C.
template <typename T>
__global__ void __launch_bounds__(256)
    cx_combine3m_kernel(const T *__restrict__ Tp, int64_t ldt, int64_t plane, T *__restrict__ C,
                        int64_t ldc, int m, int n, T ar, T ai, T br, T bi) {
  using V = typename Cx<T>::v;
  V *Cv = reinterpret_cast<V *>(C);
  const int64_t total = (int64_t)m * n;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = idx / m, i = idx - j * m;
    const int64_t at = i + j * ldt;
    const T t1 = Tp[at], t2 = Tp[plane + at], t3 = Tp[2 * plane + at];
    const T pr = t1 - t2, pi = (t3 - t1) - t2;
    const V c = Cv[i + j * ldc];
    V w;
    w.x = (ar * pr - ai * pi) + (br * c.x - bi * c.y);
    w.y = (ar * pi + ai * pr) + (br * c.y + bi * c.x);
    Cv[i + j * ldc] = w;
  }
}

unsigned elementwise_grid(int64_t total) {
  const int64_t b = (total + 255) / 256;
  return (unsigned)(b < 152 * 16 ? (b > 0 ? b : 1) : 152 * 16);
}

template <typename T, int MODE>
void launch_pack(const T *X, int64_t ld, int R, int K, bool trans, bool conj, bool scale, T sr,
                 T si, T *out, int64_t ldo, int64_t plane, cudaStream_t st) {
  const int64_t rb = (R + 31) / 32;
  const dim3 grid((unsigned)((K + 31) / 32), (unsigned)(rb < 65535 ? rb : 65535));
  cx_pack_kernel<T, MODE><<<grid, 256, 0, st>>>(X, ld, R, K, trans ? 1 : 0, conj ? 1 : 0,
                                                scale ? 1 : 0, sr, si, out, ldo, plane);
}

template <typename T>
int real_plain(char ta, char tb, int m, int n, int k, T alpha, const T *A, int lda, const T *B,
               int ldb, T beta, T *C, int ldc, cudaStream_t st, unsigned *err) {
  if constexpr (sizeof(T) == 8)
    return plain_dgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, st, err);
  else
    return plain_sgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, st, err);
}

// Workspace layout (offsets from the 256-byte aligned base).
struct CxLayout {
  bool ok = false;
  int64_t lde = 0, ldbh = 0;         // 4M / split: Ahat and Bhat leading dims (reals)
  bool bt = false;                   // Bhat stored transposed (n x 2k), see cx_layout
  int64_t ld3a = 0, ld3b = 0;        // 3M: planar A (m x k) and op(B)^T (n x k) leading dims
  size_t a_off = 0, b_off = 0, t_off = 0, s_off = 0, s_bytes = 0, total = 0;
};

inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

CxLayout cx_layout(size_t e, bool is_double, int method, char tb, int m, int n, int k,
                   int param) {
  CxLayout L;
  size_t off = 0;
  if (method == GB300_CPLX_3M) {
    // the B planes hold op(B)^T (n x k): B MN-major suits the FFMA kernel
    L.ld3a = rup(m, 32);
    L.ld3b = rup(n, 32);
    L.a_off = off;
    off = al256(off + (size_t)(3 * L.ld3a * k) * e);
    L.b_off = off;
    off = al256(off + (size_t)(3 * L.ld3b * k) * e);
    L.t_off = off;
    off = al256(off + (size_t)(3 * L.ld3a * n) * e);
  } else {
    L.lde = rup(2 * (int64_t)m, 32);
    L.a_off = off;
    off = al256(off + (size_t)(L.lde * 2 * (int64_t)k) * e);
    // The plain FP32 kernel runs fastest with B MN-major (packed f32x2 FMAs):
    // 4M CGEMM stores Bhat transposed, n x 2k, real and imaginary parts in
    // adjacent columns.
    L.bt = (method == GB300_CPLX_4M && !is_double);
    if (L.bt) {
      L.ldbh = rup(n, 32);
      L.b_off = off;
      off = al256(off + (size_t)(L.ldbh * 2 * (int64_t)k) * e);
    } else if (cx_trans(tb) || cx_conj(tb)) {
      L.ldbh = rup(2 * (int64_t)k, 32);
      L.b_off = off;
      off = al256(off + (size_t)(L.ldbh * n) * e);
    }
    if (method == GB300_CPLX_SPLIT || method == GB300_CPLX_CRT) {
      L.s_bytes = method == GB300_CPLX_CRT
                      ? crt_workspace_bytes(2 * m, n, 2 * k, param)
                      : split_workspace_bytes(is_double ? 1 : 0, 2 * m, n, 2 * k, param);
      if (!L.s_bytes) return L;
      L.s_off = off;
      off = al256(off + L.s_bytes);
    }
  }
  L.total = off + 256;
  L.ok = true;
  return L;
}

int cx_check(char ta, char tb, int m, int n, int k, int lda, int ldb, int ldc, int method) {
  if (method < GB300_CPLX_4M || method > GB300_CPLX_CRT) return GB300_ERR_ARG;
  const int arows = cx_trans(ta) ? k : m, brows = cx_trans(tb) ? n : k;
  if (m < 0 || n < 0 || k < 0 || lda < (arows > 1 ? arows : 1) ||
      ldb < (brows > 1 ? brows : 1) || ldc < (m > 1 ? m : 1))
    return GB300_ERR_ARG;
  // the embedded real problem has 2m rows, 2k inner length and ld 2*ldc
  if (m > 0x3fffffff || k > 0x3fffffff || ldc > 0x3fffffff || ldb > 0x3fffffff)
    return GB300_ERR_ARG;
  return (m == 0 || n == 0) ? -1 : GB300_OK;
}

template <typename T>
int complex_gemm(char ta, char tb, int m, int n, int k, const T *alpha, const T *A, int lda,
                 const T *B, int ldb, const T *beta, T *C, int ldc, int method, int param,
                 void *ws, size_t ws_bytes, cudaStream_t st, unsigned *err) {
  const int ck = cx_check(ta, tb, m, n, k, lda, ldb, ldc, method);
  if (ck != GB300_OK) return ck < 0 ? GB300_OK : ck;
  if (method == GB300_CPLX_CRT && sizeof(T) != 8) return GB300_ERR_ARG;  // ZGEMM only
  const T ar = alpha[0], ai = alpha[1], br = beta[0], bi = beta[1];
  const bool alpha_zero = ar == T(0) && ai == T(0);
  if (alpha_zero || k == 0) {
    if (br == T(1) && bi == T(0)) return GB300_OK;
    const int64_t total = (int64_t)m * n;
    cx_scale_kernel<T><<<elementwise_grid(total), 256, 0, st>>>(C, ldc, m, n, br, bi);
    return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
  }
  const bool dbl = sizeof(T) == 8;
  const CxLayout L = cx_layout(sizeof(T), dbl, method, tb, m, n, k, param);
  if (!L.ok) return GB300_ERR_ARG;
  if (!ws || ws_bytes < L.total) return GB300_ERR_WORKSPACE;
  uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(ws) + 255) &
                                              ~uintptr_t(255));
  const bool ta_t = cx_trans(ta), ta_c = cx_conj(ta), tb_t = cx_trans(tb), tb_c = cx_conj(tb);

  if (method == GB300_CPLX_3M) {
    T *Ap = reinterpret_cast<T *>(base + L.a_off);
    T *Bp = reinterpret_cast<T *>(base + L.b_off);
    T *Tp = reinterpret_cast<T *>(base + L.t_off);
    const int64_t pa = L.ld3a * k, pb = L.ld3b * k, pt = L.ld3a * n;
    launch_pack<T, kPackPlanar>(A, lda, m, k, ta_t, ta_c, false, T(1), T(0), Ap, L.ld3a, pa, st);
    launch_pack<T, kPackPlanar>(B, ldb, n, k, !tb_t, tb_c, false, T(1), T(0), Bp, L.ld3b, pb, st);
    // the products overwrite T (beta = 0 still reads it, so clear it first)
    if (cudaMemsetAsync(Tp, 0, (size_t)(3 * pt) * sizeof(T), st) != cudaSuccess)
      return GB300_ERR_CUDA;
    for (int p = 0; p < 3; ++p) {
      const int rc = real_plain<T>('N', 'T', m, n, k, T(1), Ap + p * pa, (int)L.ld3a, Bp + p * pb,
                                   (int)L.ld3b, T(0), Tp + p * pt, (int)L.ld3a, st, err);
      if (rc != GB300_OK) return rc;
    }
    const int64_t total = (int64_t)m * n;
    cx_combine3m_kernel<T><<<elementwise_grid(total), 256, 0, st>>>(Tp, L.ld3a, pt, C, ldc, m, n,
                                                                    ar, ai, br, bi);
    return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
  }

  // 4M / split: the embedded real problem
  T beta_r = br;
  if (bi != T(0)) {
    const int64_t total = (int64_t)m * n;
    cx_scale_kernel<T><<<elementwise_grid(total), 256, 0, st>>>(C, ldc, m, n, br, bi);
    beta_r = T(1);
  }
  const bool fold = ai != T(0);
  const T alpha_r = fold ? T(1) : ar;
  T *Ah = reinterpret_cast<T *>(base + L.a_off);
  launch_pack<T, kPackEmbed>(A, lda, m, k, ta_t, ta_c, fold, ar, ai, Ah, L.lde / 2, 0, st);
  const T *Bh = B;
  int64_t ldbh = 2 * (int64_t)ldb;
  char tbh = 'N';
  if (L.bt) {
    // op(B)^T, n x k, written as real columns (re, im) per k
    T *Bw = reinterpret_cast<T *>(base + L.b_off);
    launch_pack<T, kPackCols>(B, ldb, n, k, !tb_t, tb_c, false, T(1), T(0), Bw, L.ldbh, 0, st);
    Bh = Bw;
    ldbh = L.ldbh;
    tbh = 'T';
  } else if (tb_t || tb_c) {
    T *Bw = reinterpret_cast<T *>(base + L.b_off);
    launch_pack<T, kPackDense>(B, ldb, k, n, tb_t, tb_c, false, T(1), T(0), Bw, L.ldbh / 2, 0, st);
    Bh = Bw;
    ldbh = L.ldbh;
  }
  if (cudaGetLastError() != cudaSuccess) return GB300_ERR_CUDA;
  const int M2 = 2 * m, K2 = 2 * k, ldc2 = 2 * ldc;
  if (method == GB300_CPLX_4M)
    return real_plain<T>('N', tbh, M2, n, K2, alpha_r, Ah, (int)L.lde, Bh, (int)ldbh, beta_r, C,
                         ldc2, st, err);
  void *sws = base + L.s_off;
  if constexpr (sizeof(T) == 8) {
    if (method == GB300_CPLX_CRT)
      return crt_dgemm('N', 'N', M2, n, K2, alpha_r, Ah, (int)L.lde, Bh, (int)ldbh, beta_r, C,
                       ldc2, param, sws, L.s_bytes, st, err);
    return ozaki_dgemm('N', 'N', M2, n, K2, alpha_r, Ah, (int)L.lde, Bh, (int)ldbh, beta_r, C,
                       ldc2, param, sws, L.s_bytes, st, err);
  }
  else
    return split_sgemm('N', 'N', M2, n, K2, alpha_r, Ah, (int)L.lde, Bh, (int)ldbh, beta_r, C,
                       ldc2, param, sws, L.s_bytes, st, err);
}

}  // namespace

size_t complex_workspace_bytes(int is_double, int method, char tb, int m, int n, int k,
                               int param) {
  if (m <= 0 || n <= 0 || k <= 0 || method < GB300_CPLX_4M || method > GB300_CPLX_CRT) return 0;
  if (method == GB300_CPLX_CRT && !is_double) return 0;
  const CxLayout L =
      cx_layout(is_double ? 8 : 4, is_double != 0, method, tb, m, n, k, param);
  return L.ok ? L.total : 0;
}

int complex_gemm_d(char ta, char tb, int m, int n, int k, const double *alpha, const double *A,
                   int lda, const double *B, int ldb, const double *beta, double *C, int ldc,
                   int method, int param, void *ws, size_t ws_bytes, cudaStream_t st,
                   unsigned *err) {
  return complex_gemm<double>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, method, param,
                              ws, ws_bytes, st, err);
}

int complex_gemm_s(char ta, char tb, int m, int n, int k, const float *alpha, const float *A,
                   int lda, const float *B, int ldb, const float *beta, float *C, int ldc,
                   int method, int param, void *ws, size_t ws_bytes, cudaStream_t st,
                   unsigned *err) {
  return complex_gemm<float>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, method, param,
                             ws, ws_bytes, st, err);
}

int complex_check(char ta, char tb, int m, int n, int k, int lda, int ldb, int ldc, int method) {
  return cx_check(ta, tb, m, n, k, lda, ldb, ldc, method);
}

}  // namespace gb300
