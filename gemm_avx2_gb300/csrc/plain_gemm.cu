// plain_gemm.cu -- the drop-in ("plain") forms of the reference's sgemm_/dgemm_:
//   C = alpha*op(A)*op(B) + beta*C, column-major, any m/n/k/ld, op = N or T.
//
// Reference path replaced (wjc404/GEMM_AVX2):
//   driver blocking loop        src/gemm_driver.c:118-197  -> tile grid + grouped raster
//   A/B panel packing           src/gemm_copy.c:1-143      -> TMA boxes into shared memory
//                                                             (transposes = box orientation)
//   FMA3 register micro-kernel  src/kernel/gemm_kernel.S   -> register-blocked FFMA (FP32) /
//                                                             DMMA m16n8k8 (FP64) consumers
//   ragged-edge kernels         src/edge_kernel/*          -> TMA out-of-bounds zero fill +
//                                                             predicated epilogue stores
//   C_MULT_BETA + alpha-in-B    src/gemm_driver.c:106-116, src/gemm_copy.c:65
//                                                          -> fused alpha/beta epilogue
//   OpenMP N split + spin barrier src/gemm_driver.c:23-33,138 -> CTA grid; mbarrier pipeline
//
// Kernel shape (both precisions): 128x128 CTA tile, a 4-stage shared-memory ring
// filled by one producer warp (TMA 2-D boxes, or cp.async element copies when a
// leading dimension / base address breaks TMA's 16-byte rules), 8 consumer warps.
//   FP32: each consumer thread owns an 8x8 register tile (FFMA pipe).
//   FP64: each consumer warp owns a 64x32 tile of m16n8k8 DMMA fragments (the
//         FP64 tensor path; measured on GB300 at 8x the DFMA rate).
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "common.cuh"
#include "plain_gemm.h"
#include "plain_tiles.cuh"

namespace gb300 {

// The FP32 kernel has no dedicated producer warp: 8 warps (256 threads, up to
// 255 registers each) all compute, and thread 0 also refills the ring with TMA
// ST - 1 tiles ahead.  With a ninth warp the register budget drops to 168
// and the K-major variants spill into the inner loop.
constexpr int kThreadsS = kConsumerWarps * 32;

template <bool AK, bool BK_, int ST>
__global__ void __launch_bounds__(kThreadsS, 1)
sgemm_plain_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   OperandDesc opA, OperandDesc opB, int use_tma, int m, int n, int k, float alpha,
                   float beta, float *__restrict__ C, int ldc, int tiles_m, int tiles_n,
                   int kt_per, float *__restrict__ part, unsigned *err) {
  constexpr int BK = PlainTraits<float>::BK;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                              ~uintptr_t(1023));
  float *sA = reinterpret_cast<float *>(smem);
  float *sB = sA + ST * kBM * BK;
  uint64_t *full = reinterpret_cast<uint64_t *>(sB + ST * kBN * BK);
  uint64_t *empty = full + ST;
  volatile int *abort_flag = reinterpret_cast<volatile int *>(empty + ST);

  int tmi, tni;
  tile_coords(blockIdx.x, tiles_m, tiles_n, kGroupM, tmi, tni);
  const int m0 = tmi * kBM, n0 = tni * kBN;
  // K slice blockIdx.y: k-tiles [kt0, kt0 + ktiles) (split-K; one slice otherwise)
  const int kt0 = (int)blockIdx.y * kt_per;
  const int ktiles = max(0, min((k + BK - 1) / BK - kt0, kt_per));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool tma = use_tma != 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < ST; ++s) {
      mbar_init(&full[s], tma ? 1 : kThreadsS);
      mbar_init(&empty[s], kConsumerWarps);
    }
    *abort_flag = 0;
    fence_barrier_init();
    if (tma) { tma_prefetch_desc(&tmA); tma_prefetch_desc(&tmB); }
  }
  __syncthreads();

  // Fill the slice's k-tile kt into its stage.  TMA: thread 0 only.  Fallback:
  // every thread copies a strided share of the elements with cp.async and arrives once.
  auto fill = [&](int kt) {
    const int s = kt % ST;
    float *ta = sA + s * (kBM * BK);
    float *tb = sB + s * (kBN * BK);
    const int k0 = (kt0 + kt) * BK;
    if (tma) {
      if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(&full[s], 2 * tile_bytes<float>());
        if (AK) tma_load_2d(ta, &tmA, k0, m0, &full[s]);
        else    tma_load_2d(ta, &tmA, m0, k0, &full[s]);
        if (BK_) tma_load_2d(tb, &tmB, k0, n0, &full[s]);
        else     tma_load_2d(tb, &tmB, n0, k0, &full[s]);
      }
    } else {
      const float *baseA = static_cast<const float *>(opA.ptr);
      const float *baseB = static_cast<const float *>(opB.ptr);
      for (int e = threadIdx.x; e < kBM * BK; e += kThreadsS) {
        int mn, kk;
        if (AK) { mn = e / BK; kk = e % BK; } else { kk = e / kBM; mn = e % kBM; }
        const int r = AK ? (k0 + kk) : (m0 + mn), c = AK ? (m0 + mn) : (k0 + kk);
        const bool ok = r < opA.rows && c < opA.cols;
        cp_async_4(ta + tile_off<float, AK>(mn, kk), ok ? baseA + (int64_t)c * opA.ld + r : baseA, ok);
      }
      for (int e = threadIdx.x; e < kBN * BK; e += kThreadsS) {
        int mn, kk;
        if (BK_) { mn = e / BK; kk = e % BK; } else { kk = e / kBN; mn = e % kBN; }
        const int r = BK_ ? (k0 + kk) : (n0 + mn), c = BK_ ? (n0 + mn) : (k0 + kk);
        const bool ok = r < opB.rows && c < opB.cols;
        cp_async_4(tb + tile_off<float, BK_>(mn, kk), ok ? baseB + (int64_t)c * opB.ld + r : baseB, ok);
      }
      cp_async_mbar_arrive(&full[s]);
    }
  };

  // thread coordinates of the 8x8 register tile
  const int wm = warp & 1, wn = warp >> 1;
  const int tm = wm * 8 + (lane & 7);
  const int tn = wn * 4 + (lane >> 3);
  // Packed FMAs (fma.rn.f32x2, the same round-to-nearest FMA per element) need
  // both operand pairs in adjacent registers, which a float4 shared-memory load
  // gives along its contiguous dimension:
  //   B MN-major:             pairs along j (columns of C): acc[i][j/2]
  //   A MN-major, B K-major:  pairs along i (rows of C):    acc[i/2][j]
  //   A and B K-major:        pairs along k: acc[i][j] holds the even-k and
  //                           odd-k partial sums, added once in the epilogue
  constexpr int kPairJ = 0, kPairI = 1, kPairK = 2;
  constexpr int mode = !BK_ ? kPairJ : (AK ? kPairK : kPairI);
  float2 acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = make_float2(0.f, 0.f);

  for (int kt = 0; kt < ST - 1 && kt < ktiles; ++kt) fill(kt);

  bool ok = true;
  for (int kt = 0; kt < ktiles; ++kt) {
    // refill the stage consumed in iteration kt-1 with k-tile kt + ST - 1
    const int nk = kt + ST - 1;
    if (nk < ktiles) {
      if (kt >= 1 && (!tma || threadIdx.x == 0)) {
        if (!mbar_wait(&empty[nk % ST], ((nk / ST) - 1) & 1, err, kErrTimeoutEmpty,
                       abort_flag)) { ok = false; break; }
      }
      fill(nk);
    }
    const int s = kt % ST;
    if (!mbar_wait(&full[s], (kt / ST) & 1, err, kErrTimeoutFull, abort_flag)) { ok = false; break; }
    const float *ta = sA + s * (kBM * BK);
    const float *tb = sB + s * (kBN * BK);
    if constexpr (mode == kPairJ) {
#pragma unroll 2
      for (int kq = 0; kq < BK / 4; ++kq) {
        float a[8][4], b[8][4];
        f32_load_frag<AK>(ta, tm, kq, a);
        f32_load_frag<BK_>(tb, tn, kq, b);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float2 bp[4];
#pragma unroll
          for (int jp = 0; jp < 4; ++jp) bp[jp] = make_float2(b[2 * jp][q], b[2 * jp + 1][q]);
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const float2 ab = make_float2(a[i][q], a[i][q]);
#pragma unroll
            for (int jp = 0; jp < 4; ++jp) acc[i][jp] = __ffma2_rn(ab, bp[jp], acc[i][jp]);
          }
        }
      }
    } else if constexpr (mode == kPairI) {
#pragma unroll 2
      for (int kq = 0; kq < BK / 4; ++kq) {
        float a[8][4], b[8][4];
        f32_load_frag<AK>(ta, tm, kq, a);
        f32_load_frag<BK_>(tb, tn, kq, b);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float2 ap[4];
#pragma unroll
          for (int ip = 0; ip < 4; ++ip) ap[ip] = make_float2(a[2 * ip][q], a[2 * ip + 1][q]);
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const float2 bb = make_float2(b[j][q], b[j][q]);
#pragma unroll
            for (int ip = 0; ip < 4; ++ip) acc[ip][j] = __ffma2_rn(ap[ip], bb, acc[ip][j]);
          }
        }
      }
    } else {
#pragma unroll 1
      for (int kq = 0; kq < BK / 4; ++kq) {
        float a[8][4], b[8][4];
        f32_load_frag<AK>(ta, tm, kq, a);
        f32_load_frag<BK_>(tb, tn, kq, b);
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const float2 ap = make_float2(a[i][2 * h], a[i][2 * h + 1]);
#pragma unroll
            for (int j = 0; j < 8; ++j)
              acc[i][j] = __ffma2_rn(ap, make_float2(b[j][2 * h], b[j][2 * h + 1]), acc[i][j]);
          }
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
  if (!ok) return;

  // fused alpha/beta epilogue (beta*C first, as src/gemm_driver.c:133 does; beta == 0
  // still multiplies, so NaN/Inf already in C propagate like the reference).
  auto value = [&](int i, int j) -> float {
    if constexpr (mode == kPairJ) return (j & 1) ? acc[i][j >> 1].y : acc[i][j >> 1].x;
    else if constexpr (mode == kPairI) return (i & 1) ? acc[i >> 1][j].y : acc[i >> 1][j].x;
    else return acc[i][j].x + acc[i][j].y;
  };
  if (part) {  // split-K: the slice's raw sums, combined by splitk_reduce_kernel
    float *ps = part + (int64_t)blockIdx.y * m * n;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int col = n0 + f32_row<BK_>(tn, j);
      if (col >= n) continue;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int row = m0 + f32_row<AK>(tm, i);
        if (row < m) ps[(int64_t)col * m + row] = value(i, j);
      }
    }
    return;
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int col = n0 + f32_row<BK_>(tn, j);
    if (col >= n) continue;
    float *cc = C + (int64_t)col * ldc;
    float cv[8];  // the column's 8 loads first, then the stores
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int row = m0 + f32_row<AK>(tm, i);
      cv[i] = (row < m) ? cc[row] : 0.f;
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int row = m0 + f32_row<AK>(tm, i);
      if (row < m) {
        const float cb = (beta == 1.0f) ? cv[i] : cv[i] * beta;
        cc[row] = cb + alpha * value(i, j);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// FP64 consumer: m16n8k8 DMMA fragments, warp tile 64 (m) x 32 (n)
// ---------------------------------------------------------------------------
template <bool AK, bool BK_, int ST>
__global__ void __launch_bounds__(kThreads, 1)
dgemm_plain_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   OperandDesc opA, OperandDesc opB, int use_tma, int m, int n, int k,
                   double alpha, double beta, double *__restrict__ C, int ldc, int tiles_m,
                   int tiles_n, int kt_per, double *__restrict__ part, unsigned *err) {
  constexpr int BK = PlainTraits<double>::BK;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                              ~uintptr_t(1023));
  double *sA = reinterpret_cast<double *>(smem);
  double *sB = sA + ST * kBM * BK;
  uint64_t *full = reinterpret_cast<uint64_t *>(sB + ST * kBN * BK);
  uint64_t *empty = full + ST;
  volatile int *abort_flag = reinterpret_cast<volatile int *>(empty + ST);

  int tmi, tni;
  tile_coords(blockIdx.x, tiles_m, tiles_n, kGroupM, tmi, tni);
  const int m0 = tmi * kBM, n0 = tni * kBN;
  // K slice blockIdx.y: k-tiles [kt0, kt0 + ktiles) (split-K; one slice otherwise)
  const int kt0 = (int)blockIdx.y * kt_per;
  const int ktiles = max(0, min((k + BK - 1) / BK - kt0, kt_per));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < ST; ++s) {
      mbar_init(&full[s], use_tma ? 1 : 32);
      mbar_init(&empty[s], kConsumerWarps);
    }
    *abort_flag = 0;
    fence_barrier_init();
    if (use_tma) { tma_prefetch_desc(&tmA); tma_prefetch_desc(&tmB); }
  }
  __syncthreads();

  if (warp == kConsumerWarps) {
    producer_loop<double, AK, BK_, ST>(&tmA, &tmB, opA, opB, use_tma != 0, sA, sB, full, empty,
                                       m0, n0, kt0, ktiles, err, abort_flag);
    return;
  }

  const int wm = warp & 1, wn = warp >> 1;  // 2 x 4 warps, warp tile 64 x 32
  const int g = lane >> 2, t = lane & 3;
  double acc[4][4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.0;

  bool ok = true;
  for (int kt = 0; kt < ktiles; ++kt) {
    const int s = kt % ST;
    if (!mbar_wait(&full[s], (kt / ST) & 1, err, kErrTimeoutFull, abort_flag)) { ok = false; break; }
    const double *ta = sA + s * (kBM * BK);
    const double *tb = sB + s * (kBN * BK);
#pragma unroll
    for (int k8 = 0; k8 < BK; k8 += 8) {
      double a[4][4], b[4][2];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int mb = wm * 64 + i * 16;
#pragma unroll
        for (int r = 0; r < 4; ++r)
          a[i][r] = ta[tile_off<double, AK>(mb + g + 8 * (r & 1), k8 + t + 4 * (r >> 1))];
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int nb = wn * 32 + j * 8;
#pragma unroll
        for (int r = 0; r < 2; ++r) b[j][r] = tb[tile_off<double, BK_>(nb + g, k8 + t + 4 * r)];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) dmma_16x8x8(acc[i][j], a[i], b[j]);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
  if (!ok) return;

  if (part) {  // split-K: the slice's raw sums, combined by splitk_reduce_kernel
    double *ps = part + (int64_t)blockIdx.y * m * n;
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int cj = 0; cj < 2; ++cj) {
        const int col = n0 + wn * 32 + j * 8 + 2 * t + cj;
        if (col >= n) continue;
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int ri = 0; ri < 2; ++ri) {
            const int row = m0 + wm * 64 + i * 16 + g + 8 * ri;
            if (row < m) ps[(int64_t)col * m + row] = acc[i][j][2 * ri + cj];
          }
      }
    return;
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
#pragma unroll
    for (int cj = 0; cj < 2; ++cj) {
      const int col = n0 + wn * 32 + j * 8 + 2 * t + cj;
      if (col >= n) continue;
      double *cc = C + (int64_t)col * ldc;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
#pragma unroll
        for (int ri = 0; ri < 2; ++ri) {
          const int row = m0 + wm * 64 + i * 16 + g + 8 * ri;
          if (row < m) {
            const double c0 = cc[row];
            const double cb = (beta == 1.0) ? c0 : c0 * beta;
            cc[row] = cb + alpha * acc[i][j][2 * ri + cj];
          }
        }
      }
    }
  }
}

// C *= beta over the m x n window (alpha == 0, or k == 0 with the +0 of an empty sum).
// Column c of the copy is `wv` vectors V; each thread moves 4 of them (loads
// issued before stores), 256 threads cover 1024 vectors of one column.
template <typename V>
__global__ void __launch_bounds__(256) copy_2d_kernel(V *__restrict__ dst, size_t dp,
                                                      const V *__restrict__ src, size_t sp,
                                                      size_t wv, int cols) {
  const size_t c0 = (size_t)blockIdx.x * 1024 + threadIdx.x;
  for (int col = blockIdx.y; col < cols; col += gridDim.y) {
    const V *s = src + (size_t)col * sp;
    V *d = dst + (size_t)col * dp;
    V v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (c0 + 256 * u < wv) v[u] = s[c0 + 256 * u];
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (c0 + 256 * u < wv) d[c0 + 256 * u] = v[u];
  }
}

int copy_2d(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, int cols,
            cudaStream_t st) {
  if (width == 0 || cols <= 0) return GB300_OK;
  const uintptr_t align = reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src) |
                          dpitch | spitch | width;
  auto launch = [&](auto *tag) {
    using V = std::remove_pointer_t<decltype(tag)>;
    const size_t wv = width / sizeof(V);
    const dim3 grid((unsigned)((wv + 1023) / 1024), (unsigned)(cols < 65535 ? cols : 65535));
    copy_2d_kernel<V><<<grid, 256, 0, st>>>(static_cast<V *>(dst), dpitch / sizeof(V),
                                             static_cast<const V *>(src), spitch / sizeof(V), wv,
                                             cols);
  };
  if ((align & 15) == 0)
    launch(static_cast<uint4 *>(nullptr));
  else if ((align & 7) == 0)
    launch(static_cast<uint2 *>(nullptr));
  else if ((align & 3) == 0)
    launch(static_cast<unsigned *>(nullptr));
  else
    launch(static_cast<uint8_t *>(nullptr));
  return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
}

template <typename T>
__global__ void scale_c_kernel(int m, int n, T beta, T add, T *__restrict__ C, int ldc) {
  const int64_t total = (int64_t)m * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int col = (int)(e / m), row = (int)(e % m);
    T *p = C + (int64_t)col * ldc + row;
    *p = (beta == T(1) ? *p : *p * beta) + add;
  }
}

// Split-K combination: C = beta * C, then C += alpha * P_s for s = 0, 1, ...
// in slice order (the reference applies C_MULT_BETA first and then adds each
// K block's sum to C, src/gemm_driver.c:133,156-190).  P: S slices of m x n
// (ld m).  beta == 0 still multiplies, so NaN / Inf in C propagate.
template <typename T>
__global__ void __launch_bounds__(256) splitk_reduce_kernel(int m, int n, int S,
                                                            const T *__restrict__ P, T alpha,
                                                            T beta, T *__restrict__ C, int ldc) {
  const int64_t total = (int64_t)m * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int col = (int)(e / m), row = (int)(e % m);
    T *p = C + (int64_t)col * ldc + row;
    T c = (beta == T(1)) ? *p : *p * beta;
    for (int sl = 0; sl < S; ++sl) c = fma(alpha, P[sl * total + e], c);
    *p = c;
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 152;
  }
  return n;
}

// Split-K factor and ring depth of the plain kernels (GB300_TUNE_SPLIT_K,
// GB300_TUNE_PLAIN_STAGES; 0 = the tuned value of the shape class, else by
// shape / the default depth).
static int g_split_k = 0, g_plain_stages = 0;
void set_plain_split_k(int v) { g_split_k = v; }
void set_plain_stages(int v) { g_plain_stages = v; }
int plain_split_override() { return g_split_k; }
int plain_stages_override() { return g_plain_stages; }

// Split-K by shape: the factor S in 1..32 that minimises the modelled time
// ceil(tiles * S / SMs) waves x (ceil(ktiles / S) + 2) k-tiles (2: the ring's
// fill and drain) plus the combination pass (S + 2 slices of m x n through
// HBM, in k-tile times), with at least 8 k-tiles (128 or 256 K) per slice.
// Measured on GB300: DGEMM 2048^3 0.90 -> 1.03 TFLOP/s (S = 4), DGEMM
// 512 x 512 x 16384 0.11 -> 1.01 (S = 9), SGEMM 512 x 512 x 16384 5.6 -> 47.0.
static int split_k_by_shape(bool dbl, int m, int n, int k) {
  const int64_t tiles = (int64_t)((m + kBM - 1) / kBM) * ((n + kBN - 1) / kBN);
  const int BK = dbl ? PlainTraits<double>::BK : PlainTraits<float>::BK;
  const int ktiles = (k + BK - 1) / BK;
  const int sms = sm_count();
  if (ktiles < 16) return 1;
  // one k-tile of one CTA: 2 * 128 * 128 * BK flop at the pipe's per-SM rate
  // (FP64 1.05 TFLOP/s, FFMA about 55 TFLOP/s over 152 SMs)
  const double ktile_s = 2.0 * kBM * kBN * BK / ((dbl ? 1.05e12 : 55e12) / 152);
  const double slice_s = (double)m * n * (dbl ? 8 : 4) / 6.5e12;
  double best = 0;
  int bs = 1;
  for (int S = 1; S <= 32 && (S == 1 || ktiles / S >= 8); ++S) {
    const double waves = (double)((tiles * S + sms - 1) / sms);
    const double t = waves * ((ktiles + S - 1) / S + 2) * ktile_s +
                     (S > 1 ? (S + 2) * slice_s : 0.0);
    if (S == 1 || t < best) { best = t; bs = S; }
  }
  return bs;
}

int plain_split_k(int is_double, int m, int n, int k) {
  const int BK = is_double ? PlainTraits<double>::BK : PlainTraits<float>::BK;
  const int ktiles = (k + BK - 1) / BK;
  int S = g_split_k;
  if (!S) S = tune_plain_split(is_double ? 3 : 4, m, n, k);
  if (!S) S = split_k_by_shape(is_double != 0, m, n, k);
  if (S > ktiles) S = ktiles;
  if (S > 65535) S = 65535;
  return S < 1 ? 1 : S;
}

static int plain_stages_for(int is_double, int m, int n, int k) {
  int st = g_plain_stages;
  if (!st) st = tune_plain_stages(is_double ? 3 : 4, m, n, k);
  return st == 6 ? 6 : kStages;
}

size_t plain_workspace_bytes(int is_double, int m, int n, int k) {
  if (m <= 0 || n <= 0 || k <= 0) return 0;
  const int S = plain_split_k(is_double, m, n, k);
  return S > 1 ? (size_t)S * m * n * (is_double ? 8 : 4) : 0;
}
template <typename T>
static void make_desc(OperandDesc &d, const T *p, int ld, int rows, int cols) {
  d.ptr = p; d.ld = ld; d.rows = rows; d.cols = cols;
}

template <typename T, bool AK, bool BK_, int ST>
static int launch_one(const CUtensorMap &tA, const CUtensorMap &tB, const OperandDesc &oA,
                      const OperandDesc &oB, bool tma, int m, int n, int k, T alpha, T beta, T *C,
                      int ldc, int S, T *part, cudaStream_t st, unsigned *err) {
  const int tiles_m = (m + kBM - 1) / kBM, tiles_n = (n + kBN - 1) / kBN;
  const int smem = plain_smem_bytes<T, ST>();
  void (*kern)(const CUtensorMap, const CUtensorMap, OperandDesc, OperandDesc, int, int, int, int,
               T, T, T *, int, int, int, int, T *, unsigned *);
  if constexpr (sizeof(T) == 4)
    kern = sgemm_plain_kernel<AK, BK_, ST>;
  else
    kern = dgemm_plain_kernel<AK, BK_, ST>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return GB300_ERR_CUDA;
  const int64_t ntiles = (int64_t)tiles_m * tiles_n;
  if (ntiles > 0x7fffffff) return GB300_ERR_ARG;
  constexpr int BK = PlainTraits<T>::BK;
  const int ktiles = (k + BK - 1) / BK;
  const int kt_per = (ktiles + S - 1) / S;
  const int slices = (ktiles + kt_per - 1) / kt_per;  // every slice has a k-tile
  kern<<<dim3((unsigned)ntiles, (unsigned)slices), sizeof(T) == 4 ? kThreadsS : kThreads, smem,
         st>>>(tA, tB, oA, oB, tma ? 1 : 0, m, n, k, alpha, beta, C, ldc, tiles_m, tiles_n,
               kt_per, slices > 1 ? part : nullptr, err);
  if (cudaGetLastError() != cudaSuccess) return GB300_ERR_CUDA;
  if (slices > 1) {
    const int64_t total = (int64_t)m * n;
    int blocks = (int)((total + 255) / 256);
    if (blocks > sm_count() * 8) blocks = sm_count() * 8;
    splitk_reduce_kernel<T><<<blocks, 256, 0, st>>>(m, n, slices, part, alpha, beta, C, ldc);
    if (cudaGetLastError() != cudaSuccess) return GB300_ERR_CUDA;
  }
  return GB300_OK;
}

template <typename T, bool AK, bool BK_>
static int launch_depth(int ST, const CUtensorMap &tA, const CUtensorMap &tB,
                        const OperandDesc &oA, const OperandDesc &oB, bool tma, int m, int n,
                        int k, T alpha, T beta, T *C, int ldc, int S, T *part, cudaStream_t st,
                        unsigned *err) {
  if (ST == 6)
    return launch_one<T, AK, BK_, 6>(tA, tB, oA, oB, tma, m, n, k, alpha, beta, C, ldc, S, part,
                                     st, err);
  return launch_one<T, AK, BK_, kStages>(tA, tB, oA, oB, tma, m, n, k, alpha, beta, C, ldc, S,
                                         part, st, err);
}

template <typename T>
static int plain_gemm(char ta, char tb, int m, int n, int k, T alpha, const T *A, int lda,
                      const T *B, int ldb, T beta, T *C, int ldc, cudaStream_t st, unsigned *err,
                      void *ws, size_t ws_bytes) {
  const bool an = notrans(ta), bn = notrans(tb);
  const int arows = an ? m : k, brows = bn ? k : n;
  if (m < 0 || n < 0 || k < 0 || lda < (arows > 1 ? arows : 1) ||
      ldb < (brows > 1 ? brows : 1) || ldc < (m > 1 ? m : 1))
    return GB300_ERR_ARG;
  if (m == 0 || n == 0) return GB300_OK;
  if (alpha == T(0) || k == 0) {
    if (alpha == T(0) && beta == T(1)) return GB300_OK;
    // alpha == 0: beta scaling only (src/gemm_driver.c:133-134); k == 0: the
    // reference still adds an empty (zero) sum.
    const T add = (alpha == T(0)) ? T(-0.0) : T(0);  // -0.0 leaves beta*C untouched
    const int64_t total = (int64_t)m * n;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    scale_c_kernel<T><<<blocks, 256, 0, st>>>(m, n, beta, add, C, ldc);
    return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
  }
  // Operand A: N -> stored m x k (MN-major tile), T -> stored k x m (K-major tile).
  OperandDesc oA, oB;
  make_desc(oA, A, lda, an ? m : k, an ? k : m);
  make_desc(oB, B, ldb, bn ? k : n, bn ? n : k);
  constexpr int BK = PlainTraits<T>::BK;
  CUtensorMap tA{}, tB{};
  bool tma = tma_ok(A, lda, sizeof(T)) && tma_ok(B, ldb, sizeof(T));
  if (tma) {
    // K-major operands use the 128-byte swizzle (box inner = BK elements = 128 B).
    tma = encode_2d(&tA, A, sizeof(T), oA.rows, oA.cols, lda, an ? kBM : BK, an ? BK : kBM,
                    /*swizzle128=*/!an) &&
          encode_2d(&tB, B, sizeof(T), oB.rows, oB.cols, ldb, bn ? BK : kBN, bn ? kBN : BK,
                    /*swizzle128=*/bn);
  }
  // split-K where the caller gave room for its slices (else one slice)
  const int dbl = sizeof(T) == 8 ? 1 : 0;
  int S = plain_split_k(dbl, m, n, k);
  if (S > 1 && (!ws || ws_bytes < (size_t)S * m * n * sizeof(T))) S = 1;
  T *part = static_cast<T *>(ws);
  const int ST = plain_stages_for(dbl, m, n, k);
  const bool AK = !an, BKm = bn;
  if (!AK && !BKm)
    return launch_depth<T, false, false>(ST, tA, tB, oA, oB, tma, m, n, k, alpha, beta, C, ldc,
                                         S, part, st, err);
  if (!AK && BKm)
    return launch_depth<T, false, true>(ST, tA, tB, oA, oB, tma, m, n, k, alpha, beta, C, ldc,
                                        S, part, st, err);
  if (AK && !BKm)
    return launch_depth<T, true, false>(ST, tA, tB, oA, oB, tma, m, n, k, alpha, beta, C, ldc,
                                        S, part, st, err);
  return launch_depth<T, true, true>(ST, tA, tB, oA, oB, tma, m, n, k, alpha, beta, C, ldc, S,
                                     part, st, err);
}

int plain_dgemm(char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
                const double *B, int ldb, double beta, double *C, int ldc, cudaStream_t st,
                unsigned *err, void *ws, size_t ws_bytes) {
  return plain_gemm<double>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, st, err, ws,
                            ws_bytes);
}
int plain_sgemm(char ta, char tb, int m, int n, int k, float alpha, const float *A, int lda,
                const float *B, int ldb, float beta, float *C, int ldc, cudaStream_t st,
                unsigned *err, void *ws, size_t ws_bytes) {
  return plain_gemm<float>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, st, err, ws,
                           ws_bytes);
}

}  // namespace gb300
