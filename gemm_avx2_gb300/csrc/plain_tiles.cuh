// plain_tiles.cuh -- tile geometry, shared-memory layouts and register
// micro-kernels of the plain FP32/FP64 GEMMs, shared by the single-problem
// kernels (plain_gemm.cu) and the grouped persistent kernel (grouped.cu).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"

namespace gb300 {

constexpr int kBM = 128, kBN = 128, kStages = 4;
constexpr int kConsumerWarps = 8;
constexpr int kThreads = (kConsumerWarps + 1) * 32;  // + 1 producer warp

template <typename T>
struct PlainTraits;
template <>
struct PlainTraits<float> {
  static constexpr int BK = 32;  // 128-byte rows for the K-major swizzled layout
};
template <>
struct PlainTraits<double> {
  static constexpr int BK = 16;
};

template <typename T>
__host__ __device__ constexpr int tile_bytes() {
  return kBM * PlainTraits<T>::BK * (int)sizeof(T);
}
// ST: ring depth (stages) of the single-problem kernels (kStages by default;
// the tuned depth of the shape class otherwise).
template <typename T, int ST = kStages>
__host__ __device__ constexpr int plain_smem_bytes() {
  return ST * 2 * tile_bytes<T>() + 1024 /*alignment slack*/ + 256 /*barriers*/;
}

constexpr int kGroupM = 16;

// Offset (in elements) of logical (mn, k) inside one stage tile.
//   MN-major tile: [BK][128] (mn contiguous), no swizzle.
//   K-major tile : [128][BK] rows of 128 bytes, 128-byte swizzle: the 16-byte
//                  chunk c of row r lives at chunk c ^ (r & 7).
template <typename T, bool KMAJ>
__device__ __forceinline__ int tile_off(int mn, int k) {
  constexpr int BK = PlainTraits<T>::BK;
  constexpr int EPC = 16 / (int)sizeof(T);  // elements per 16-byte chunk
  if (KMAJ) {
    const int chunk = (k / EPC) ^ (mn & 7);
    return mn * BK + chunk * EPC + (k % EPC);
  } else {
    return k * kBM + mn;
  }
}

// ---------------------------------------------------------------------------
// producer: fill one stage
// ---------------------------------------------------------------------------
struct OperandDesc {
  const void *ptr;  // base of the stored matrix (column-major, ld)
  int ld;
  int rows, cols;   // stored shape
};

// cp.async fallback: every lane copies a strided share of the tile's elements.
// Out-of-range elements are zero-filled (src-size 0), mirroring TMA's OOB fill.
template <typename T, bool KMAJ>
__device__ __forceinline__ void fallback_fill(T *tile, const OperandDesc &op, int mn0, int k0,
                                              int lane) {
  constexpr int BK = PlainTraits<T>::BK;
  const T *base = static_cast<const T *>(op.ptr);
  // stored (row, col): MN-major operand stores mn along rows; K-major stores k along rows.
  for (int e = lane; e < kBM * BK; e += 32) {
    int mn, k;
    if (KMAJ) { mn = e / BK; k = e % BK; } else { k = e / kBM; mn = e % kBM; }
    const int r = KMAJ ? (k0 + k) : (mn0 + mn);
    const int c = KMAJ ? (mn0 + mn) : (k0 + k);
    const bool ok = (r < op.rows) && (c < op.cols);
    const T *src = ok ? base + (int64_t)c * op.ld + r : base;
    if (sizeof(T) == 4)
      cp_async_4(tile + tile_off<T, KMAJ>(mn, k), src, ok);
    else
      cp_async_8(tile + tile_off<T, KMAJ>(mn, k), src, ok);
  }
}

// Fills k-tiles kt0 .. kt0 + ktiles - 1 (a K slice) into an ST-deep ring.
template <typename T, bool AK, bool BK_, int ST>
__device__ __forceinline__ void producer_loop(const CUtensorMap *tmA, const CUtensorMap *tmB,
                                              const OperandDesc &opA, const OperandDesc &opB,
                                              bool use_tma, T *sA, T *sB, uint64_t *full,
                                              uint64_t *empty, int m0, int n0, int kt0,
                                              int ktiles, unsigned *err,
                                              volatile int *abort_flag) {
  constexpr int BK = PlainTraits<T>::BK;
  const int lane = threadIdx.x & 31;
  for (int kt = 0; kt < ktiles; ++kt) {
    const int s = kt % ST;
    if (kt >= ST) {
      if (!mbar_wait(&empty[s], ((kt / ST) - 1) & 1, err, kErrTimeoutEmpty, abort_flag)) return;
    }
    T *ta = sA + s * (kBM * BK);
    T *tb = sB + s * (kBN * BK);
    const int k0 = (kt0 + kt) * BK;
    if (use_tma) {
      if (lane == 0) {
        mbar_arrive_expect_tx(&full[s], 2 * tile_bytes<T>());
        // A: MN-major -> box (m, k) at (m0, k0); K-major -> box (k, m) at (k0, m0)
        if (AK) tma_load_2d(ta, tmA, k0, m0, &full[s]);
        else    tma_load_2d(ta, tmA, m0, k0, &full[s]);
        if (BK_) tma_load_2d(tb, tmB, k0, n0, &full[s]);
        else     tma_load_2d(tb, tmB, n0, k0, &full[s]);
      }
    } else {
      fallback_fill<T, AK>(ta, opA, m0, k0, lane);
      fallback_fill<T, BK_>(tb, opB, n0, k0, lane);
      cp_async_mbar_arrive(&full[s]);
    }
  }
}

// ---------------------------------------------------------------------------
// FP32 consumer: 8x8 register tile per thread (FFMA)
// ---------------------------------------------------------------------------
template <bool KMAJ>
__device__ __forceinline__ int f32_row(int t, int i) {
  // K-major tiles interleave rows (t + 16 i) so that a warp's eight distinct t
  // hit eight different swizzle chunks; MN-major tiles use two 4-wide runs.
  return KMAJ ? (t + 16 * i) : ((i < 4) ? (4 * t + i) : (64 + 4 * t + (i - 4)));
}

template <bool KMAJ>
__device__ __forceinline__ void f32_load_frag(const float *tile, int t, int kq, float (&f)[8][4]) {
  if (KMAJ) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = t + 16 * i;
      const float4 v = *reinterpret_cast<const float4 *>(tile + r * 32 + ((kq ^ (r & 7)) << 2));
      f[i][0] = v.x; f[i][1] = v.y; f[i][2] = v.z; f[i][3] = v.w;
    }
  } else {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float *row = tile + (4 * kq + q) * kBM;
      const float4 v0 = *reinterpret_cast<const float4 *>(row + 4 * t);
      const float4 v1 = *reinterpret_cast<const float4 *>(row + 64 + 4 * t);
      f[0][q] = v0.x; f[1][q] = v0.y; f[2][q] = v0.z; f[3][q] = v0.w;
      f[4][q] = v1.x; f[5][q] = v1.y; f[6][q] = v1.z; f[7][q] = v1.w;
    }
  }
}

// ---------------------------------------------------------------------------
// FP64 micro-kernel: one m16n8k8 DMMA
// ---------------------------------------------------------------------------
__device__ __forceinline__ void dmma_16x8x8(double (&c)[4], const double (&a)[4],
                                            const double (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+d"(c[0]), "+d"(c[1]), "+d"(c[2]), "+d"(c[3])
      : "d"(a[0]), "d"(a[1]), "d"(a[2]), "d"(a[3]), "d"(b[0]), "d"(b[1]));
}

}  // namespace gb300
