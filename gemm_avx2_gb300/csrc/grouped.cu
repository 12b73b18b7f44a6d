// grouped.cu -- many independent GEMMs of uneven sizes, mixed FP64/FP32 and
// any transposes, in ONE persistent launch with a device-side tile scheduler,
// plus CUDA-graph capture/replay of a fixed batch.
//
// The reference computes one problem per dgemm_/sgemm_ call (wjc404/GEMM_AVX2
// src/gemm_driver.c:118) and splits a call's N columns statically over its
// OpenMP team (src/gemm_driver.c:138); it has no batched form.  Here the
// 128 x 128 tiles of all problems are concatenated, ordered by the host
// longest-work-first (an FP64 tile is ~40x an FP32 tile of the same K on GB300),
// and each persistent CTA takes the next tile from a global atomic counter.
// The tile code is the plain kernels' (plain_tiles.cuh): FFMA 8x8 register
// tiles for FP32, m16n8k8 DMMA warp tiles for FP64, a 4-stage shared-memory
// ring filled by TMA (per-problem tensor maps in global memory) or, for a
// problem whose leading dimensions / base addresses break TMA's 16-byte rules,
// by cp.async element copies.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "common.cuh"
#include "plain_gemm.h"
#include "plain_tiles.cuh"
#include "split_gemm.h"

namespace gb300 {

enum : int { kGDouble = 1, kGAK = 2, kGBK = 4, kGTma = 8 };

struct GroupedProblemDev {
  const void *A, *B;
  void *C;
  int lda, ldb, ldc, m, n, k;
  int tiles_m, tiles_n;
  int flags;
  int a_rows, a_cols, b_rows, b_cols;
  double alpha, beta;
};

constexpr int kGThreads = kConsumerWarps * 32;  // 256: every warp computes
constexpr int kGSmem = kStages * 2 * (kBM * 32 * 4) + 1024 + 256;

// Each stage has two "full" barriers: full[s] (expected count 1, TMA
// transactions) for problems loaded by TMA, fullc[s] (expected count 256, one
// cp.async completion arrival per thread) for problems on the cp.async path.
// Every thread tracks the next phase parity of each with a bit mask (bit s),
// so consecutive problems may use either path without any CTA-wide barrier.
struct GPhase {
  uint32_t tma = 0, cp = 0;
};

// Fill k-tile `kt` of the current tile into stage (it + kt) % kStages.
template <typename T, bool AK, bool BK_>
__device__ __forceinline__ bool g_fill(const GroupedProblemDev &p, const CUtensorMap *tmA,
                                       const CUtensorMap *tmB, bool tma, int m0, int n0, int kt,
                                       uint32_t it, T *sA, T *sB, uint64_t *full, uint64_t *fullc,
                                       uint64_t *empty, unsigned *err, volatile int *abort_flag) {
  constexpr int BK = PlainTraits<T>::BK;
  const uint32_t g = it + kt;
  const int s = g % kStages;
  T *ta = sA + s * (kBM * BK);
  T *tb = sB + s * (kBN * BK);
  const int k0 = kt * BK;
  if (tma) {
    if (threadIdx.x == 0) {
      if (g >= (uint32_t)kStages &&
          !mbar_wait(&empty[s], ((g / kStages) - 1) & 1, err, kErrTimeoutEmpty, abort_flag))
        return false;
      mbar_arrive_expect_tx(&full[s], 2 * tile_bytes<T>());
      if (AK) tma_load_2d(ta, tmA, k0, m0, &full[s]);
      else    tma_load_2d(ta, tmA, m0, k0, &full[s]);
      if (BK_) tma_load_2d(tb, tmB, k0, n0, &full[s]);
      else     tma_load_2d(tb, tmB, n0, k0, &full[s]);
    }
    return true;
  }
  if (g >= (uint32_t)kStages &&
      !mbar_wait(&empty[s], ((g / kStages) - 1) & 1, err, kErrTimeoutEmpty, abort_flag))
    return false;
  const T *baseA = static_cast<const T *>(p.A);
  const T *baseB = static_cast<const T *>(p.B);
  for (int e = threadIdx.x; e < kBM * BK; e += kGThreads) {
    int mn, kk;
    if (AK) { mn = e / BK; kk = e % BK; } else { kk = e / kBM; mn = e % kBM; }
    const int r = AK ? (k0 + kk) : (m0 + mn), c = AK ? (m0 + mn) : (k0 + kk);
    const bool ok = r < p.a_rows && c < p.a_cols;
    const T *src = ok ? baseA + (int64_t)c * p.lda + r : baseA;
    if (sizeof(T) == 4) cp_async_4(ta + tile_off<T, AK>(mn, kk), src, ok);
    else                cp_async_8(ta + tile_off<T, AK>(mn, kk), src, ok);
  }
  for (int e = threadIdx.x; e < kBN * BK; e += kGThreads) {
    int mn, kk;
    if (BK_) { mn = e / BK; kk = e % BK; } else { kk = e / kBN; mn = e % kBN; }
    const int r = BK_ ? (k0 + kk) : (n0 + mn), c = BK_ ? (n0 + mn) : (k0 + kk);
    const bool ok = r < p.b_rows && c < p.b_cols;
    const T *src = ok ? baseB + (int64_t)c * p.ldb + r : baseB;
    if (sizeof(T) == 4) cp_async_4(tb + tile_off<T, BK_>(mn, kk), src, ok);
    else                cp_async_8(tb + tile_off<T, BK_>(mn, kk), src, ok);
  }
  cp_async_mbar_arrive(&fullc[s]);
  return true;
}

// Wait for stage s of the current problem's path and advance that barrier's parity.
__device__ __forceinline__ bool g_wait_full(bool tma, int s, uint64_t *full, uint64_t *fullc,
                                            GPhase &ph, unsigned *err, volatile int *abort_flag) {
  uint32_t &bits = tma ? ph.tma : ph.cp;
  const bool ok = mbar_wait(tma ? &full[s] : &fullc[s], (bits >> s) & 1u, err, kErrTimeoutFull,
                            abort_flag);
  bits ^= (1u << s);
  return ok;
}

// One 128 x 128 tile of one problem.  `it` counts the k-tiles this CTA has
// consumed so far (the ring's phase state carries across tiles).
template <typename T, bool AK, bool BK_>
__device__ void g_tile(const GroupedProblemDev &p, const CUtensorMap *tmA, const CUtensorMap *tmB,
                       int tmi, int tni, uint8_t *smem, uint64_t *full, uint64_t *fullc,
                       uint64_t *empty, uint32_t &it, GPhase &ph, unsigned *err,
                       volatile int *abort_flag, bool &ok) {
  constexpr int BK = PlainTraits<T>::BK;
  T *sA = reinterpret_cast<T *>(smem);
  T *sB = sA + kStages * kBM * BK;
  const bool tma = (p.flags & kGTma) != 0;
  const int m0 = tmi * kBM, n0 = tni * kBN;
  const int ktiles = (p.k + BK - 1) / BK;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  for (int kt = 0; kt < kStages - 1 && kt < ktiles && ok; ++kt)
    ok = g_fill<T, AK, BK_>(p, tmA, tmB, tma, m0, n0, kt, it, sA, sB, full, fullc, empty, err,
                            abort_flag);

  if constexpr (sizeof(T) == 4) {
    const int wm = warp & 1, wn = warp >> 1;
    const int tm = wm * 8 + (lane & 7), tn = wn * 4 + (lane >> 3);
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
    for (int kt = 0; kt < ktiles && ok; ++kt) {
      if (kt + kStages - 1 < ktiles)
        ok = g_fill<T, AK, BK_>(p, tmA, tmB, tma, m0, n0, kt + kStages - 1, it, sA, sB, full,
                                fullc, empty, err, abort_flag);
      const uint32_t g = it + kt;
      const int s = g % kStages;
      if (!ok || !g_wait_full(tma, s, full, fullc, ph, err, abort_flag)) {
        ok = false;
        break;
      }
      const float *ta = reinterpret_cast<const float *>(sA) + s * (kBM * BK);
      const float *tb = reinterpret_cast<const float *>(sB) + s * (kBN * BK);
#pragma unroll 2
      for (int kq = 0; kq < BK / 4; ++kq) {
        float a[8][4], b[8][4];
        f32_load_frag<AK>(ta, tm, kq, a);
        f32_load_frag<BK_>(tb, tn, kq, b);
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i][q], b[j][q], acc[i][j]);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
    }
    if (!ok) return;
    const float alpha = (float)p.alpha, beta = (float)p.beta;
    float *C = static_cast<float *>(p.C);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int col = n0 + f32_row<BK_>(tn, j);
      if (col >= p.n) continue;
      float *cc = C + (int64_t)col * p.ldc;
      float cv[8];  // the column's 8 loads first, then the stores
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int row = m0 + f32_row<AK>(tm, i);
        cv[i] = (row < p.m) ? cc[row] : 0.f;
      }
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int row = m0 + f32_row<AK>(tm, i);
        if (row < p.m) {
          float v = (beta == 1.0f) ? cv[i] : cv[i] * beta;
          if (alpha != 0.0f) v = v + alpha * acc[i][j];
          cc[row] = v;
        }
      }
    }
  } else {
    const int wm = warp & 1, wn = warp >> 1;
    const int g8 = lane >> 2, t4 = lane & 3;
    double acc[4][4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.0;
    for (int kt = 0; kt < ktiles && ok; ++kt) {
      if (kt + kStages - 1 < ktiles)
        ok = g_fill<T, AK, BK_>(p, tmA, tmB, tma, m0, n0, kt + kStages - 1, it, sA, sB, full,
                                fullc, empty, err, abort_flag);
      const uint32_t g = it + kt;
      const int s = g % kStages;
      if (!ok || !g_wait_full(tma, s, full, fullc, ph, err, abort_flag)) {
        ok = false;
        break;
      }
      const double *ta = reinterpret_cast<const double *>(sA) + s * (kBM * BK);
      const double *tb = reinterpret_cast<const double *>(sB) + s * (kBN * BK);
#pragma unroll
      for (int k8 = 0; k8 < BK; k8 += 8) {
        double a[4][4], b[4][2];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int mb = wm * 64 + i * 16;
#pragma unroll
          for (int r = 0; r < 4; ++r)
            a[i][r] = ta[tile_off<double, AK>(mb + g8 + 8 * (r & 1), k8 + t4 + 4 * (r >> 1))];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int nb = wn * 32 + j * 8;
#pragma unroll
          for (int r = 0; r < 2; ++r) b[j][r] = tb[tile_off<double, BK_>(nb + g8, k8 + t4 + 4 * r)];
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
    double *C = static_cast<double *>(p.C);
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int cj = 0; cj < 2; ++cj) {
        const int col = n0 + wn * 32 + j * 8 + 2 * t4 + cj;
        if (col >= p.n) continue;
        double *cc = C + (int64_t)col * p.ldc;
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int ri = 0; ri < 2; ++ri) {
            const int row = m0 + wm * 64 + i * 16 + g8 + 8 * ri;
            if (row < p.m) {
              const double c0 = cc[row];
              double v = (p.beta == 1.0) ? c0 : c0 * p.beta;
              if (p.alpha != 0.0) v = v + p.alpha * acc[i][j][2 * ri + cj];
              cc[row] = v;
            }
          }
      }
  }
  it += ktiles;
}

__global__ void __launch_bounds__(kGThreads, 1)
grouped_plain_kernel(const GroupedProblemDev *__restrict__ probs, const CUtensorMap *maps,
                     const int *__restrict__ tile_off, int count, int total_tiles, int *counter,
                     unsigned *err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                              ~uintptr_t(1023));
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + kStages * 2 * (kBM * 32 * 4));
  uint64_t *fullc = full + kStages;
  uint64_t *empty = fullc + kStages;
  volatile int *abort_flag = reinterpret_cast<volatile int *>(empty + kStages);
  __shared__ int s_tile;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&fullc[s], kGThreads);
      mbar_init(&empty[s], kConsumerWarps);
    }
    *abort_flag = 0;
    fence_barrier_init();
  }
  __syncthreads();
  uint32_t it = 0;
  GPhase ph;
  bool ok = true;
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1);
    __syncthreads();
    const int t = s_tile;
    __syncthreads();
    if (t >= total_tiles || *abort_flag) break;
    // the problem owning tile t: the last p with tile_off[p] <= t
    int lo = 0, hi = count - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tile_off[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const GroupedProblemDev &p = probs[lo];
    const int local = t - tile_off[lo];
    const int tmi = local % p.tiles_m, tni = local / p.tiles_m;
    const CUtensorMap *tA = maps + 2 * lo, *tB = maps + 2 * lo + 1;
    switch (p.flags & (kGDouble | kGAK | kGBK)) {
      case 0:                         g_tile<float, false, false>(p, tA, tB, tmi, tni, smem, full, fullc, empty, it, ph, err, abort_flag, ok); break;
      case kGBK:                      g_tile<float, false, true >(p, tA, tB, tmi, tni, smem, full, fullc, empty, it, ph, err, abort_flag, ok); break;
      case kGAK:                      g_tile<float, true,  false>(p, tA, tB, tmi, tni, smem, full, fullc, empty, it, ph, err, abort_flag, ok); break;
      case kGAK | kGBK:               g_tile<float, true,  true >(p, tA, tB, tmi, tni, smem, full, fullc, empty, it, ph, err, abort_flag, ok); break;
      case kGDouble:                  g_tile<double, false, false>(p, tA, tB, tmi, tni, smem, full, fullc, empty, it, ph, err, abort_flag, ok); break;
      case kGDouble | kGBK:           g_tile<double, false, true >(p, tA, tB, tmi, tni, smem, full, fullc, empty, it, ph, err, abort_flag, ok); break;
      case kGDouble | kGAK:           g_tile<double, true,  false>(p, tA, tB, tmi, tni, smem, full, fullc, empty, it, ph, err, abort_flag, ok); break;
      default:                        g_tile<double, true,  true >(p, tA, tB, tmi, tni, smem, full, fullc, empty, it, ph, err, abort_flag, ok); break;
    }
    if (!ok) break;
  }
}

// ===========================================================================
// host side
// ===========================================================================
static inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Metadata blob layout (one device buffer, uploaded with one copy):
//   [0, 256)             scheduler counter (int), zero at upload
//   [256, +256*count)    2 CUtensorMap per problem (A, B), 64-byte aligned
//   [.., +sizeof*count)  GroupedProblemDev per problem (tile order)
//   [.., +4*(count+1))   tile offsets (prefix sums of tiles per problem)
struct BlobLayout {
  size_t maps, probs, offs, total;
};
static BlobLayout blob_layout(int count) {
  BlobLayout L;
  L.maps = 256;
  L.probs = align_up(L.maps + sizeof(CUtensorMap) * 2 * (size_t)count, 256);
  L.offs = align_up(L.probs + sizeof(GroupedProblemDev) * (size_t)count, 256);
  L.total = align_up(L.offs + sizeof(int) * ((size_t)count + 1), 256);
  return L;
}

size_t grouped_workspace_bytes(int count) {
  return count <= 0 ? 0 : blob_layout(count).total + 256;
}

static int validate_problem(const gb300_gemm_problem &q) {
  if (q.precision != 'd' && q.precision != 's') return GB300_ERR_ARG;
  return check_args(q.transa, q.transb, q.m, q.n, q.k, q.lda, q.ldb, q.ldc);
}

// Build the metadata blob (host image) for the problems that need work.
// Returns GB300_OK and sets count_used / total_tiles.
int grouped_build(const gb300_gemm_problem *P, int count, void *dev_base,
                  std::vector<uint8_t> &blob, int &count_used, int &total_tiles) {
  std::vector<int> idx;
  for (int i = 0; i < count; ++i) {
    const int rc = validate_problem(P[i]);
    if (rc == GB300_ERR_ARG) return rc;
    if (rc < 0) continue;                                   // m or n == 0
    if (P[i].alpha == 0.0 && P[i].beta == 1.0) continue;     // C unchanged
    idx.push_back(i);
  }
  // longest work per tile first: K tiles x (an FP64 tile is ~40x an FP32 one)
  auto cost = [&](int i) {
    const gb300_gemm_problem &q = P[i];
    const double kt = q.precision == 'd' ? (q.k + 15) / 16 : (q.k + 31) / 32;
    return kt * (q.precision == 'd' ? 80.0 : 1.0);
  };
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return cost(a) > cost(b); });
  count_used = (int)idx.size();
  const BlobLayout L = blob_layout(count_used > 0 ? count_used : 1);
  blob.assign(L.total, 0);
  CUtensorMap *maps = reinterpret_cast<CUtensorMap *>(blob.data() + L.maps);
  GroupedProblemDev *probs = reinterpret_cast<GroupedProblemDev *>(blob.data() + L.probs);
  int *offs = reinterpret_cast<int *>(blob.data() + L.offs);
  int64_t tiles = 0;
  for (int j = 0; j < count_used; ++j) {
    const gb300_gemm_problem &q = P[idx[j]];
    const bool dbl = q.precision == 'd';
    const bool an = notrans(q.transa), bn = notrans(q.transb);
    GroupedProblemDev &g = probs[j];
    g.A = q.A; g.B = q.B; g.C = q.C;
    g.lda = q.lda; g.ldb = q.ldb; g.ldc = q.ldc;
    g.m = q.m; g.n = q.n; g.k = (q.alpha == 0.0) ? 0 : q.k;
    g.tiles_m = (q.m + kBM - 1) / kBM;
    g.tiles_n = (q.n + kBN - 1) / kBN;
    g.a_rows = an ? q.m : q.k; g.a_cols = an ? q.k : q.m;
    g.b_rows = bn ? q.k : q.n; g.b_cols = bn ? q.n : q.k;
    g.alpha = q.alpha; g.beta = q.beta;
    g.flags = (dbl ? kGDouble : 0) | (an ? 0 : kGAK) | (bn ? kGBK : 0);
    const size_t esz = dbl ? 8 : 4;
    const int BK = dbl ? 16 : 32;
    bool tma = g.k > 0 && tma_ok(q.A, q.lda, esz) && tma_ok(q.B, q.ldb, esz);
    if (tma)
      tma = encode_2d(&maps[2 * j], q.A, esz, g.a_rows, g.a_cols, q.lda, an ? kBM : BK,
                      an ? BK : kBM, !an) &&
            encode_2d(&maps[2 * j + 1], q.B, esz, g.b_rows, g.b_cols, q.ldb, bn ? BK : kBN,
                      bn ? kBN : BK, bn);
    if (tma) g.flags |= kGTma;
    offs[j] = (int)tiles;
    tiles += (int64_t)g.tiles_m * g.tiles_n;
    if (tiles > 0x7fffffff) return GB300_ERR_ARG;
  }
  offs[count_used] = (int)tiles;
  total_tiles = (int)tiles;
  (void)dev_base;
  return GB300_OK;
}

static int sms() {
  int d = 0, n = 0;
  cudaGetDevice(&d);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, d);
  return n > 0 ? n : 148;
}

// Launch the persistent kernel on a metadata blob already in device memory.
int grouped_launch_blob(void *dev_blob, int count_used, int total_tiles, cudaStream_t st,
                        unsigned *err) {
  if (count_used == 0 || total_tiles == 0) return GB300_OK;
  const BlobLayout L = blob_layout(count_used);
  uint8_t *base = static_cast<uint8_t *>(dev_blob);
  if (cudaFuncSetAttribute(grouped_plain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kGSmem) != cudaSuccess)
    return GB300_ERR_CUDA;
  const int grid = total_tiles < sms() ? total_tiles : sms();
  grouped_plain_kernel<<<grid, kGThreads, kGSmem, st>>>(
      reinterpret_cast<const GroupedProblemDev *>(base + L.probs),
      reinterpret_cast<const CUtensorMap *>(base + L.maps),
      reinterpret_cast<const int *>(base + L.offs), count_used, total_tiles,
      reinterpret_cast<int *>(base), err);
  return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
}

size_t grouped_blob_bytes(int count_used) { return blob_layout(count_used > 0 ? count_used : 1).total; }

int grouped_plain(const gb300_gemm_problem *P, int count, void *ws, size_t ws_bytes,
                  cudaStream_t st, unsigned *err) {
  if (count < 0 || (count > 0 && !P)) return GB300_ERR_ARG;
  if (count == 0) return GB300_OK;
  std::vector<uint8_t> blob;
  int used = 0, tiles = 0;
  const int rc = grouped_build(P, count, ws, blob, used, tiles);
  if (rc != GB300_OK) return rc;
  if (used == 0) return GB300_OK;
  if (!ws || ws_bytes < blob.size() + 256) return GB300_ERR_WORKSPACE;
  void *base = reinterpret_cast<void *>((reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
  // pageable source: the copy has consumed `blob` when cudaMemcpyAsync returns
  if (cudaMemcpyAsync(base, blob.data(), blob.size(), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return GB300_ERR_CUDA;
  return grouped_launch_blob(base, used, tiles, st, err);
}

}  // namespace gb300
