// tc_gemm.cu -- tensor-core (tcgen05, sm_103a) split-precision forms of the
// reference's sgemm_/dgemm_ (wjc404/GEMM_AVX2 src/gemm_driver.c:118; same
// operand semantics, no reference kernel counterpart).
//
//  * BF16xP SGEMM: op(A), op(B) are split into BF16 terms by a split kernel that
//    also absorbs the transposes and writes K-major operands (the role of the
//    reference's packing, src/gemm_copy.c).  The P cross products are laid
//    side by side along K, so one BF16 GEMM with FP32 accumulation in TMEM over
//    K' = P * K computes their sum.
//  * Ozaki DGEMM: rows of op(A) / columns of op(B) are scaled by powers of two
//    and cut into S slices of signed 7-bit integers (|d| <= 127, int8 range).
//    tcgen05 on sm_103a has no kind::i8, so the integer slices ride the BF16
//    pipe: each slice value is exact in BF16, each product (< 2^14) exact in
//    FP32, and every accumulation chunk is capped at 1024 K-steps so partial sums
//    stay below 1024*127^2 < 2^24 -- integer-valued FP32 is then exact.  The epilogue warps
//    drain each chunk from TMEM into 32-bit integer sums (exact), and fold each
//    slice group t = i + j into an FP64 result scratch with weight 2^-7t.  The
//    same kernel runs the CRT form (crt.cu): one residue pair per modulus,
//    sums reduced mod p and stored instead of folded.
//
// Both GEMMs are persistent, warp-specialised kernels: warp 0 issues TMA loads
// into a shared-memory ring, warp 1 allocates TMEM and issues tcgen05.mma from
// one thread, the remaining warps run the epilogue from TMEM.  Two TMEM
// accumulators let the epilogue of one tile/chunk overlap the next one's MMAs.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "common.cuh"
#include "plain_gemm.h"
#include "split_gemm.h"
#include "split_tiles.cuh"

namespace gb300 {

static_assert(kFp16x3 == GB300_SPLIT_FP16X3, "products code of the scaled FP16 form");

static inline int64_t round_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }
// grid.y of the split / slice kernels: the 32-row blocks of Rp, capped at the
// grid limit (the kernels stride over the rest).
static inline unsigned row_blocks(int64_t Rp) { return (unsigned)(Rp / 32 < 65535 ? Rp / 32 : 65535); }
constexpr int kSplitGroupM = 16;

// ===========================================================================
// split kernels: read op(X) (R x K view of a column-major matrix) in 32 x 64
// tiles through shared memory so that both the read and the K-major write
// are coalesced whatever the transpose.
// ===========================================================================
// term[] of x: t0 = bf16(x), t1 = bf16(x - t0), t2 = bf16(x - t0 - t1); every
// residual is exact in FP32.
__device__ __forceinline__ void bf16_terms(float x, int nterms, __nv_bfloat16 (&t)[3]) {
  float r = x;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (i < nterms) {
      t[i] = __float2bfloat16_rn(r);
      r = r - __bfloat162float(t[i]);
    } else {
      t[i] = __float2bfloat16_rn(0.f);
    }
  }
}

// The product stream of the split GEMM: segment s multiplies term term[s] of
// op(A) with term term[s] of op(B) (each operand's map), over K.
struct SegMap {
  int nseg;
  int term[6];
};

// Scaled FP16 terms of one value of a row with scale exponent E (max |x| of
// the row in [2^(E-1), 2^E)): y = x * 2^(15-E) lies in (-2^15, 2^15); hi =
// fp16(y), lo = fp16((y - hi) * 2^11).  The residual y - hi is exact in FP32;
// scaling up by 2^(15-E) is exact, scaling down (E > 15) only rounds values
// below 2^-126, far under what hi and lo keep.  Returns (hi, lo) as bit patterns.
__device__ __forceinline__ void f16_terms(float x, int s, unsigned short &hi, unsigned short &lo) {
  const float y = s > 127 ? (x * pow2f(127)) * pow2f(s - 127) : x * pow2f(s);
  const __half h = __float2half_rn(y);
  const __half l = __float2half_rn((y - __half2float(h)) * 2048.0f);
  hi = __half_as_ushort(h);
  lo = __half_as_ushort(l);
}

// Both operands of one split in a single launch (blockIdx.z = 0: op(A),
// 1: op(B) read as its n x k transpose).
struct SplitArgs {
  const float *X0, *X1;
  int ld0, ld1, R0, R1, kc0, kc1, Rp0, Rp1;
  const int *ex0, *ex1;
  __nv_bfloat16 *out0, *out1;
  int K, Kp, nterms;
  int64_t ldo;
  int zbase;  // operand of blockIdx.z = 0 (1: a launch over op(B) alone)
};

// out: Rp x (nterms * Kp) row-major 16-bit terms, term t in columns
// [t Kp, (t + 1) Kp) (row stride ldo = nterms * Kp elements); grid.y strides
// over the 32-row blocks that hold rows of op(X) (rows past R are left
// unwritten: the GEMM's maps end there; columns [K, Kp) are written as
// zeros).  Each thread writes 8 consecutive k of one row (16 bytes) per term.
//   F16 = false: BF16 terms t0 = bf16(x), t1 = bf16(x - t0), t2 (nterms of them).
//   F16 = true : the scaled FP16 (hi, lo) of f16_terms with the row exponents
//                ex[] (Rp entries); a row whose max is not finite is all NaN.
template <bool F16>
__global__ void __launch_bounds__(256) split_bf16_kernel(const __grid_constant__ SplitArgs p) {
  const int z = blockIdx.z + p.zbase;
  const float *__restrict__ X = z ? p.X1 : p.X0;
  const int ld = z ? p.ld1 : p.ld0, R = z ? p.R1 : p.R0, kcontig = z ? p.kc1 : p.kc0;
  const int K = p.K, Kp = p.Kp, nterms = p.nterms;
  const int *__restrict__ ex = z ? p.ex1 : p.ex0;
  __nv_bfloat16 *__restrict__ out = z ? p.out1 : p.out0;
  const int64_t ldo = p.ldo;
  __shared__ float tile[32][65];
  const int k0 = blockIdx.x * 64;
  const int r = threadIdx.x >> 3, kq = (threadIdx.x & 7) * 8;
  // rows past R are never read (the GEMM's maps end at the problem's rows),
  // so only row blocks holding data are written
  for (int r0 = blockIdx.y * 32; r0 < R; r0 += gridDim.y * 32) {
    load_tile_32x64<float>(X, ld, R, K, kcontig != 0, r0, k0, tile);
    __syncthreads();
    unsigned w[3][4];  // term t of the 8 values, packed in pairs
    if (F16) {
      const int e = ex[r0 + r];
      if (e == kNonFiniteExp) {
#pragma unroll
        for (int t = 0; t < 3; ++t)
#pragma unroll
          for (int q = 0; q < 4; ++q) w[t][q] = 0x7e007e00u;
      } else {
        const int sc = 15 - e;
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
          unsigned short h0, l0, h1, l1;
          f16_terms(tile[r][kq + j], sc, h0, l0);
          f16_terms(tile[r][kq + j + 1], sc, h1, l1);
          w[0][j / 2] = (unsigned)h0 | ((unsigned)h1 << 16);
          w[1][j / 2] = (unsigned)l0 | ((unsigned)l1 << 16);
          w[2][j / 2] = 0u;
        }
      }
    } else {
#pragma unroll
      for (int j = 0; j < 8; j += 2) {
        __nv_bfloat16 t0[3], t1[3];
        bf16_terms(tile[r][kq + j], nterms, t0);
        bf16_terms(tile[r][kq + j + 1], nterms, t1);
#pragma unroll
        for (int t = 0; t < 3; ++t)
          w[t][j / 2] = (unsigned)__bfloat16_as_ushort(t0[t]) |
                        ((unsigned)__bfloat16_as_ushort(t1[t]) << 16);
      }
    }
    __nv_bfloat16 *row = out + (int64_t)(r0 + r) * ldo + k0 + kq;
#pragma unroll
    for (int t = 0; t < 3; ++t)
      if (t < nterms)
        *reinterpret_cast<uint4 *>(row + (int64_t)t * Kp) =
            make_uint4(w[t][0], w[t][1], w[t][2], w[t][3]);
    __syncthreads();  // the tile is refilled for the next row block
  }
}

// Fused max pass and scaled FP16 split of k-contiguous rows (rows of op(A)
// when A is transposed, columns of op(B) when B is not): one CTA per row, the
// row held in registers (VPT values a thread, Kp <= 256 VPT) between the
// block-wide max and the split, so it is read from memory once.  Writes the
// row's exponent and its terms exactly as row_absmax_kernel followed by
// split_bf16_kernel<true> do (columns [K, Kp) as zeros; rows past R left
// unwritten).
struct RowSplitArgs {
  const float *X0, *X1;  // first row of each operand (part)
  int ld0, ld1, R0, R1, Rp0, Rp1;
  int *ex0, *ex1;
  __nv_bfloat16 *out0, *out1;
  int K, Kp;
  int64_t ldo;
  int zbase;  // operand of blockIdx.z = 0
  int vec;    // every row starts on 16 bytes: float4 loads
};

template <int VPT>
__device__ __forceinline__ void row_load(const float *__restrict__ X, int K, bool live, bool vec,
                                         int t, float (&v)[VPT]) {
#pragma unroll
  for (int j = 0; j < VPT / 4; ++j) {
    const int e0 = 1024 * j + 4 * t;
    if (live && vec && e0 + 3 < K) {
      const float4 f = *reinterpret_cast<const float4 *>(X + e0);
      v[4 * j] = f.x; v[4 * j + 1] = f.y; v[4 * j + 2] = f.z; v[4 * j + 3] = f.w;
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q) v[4 * j + q] = (live && e0 + q < K) ? X[e0 + q] : 0.0f;
    }
  }
}

// Persistent over rows blockIdx.x, + gridDim.x, ...: the next row's loads are
// issued before the current row is reduced and written, so each CTA keeps
// reads in flight while it stores.
template <int VPT>
__global__ void __launch_bounds__(256) f16_row_split_kernel(const __grid_constant__ RowSplitArgs p) {
  const int z = blockIdx.z + p.zbase;
  const int R = z ? p.R1 : p.R0;
  const int ld = z ? p.ld1 : p.ld0;
  const float *__restrict__ X0 = z ? p.X1 : p.X0;
  int *__restrict__ exo = z ? p.ex1 : p.ex0;
  __nv_bfloat16 *__restrict__ out0 = z ? p.out1 : p.out0;
  const int K = p.K, Kp = p.Kp, t = threadIdx.x;
  const bool vec = p.vec != 0;
  __shared__ unsigned wmax[2][8];  // by row parity: a fast warp may start the next row
  int row = blockIdx.x;
  // rows past R are never read (the GEMM's maps end at the problem's rows)
  if (row >= R) return;  // the other operand has more rows (uniform per CTA)
  // value 4 j + q of this thread is element 1024 j + 4 t + q: a warp reads and
  // writes contiguous runs
  float v[VPT], nv[VPT];
  row_load<VPT>(X0 + (int64_t)row * ld, K, row < R, vec, t, v);
  for (int it = 0; row < R; row += gridDim.x, ++it) {
    const int next = row + gridDim.x;
    if (next < R) row_load<VPT>(X0 + (int64_t)next * ld, K, true, vec, t, nv);
    const bool live = row < R;
    // max |x| as a bit pattern (NaN and Inf above every finite value)
    unsigned mx = 0;
#pragma unroll
    for (int i = 0; i < VPT; ++i) mx = max(mx, __float_as_uint(fabsf(v[i])));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((t & 31) == 0) wmax[it & 1][t >> 5] = mx;
    __syncthreads();
    mx = wmax[it & 1][0];
#pragma unroll
    for (int w = 1; w < 8; ++w) mx = max(mx, wmax[it & 1][w]);
    const int e = live ? row_exponent_f32(mx) : 0;
    if (t == 0) exo[row] = e;
    __nv_bfloat16 *out = out0 + (int64_t)row * p.ldo;
    const bool bad = e == kNonFiniteExp;  // a row of Inf / NaN: all terms NaN
#pragma unroll
    for (int j = 0; j < VPT / 4; ++j) {
      const int e0 = 1024 * j + 4 * t;
      if (e0 >= Kp) continue;  // Kp is a multiple of 64: e0 < Kp covers e0 + 3
      uint2 w0, w1;  // hi and lo of the 4 values
      if (bad) {
        w0 = w1 = make_uint2(0x7e007e00u, 0x7e007e00u);
      } else {
        unsigned short h[4], l[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) f16_terms(v[4 * j + q], 15 - e, h[q], l[q]);
        w0 = make_uint2((unsigned)h[0] | ((unsigned)h[1] << 16),
                        (unsigned)h[2] | ((unsigned)h[3] << 16));
        w1 = make_uint2((unsigned)l[0] | ((unsigned)l[1] << 16),
                        (unsigned)l[2] | ((unsigned)l[3] << 16));
      }
      *reinterpret_cast<uint2 *>(out + e0) = w0;                   // term 0: hi
      *reinterpret_cast<uint2 *>(out + (int64_t)Kp + e0) = w1;     // term 1: lo
    }
#pragma unroll
    for (int i = 0; i < VPT; ++i) v[i] = nv[i];
  }
}

// Values a thread holds in the fused row split for k (0: k outside its range;
// short rows stay with the two-pass kernels, which cover 32 rows a CTA).
static int row_split_vpt(int k) {
  const int64_t kp = (k + 63) / 64 * 64;
  if (k < 1024) return 0;
  for (int v = 4; v <= 64; v *= 2)
    if (256 * v >= kp) return v;
  return 0;
}

static int sm_count();
static void row_split_launch(const RowSplitArgs &a, int vpt, unsigned rows, unsigned nz,
                             cudaStream_t st) {
  // persistent CTAs: 4 per SM per operand (each holds two rows in registers)
  const unsigned ctas = (unsigned)sm_count() * 4u;
  const dim3 grid(rows < ctas ? rows : ctas, 1, nz);
  switch (vpt) {
    case 4: f16_row_split_kernel<4><<<grid, 256, 0, st>>>(a); break;
    case 8: f16_row_split_kernel<8><<<grid, 256, 0, st>>>(a); break;
    case 16: f16_row_split_kernel<16><<<grid, 256, 0, st>>>(a); break;
    case 32: f16_row_split_kernel<32><<<grid, 256, 0, st>>>(a); break;
    default: f16_row_split_kernel<64><<<grid, 256, 0, st>>>(a); break;
  }
}

// Ozaki step 1: per-row max |x| of op(X) as the bit pattern of the
// non-negative value (monotone as an unsigned integer; NaN/Inf compare above
// finite values), for FP64 and (scaled FP16 split) FP32 rows.
// Short k ranges per grid row and unrolled loads keep enough reads in flight.
// The k range of one warp (k-contiguous rows) or one thread (row-contiguous
// columns) starts at these and doubles until the grid's y extent fits.
constexpr int kAmaxSpanK = 1024;
constexpr int kAmaxSpanR = 64;
template <typename T> struct AbsBits;
template <> struct AbsBits<double> {
  using U = unsigned long long;
  static __device__ __forceinline__ U of(double x) { return (U)__double_as_longlong(fabs(x)); }
  static __device__ __forceinline__ int exponent(U b) { return row_exponent(b); }
};
template <> struct AbsBits<float> {
  using U = unsigned;
  static __device__ __forceinline__ U of(float x) { return __float_as_uint(fabsf(x)); }
  static __device__ __forceinline__ int exponent(U b) { return row_exponent_f32(b); }
};

// Both operands in one launch: blockIdx.z = 0 reads the rows of op(A) into
// amax[0, Mp), z = 1 the columns of op(B) into amax[Mp, Mp + Np).  The last
// CTA to finish (a counter the caller zeroes with amax) writes the exponents
// of entries [first, first + total), so no separate exponent launch is
// needed.  A launch over one operand part (zbase = its operand, gridDim.z = 1)
// gets amax / ex offset to the part's first row.
template <typename T>
struct AbsmaxArgs {
  const T *X0, *X1;
  int ld0, ld1, R0, R1, kc0, kc1, span0, span1, K, Mp, first, total, zbase;
  typename AbsBits<T>::U *amax;
  int *ex;
  unsigned *counter;
  unsigned nblocks;  // CTAs in the grid
};

template <typename T>
__global__ void __launch_bounds__(256) row_absmax_kernel(const __grid_constant__ AbsmaxArgs<T> p) {
  using U = typename AbsBits<T>::U;
  const int z = blockIdx.z + p.zbase;
  const T *X = z ? p.X1 : p.X0;
  const int ld = z ? p.ld1 : p.ld0, R = z ? p.R1 : p.R0, span = z ? p.span1 : p.span0;
  const bool kcontig = (z ? p.kc1 : p.kc0) != 0;
  U *amax = p.amax + (z ? p.Mp : 0);
  const int k0 = blockIdx.y * span, k1 = min(p.K, k0 + span);
  if (kcontig) {
    // one warp per (row, k range)
    const int r = (blockIdx.x * 8) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (r < R && k0 < p.K) {
      U m = 0;
      const T *row = X + (int64_t)r * ld;
#pragma unroll 8
      for (int kk = k0 + lane; kk < k1; kk += 32) {
        const U b = AbsBits<T>::of(row[kk]);
        m = b > m ? b : m;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const U x = __shfl_xor_sync(0xffffffffu, m, o);
        m = x > m ? x : m;
      }
      if (lane == 0 && m) atomicMax(&amax[r], m);
    }
  } else {
    // one thread per row, one k range per grid row
    const int r = blockIdx.x * 256 + threadIdx.x;
    if (r < R && k0 < p.K) {
      U m = 0;
#pragma unroll 8
      for (int kk = k0; kk < k1; ++kk) {
        const U b = AbsBits<T>::of(X[r + (int64_t)kk * ld]);
        m = b > m ? b : m;
      }
      if (m) atomicMax(&amax[r], m);
    }
  }
  // every thread's atomics are visible before the CTA counts itself done
  __threadfence();
  __syncthreads();
  __shared__ bool last;
  if (threadIdx.x == 0) last = atomicAdd(p.counter, 1u) == p.nblocks - 1;
  __syncthreads();
  if (last) {
    __threadfence();
    for (int i = p.first + threadIdx.x; i < p.first + p.total; i += blockDim.x)
      p.ex[i] = AbsBits<T>::exponent(__ldcg(&p.amax[i]));
  }
}

// The S digits of 8 consecutive values of one row (row exponent e), packed as
// BF16 and written to dst[(s-1) * step].
__device__ __forceinline__ void slice_digits(const double *x, int e, int S, uint4 *dst,
                                             int64_t step) {
  unsigned long long mag[8];
  int sh[8];          // E - b: digit s sits at bits [sh - 7s, sh - 7s + 7) of M
  unsigned neg = 0;   // sign bits
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(x[j]);
    const int be = (int)((u >> 52) & 0x7ff);
    mag[j] = (u & 0xfffffffffffffull) | (be ? (1ull << 52) : 0ull);
    sh[j] = e - ((be ? be : 1) - 1075);
    neg |= (unsigned)(u >> 63) << j;
  }
  for (int s = 1; s <= S; ++s) {
    unsigned w[4];
#pragma unroll
    for (int j = 0; j < 8; j += 2) {
      unsigned h[2];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int t = sh[j + q] - 7 * s;
        const unsigned long long v =
            t >= 64 ? 0ull : (t >= 0 ? mag[j + q] >> t : (t > -7 ? mag[j + q] << -t : 0ull));
        const int d = (int)(v & 127);
        const float f = (float)(((neg >> (j + q)) & 1) ? -d : d);
        h[q] = __float_as_uint(f) >> 16;  // |d| < 2^7: the BF16 of f is its top half
      }
      w[j / 2] = h[0] | (h[1] << 16);
    }
    dst[(s - 1) * step] = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// Ozaki step 2: slices.  y = op(X)(r,k) * 2^-E_r lies in (-1,1); its truncated
// base-128 digits d_1..d_S (|d_s| <= 127, sign of y) are what the recurrence
// y <- 128 y, d = trunc(y), y <- y - d produces, each step exact.  They are read
// here straight from the bits: |x| = M * 2^b with M the 53-bit significand, so
// d_s = floor(M * 2^(b - E + 7s)) mod 128, a shift and a mask (the GPU's FP64
// rate would make the recurrence itself the bottleneck of this pass).
// out: S blocks of Rp rows x Kp (row-major BF16), slice s at rows (s-1)*Rp;
// each thread writes 8 consecutive k of one row (16 bytes) per slice; rows
// past R are left unwritten (the GEMM's maps end there).  Both operands in
// one launch (blockIdx.z).
__global__ void __launch_bounds__(256) ozaki_slice_kernel(const __grid_constant__ OperandPair p,
                                                          int S) {
  const int z = blockIdx.z;
  const double *__restrict__ X = z ? p.X1 : p.X0;
  const int ld = z ? p.ld1 : p.ld0, R = z ? p.R1 : p.R0, kcontig = z ? p.kc1 : p.kc0;
  const int Rp = z ? p.Rp1 : p.Rp0, K = p.K, Kp = p.Kp;
  const int *__restrict__ ex = z ? p.ex1 : p.ex0;
  __nv_bfloat16 *__restrict__ out = static_cast<__nv_bfloat16 *>(z ? p.out1 : p.out0);
  __shared__ double tile[32][65];
  const int k0 = blockIdx.x * 64;
  const int r = threadIdx.x >> 3, kq = (threadIdx.x & 7) * 8;
  const int64_t step = (int64_t)Rp * Kp / 8;  // one slice block, in uint4
  for (int r0 = blockIdx.y * 32; r0 < R; r0 += gridDim.y * 32) {
    load_tile_32x64<double>(X, ld, R, K, kcontig != 0, r0, k0, tile);
    __syncthreads();
    const int gr = r0 + r;
    const int e = (gr < R) ? ex[gr] : 0;
    uint4 *dst = reinterpret_cast<uint4 *>(out + (int64_t)gr * Kp + k0 + kq);
    if (e == kNonFiniteExp) {
      const uint4 nan4 = make_uint4(0x7fc07fc0u, 0x7fc07fc0u, 0x7fc07fc0u, 0x7fc07fc0u);
      for (int s = 0; s < S; ++s) dst[s * step] = nan4;
    } else {
      slice_digits(tile[r] + kq, e, S, dst, step);
    }
    __syncthreads();  // the tile is refilled for the next row block
  }
}

// ===========================================================================
// BF16xP GEMM: C = alpha * A'B'^T + beta * C, persistent, 128 x 256 tiles.
//
// The tensor core's FP32 accumulation over a long K' is less accurate than a
// round-to-nearest FFMA chain (measured: both 3x and 6x forms ~9e-6 relative
// at K' = 3*8192 and 6*8192).  So TMEM accumulates bounded chunks only; the 16
// epilogue warps (64 columns each) add every chunk into FP32 running sums in
// registers (round to nearest) while the MMA warp fills the other TMEM buffer
// with the next chunk.  Chunks never cross a segment (one cross product), and
// their length follows the segment's magnitude: order-2 products (~2^-16 of
// the result) need no chunking, order-1 products (~2^-8; ~2^-11 in the scaled
// FP16 form) chunks of 16 (128) blocks, the hi*hi segment chunks of `chunk0`
// blocks.  Small segments come first in K', so each tile starts with a long
// chunk that hides the previous tile's C store.  (8 epilogue warps with 128
// columns each spilled at the 168-register cap and drained a chunk in about
// 2.7 us, twice the MMA time of a 4-block chunk.)
// ===========================================================================
struct Bf16xParams {
  // C's window (m x n, ldc) in boxes of 128 rows x 64 columns, when c_pf:
  // the producer prefetches each tile's C into L2 as the tile starts, and the
  // staged-C kernel (CS) loads the boxes into shared memory for its epilogue
  CUtensorMap tmC;
  int c_pf;
  int m, n, tiles_m, tiles_n, kblocks;
  // K' = nseg segments of skb 64-wide blocks; segment s reads the term block
  // (segA >> 4 s) & 15 of A' and (segB >> 4 s) & 15 of B' (each term stored
  // once, term t at columns [t Kp, (t + 1) Kp))
  int skb;
  unsigned segA, segB;
  // K' is cut into runs of consecutive segments whose products have the same
  // order (i + j): run r ends at block run_end<r> and is accumulated in TMEM
  // chunks of run_chunk<r> blocks (0 = the whole run).  Scalars, not arrays,
  // so that no parameter is indexed at run time.
  int nruns;
  int run_end0, run_end1, run_end2;
  int run_chunk0, run_chunk1, run_chunk2;
  float alpha, beta;
  float *C;
  int ldc;
  unsigned *err;
  // scaled FP16 form (kernel F16 = true): the running sums are multiplied by
  // `rescale` before chunk `rescale_chunk` of each tile is added, and the
  // result is scaled by 2^(expA[row] + expB[col] - 30).
  int rescale_chunk;
  float rescale;
  const int *expA, *expB;
  // grouped launches (kernel GR = true): the table of GBxProblem, its length
  // and the total number of work units (tiles) over all problems
  const void *grp;
  int nprob, total_units;
};

// One problem of a grouped launch of bf16x_gemm_kernel: its tensor maps over
// its own prepared operands, its parameters and its first work unit; the
// problems' units are concatenated in table order.
struct alignas(128) GBxProblem {
  CUtensorMap tmA, tmB;
  Bf16xParams prm;
  int unit0;
};

constexpr int kBxEpiWarps = 16;                     // 4 per TMEM lane quarter
constexpr int kBxThreads = (2 + kBxEpiWarps) * 32;  // producer, MMA, epilogue
constexpr int kBxABytes = kSplitBM * 128;
constexpr int kBxDefaultChunk = 4;                  // 4 x 64 = 256 K' per chunk

// Geometry of a 128 x BN output tile (BN = 256, or 128 for shapes with few
// tiles): B tile bytes per 64-wide K block, the stage (A + B), the ring depth
// that fits in shared memory (4 stages of 48 KB or 6 of 32 KB), and the
// columns each of the 16 epilogue warps owns (BN / 4).
template <int BN>
struct TileN {
  static constexpr int kBBytes = BN * 128;
  static constexpr int kStage = kSplitBM * 128 + kBBytes;
  static constexpr int kStages = BN == 256 ? 4 : 6;
  static constexpr int kSmem = kStages * kStage + 1024 + 256;
  static constexpr int kCols = BN / 4;
};

// Cluster modes of the tile kernels: 0 = one CTA per tile, loading its own A
// and B tiles; 2 = pair MMAs (cta_group::2, M = 256) on 2-CTA clusters over
// the row tiles 2u and 2u + 1 of one column tile: each CTA holds its 128 rows
// of A and half of the B tile, the even CTA issues the MMAs for both, so a
// stage is 32 KB instead of 48 KB, the ring is 6 deep instead of 4, and each
// B tile is read from L2 once per pair.  In mode 2 both CTAs' TMA loads
// complete on the even CTA's full barrier, and the odd CTA's epilogue warps
// report drained TMEM buffers to the even CTA with plain (default-semantics)
// remote arrives: cluster-scope release arrives made the kernel 2.5x slower.
// Every TMA load lands in the issuing CTA's own shared memory.
template <int CL, int BN>
struct ClusterTile {
  static constexpr bool kPair = CL == 2;
  static constexpr int kBBytes = (kPair ? BN / 2 : BN) * 128;  // B bytes in one CTA's stage
  static constexpr int kStage = kSplitBM * 128 + kBBytes;
  static constexpr int kStages = kPair ? (BN == 256 ? 6 : 8) : TileN<BN>::kStages;
  static constexpr int kSmem = kStages * kStage + 1024 + 256;
};

// Staged C (kernel CS = true; pair MMAs, 256-wide tiles): the epilogue's plain
// loads of C, a few per thread in flight, took 10.5 us of a rank-256 tile's
// 14.5 (a timeline of one CTA; 3.3 us without them), longer than the tile's
// MMAs.  So C moves by TMA instead: in place of one ring stage, a shared-memory
// slot of 128 rows x 32 columns for each column block (the 4 epilogue warps
// of 64 columns).  Each block loads the first half of its C as the tile
// starts, under its MMAs; its warps write the results back into the slot and
// one TMA store takes them to C; the second half follows in the same slot
// once that store has read it.  (Two 64-column slots shared by the blocks
// kept blocks 2 and 3 waiting for blocks 0 and 1: 5.7 us against 1.4 us.)
constexpr int kCsSlotBytes = kSplitBM * 32 * 4;
template <int CL, int BN, bool CS>
struct BxSmem {
  static constexpr int kStages = CS ? ClusterTile<CL, BN>::kStages - 1 : ClusterTile<CL, BN>::kStages;
  static constexpr int kBytes = kStages * ClusterTile<CL, BN>::kStage + (CS ? 4 * kCsSlotBytes : 0) +
                                1024 + 256;
};
// Staged C for tiles of at most this many K blocks (MMAs shorter than the C
// update they have to hide; 24 at k = 256 with 6 products), and for C
// windows whose rows fill whole 16-byte units (m a multiple of 4).
constexpr int kBxStagedMaxKBlocks = 48;
// Row-tile pairs in a group of the staged-C kernel's raster (8 otherwise):
// short K leaves each A' row panel small enough (1.5 MB a pair at k = 256)
// for a larger group to stay in L2 while B' is swept once per group
// (rank-256 SGEMM, one box: 8 -> 221.1, 16 -> 237.3, 32 -> 231.9, 64 -> 232.2
// TFLOP/s).
constexpr int kCsGroupM = 16;
// Row-tile pairs in a group of the pair-MMA raster at long K: 16 from 64
// pairs, else 8 (SGEMM TN 3xFP16, one box, groups of 4 / 8 / 16: 8192^3
// 505 / 518 / 515 TFLOP/s, 16384^3 493 / 499 / 510).
__device__ __forceinline__ int pair_group_m(int pairs) { return pairs >= 64 ? 16 : 8; }

// GR: a grouped launch over the problems of p.grp (one CTA per tile; the
// kernel parameters' maps are unused), each unit a tile of one problem, with
// that problem's K extent, chunk runs and epilogue parameters.
template <int CL, bool F16, int BN, bool GR = false, bool CS = false>
__global__ void __launch_bounds__(kBxThreads, 1)
bf16x_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                  const __grid_constant__ Bf16xParams p) {
  using T = TileN<BN>;
  using CT = ClusterTile<CL, BN>;
  static_assert(CL == 0 || CL == 2, "cluster modes: 0 (one CTA per tile) or 2 (pair MMAs)");
  static_assert(!GR || CL == 0, "grouped launches run one CTA per tile");
  static_assert(!CS || (CL == 2 && BN == 256 && !GR), "staged C: pair MMAs on 256-wide tiles");
  constexpr bool PAIR = CT::kPair;
  constexpr int kBxStages = BxSmem<CL, BN, CS>::kStages, kBxStage = CT::kStage;
  constexpr int kBxColsPerWarp = T::kCols;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                              ~uintptr_t(1023));
  uint8_t *cslot = smem + kBxStages * kBxStage;  // CS: the C slots of the 4 column blocks
  uint64_t *full = reinterpret_cast<uint64_t *>(cslot + (CS ? 4 * kCsSlotBytes : 0));
  uint64_t *empty = full + kBxStages;
  uint64_t *accf = empty + kBxStages;
  uint64_t *acce = accf + 2;
  uint64_t *done = acce + 2;
  // CS, per column block: its slot loaded (cfull), its results written into
  // the slot (cwr), the slot read by their store (crel); two phases a tile each
  uint64_t *cfull = done + 1, *cwr = cfull + (CS ? 4 : 0), *crel = cwr + (CS ? 4 : 0);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(crel + (CS ? 4 : 0));
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kBxStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);  // pair: one multicast commit frees both CTAs' stage
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], PAIR ? 2 * kBxEpiWarps : kBxEpiWarps);  // pair: both CTAs drain
    }
    mbar_init(done, 1);
    if (CS) {
      for (int c = 0; c < 4; ++c) {
        mbar_init(&cfull[c], 1);  // the loading thread's expect_tx
        mbar_init(&cwr[c], 4);    // the block's 4 warps
        mbar_init(&crel[c], 1);   // the storing thread, once its store has read the slot
      }
    }
    *abort_flag = 0;
    fence_barrier_init();
    if (!GR) {
      tma_prefetch_desc(&tmA);
      tma_prefetch_desc(&tmB);
      if (p.c_pf) tma_prefetch_desc(&p.tmC);
    }
  }
  if (warp == 1) {
    if (PAIR) { tmem_alloc_pair(tmem_slot, 512); tmem_relinquish_pair(); }
    else { tmem_alloc(tmem_slot, 512); tmem_relinquish(); }
  }
  tc_fence_before();
  __syncthreads();
  if (PAIR) cluster_sync();  // the peer's barriers are initialised before any remote arrive
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  // work units: tiles, or (PAIR) row-tile pairs whose rank-th row tile is this CTA's
  const uint32_t rank = PAIR ? cluster_ctarank() : 0u;
  const GBxProblem *grp = static_cast<const GBxProblem *>(p.grp);
  const int pm = PAIR ? (p.tiles_m + 1) / 2 : p.tiles_m;
  const int nunits = GR ? p.total_units : pm * p.tiles_n;
  const int first = PAIR ? (int)(blockIdx.x >> 1) : (int)blockIdx.x;
  const int stride = PAIR ? (int)(gridDim.x >> 1) : (int)gridDim.x;
  // grouped: the problem of unit u (the last whose unit0 <= u) and its parameters
  auto prob_of = [&](int u) -> int {
    if constexpr (!GR) return 0;
    int lo = 0, hi = p.nprob - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (grp[mid].unit0 <= u) lo = mid; else hi = mid - 1;
    }
    return lo;
  };
  auto prm = [&](int i) -> const Bf16xParams * {
    if constexpr (GR) return &grp[i].prm;
    else return &p;
  };
  auto map_a = [&](int i) -> const void * {
    if constexpr (GR) return &grp[i].tmA;
    else return &tmA;
  };
  auto map_b = [&](int i) -> const void * {
    if constexpr (GR) return &grp[i].tmB;
    else return &tmB;
  };
  auto unit_tile = [&](int u, int i, int &tm, int &tn) {
    if constexpr (GR) {
      const Bf16xParams &q = grp[i].prm;
      tile_coords(u - grp[i].unit0, q.tiles_m, q.tiles_n, kSplitGroupM, tm, tn);
    } else {
      int um;
      tile_coords(u, pm, p.tiles_n, CS ? kCsGroupM : PAIR ? pair_group_m(pm) : kSplitGroupM, um,
                  tn);
      tm = PAIR ? 2 * um + (int)rank : um;  // PAIR: a row tile past the end is zero-filled, not stored
    }
  };
  auto run_end = [&](const Bf16xParams &q, int r) {
    return r == 0 ? q.run_end0 : (r == 1 ? q.run_end1 : q.run_end2);
  };
  auto run_chunk = [&](const Bf16xParams &q, int r) {  // chunk length of run r in K blocks
    const int len = run_end(q, r) - (r == 0 ? 0 : run_end(q, r - 1));
    const int cl = r == 0 ? q.run_chunk0 : (r == 1 ? q.run_chunk1 : q.run_chunk2);
    return cl > 0 ? cl : len;
  };
  auto nchunks_of = [&](const Bf16xParams &q) {
    int nc = 0;
    for (int r = 0; r < q.nruns; ++r) {
      const int len = run_end(q, r) - (r == 0 ? 0 : run_end(q, r - 1));
      nc += (len + run_chunk(q, r) - 1) / run_chunk(q, r);
    }
    return nc;
  };
  const int nchunks1 = GR ? 0 : nchunks_of(p);  // the single problem's chunks per tile

  if (warp == 0) {
    if (lane == 0) {
      uint32_t L = 0;
      for (int u = first; u < nunits && !*abort_flag; u += stride) {
        const int pi = prob_of(u);
        const int kblocks = prm(pi)->kblocks;
        const void *mA = map_a(pi), *mB = map_b(pi);
        const Bf16xParams &q = *prm(pi);
        const int skb = q.skb;
        const unsigned segA = q.segA, segB = q.segB;
        int tm, tn;
        unit_tile(u, pi, tm, tn);
        // C of the tile into L2 for its epilogue, where the tile's MMAs are
        // too short to hide the C reads (a long tile's prefetched C only
        // displaces operands: SGEMM TN 8192^3 read 5.35-5.58 GB a launch with
        // it, 4.85-5.39 without)
        if (q.c_pf && q.kblocks <= kBxStagedMaxKBlocks)
          for (int cb = 0; cb < BN / 32; ++cb) tma_prefetch_l2_2d(&q.tmC, tm * kSplitBM, tn * BN + cb * 32);
        int sg = 0, kk = 0;  // segment of block kb and the block within it
        for (int kb = 0; kb < kblocks; ++kb, ++L, ++kk) {
          if (kk == skb) { ++sg; kk = 0; }
          // 3-D maps of k x terms x rows: (K in the term block, term, row)
          const int xk = kk * kSplitBK;
          const int za = (int)((segA >> (4 * sg)) & 15u), zb = (int)((segB >> (4 * sg)) & 15u);
          const int s = L % kBxStages;
          const uint32_t r = L / kBxStages;
          if (!mbar_wait(&empty[s], (r & 1) ^ 1, p.err, kErrTimeoutEmpty, abort_flag)) break;
          uint8_t *sa = smem + s * kBxStage;
          if (PAIR) {
            // both CTAs' A rows and B halves land on the even CTA's full barrier
            if (rank == 0) mbar_arrive_expect_tx(&full[s], 2 * kBxStage);
            const uint32_t fb = cluster_addr(&full[s], 0);
            tma_load_3d_pair(sa, mA, xk, za, tm * kSplitBM, fb);
            tma_load_3d_pair(sa + kBxABytes, mB, xk, zb, tn * BN + (int)rank * (BN / 2), fb);
            continue;
          }
          mbar_arrive_expect_tx(&full[s], kBxStage);  // own A and B tiles
          tma_load_3d(sa, mA, xk, za, tm * kSplitBM, &full[s]);
          tma_load_3d(sa + kBxABytes, mB, xk, zb, tn * BN, &full[s]);
        }
      }
    }
  } else if (warp == 1 && PAIR && rank == 1) {
    // odd CTA of a pair: the even CTA issues the MMAs of both
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr int kM = PAIR ? 2 * kSplitBM : kSplitBM;
      constexpr uint32_t idesc = F16 ? idesc_f16_f32(kM, BN) : idesc_bf16_f32(kM, BN);
      uint32_t L = 0, chunk = 0;
      bool ok = true;
      for (int u = first; u < nunits && ok; u += stride) {
        const Bf16xParams &q = *prm(prob_of(u));
        const int nchunks = GR ? nchunks_of(q) : nchunks1;
        int rn = 0, c0 = 0;
        for (int c = 0; c < nchunks && ok; ++c, ++chunk) {
          // chunk c covers K blocks [c0, c1) of run rn
          const int rend = run_end(q, rn);
          const int c1 = min(rend, c0 + run_chunk(q, rn));
          const int b = chunk & 1;
          const uint32_t u = chunk >> 1;
          // pair: half of the arrivals come from the odd CTA's epilogue warps
          if (!mbar_wait(&acce[b], (u & 1) ^ 1, p.err, kErrTimeoutMma, abort_flag)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t dt = tmem + b * BN;
          for (int kb = c0; kb < c1; ++kb, ++L) {
            const int s = L % kBxStages;
            const uint32_t r = L / kBxStages;
            if (!mbar_wait(&full[s], r & 1, p.err, kErrTimeoutFull, abort_flag)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t sa = smem_u32(smem + s * kBxStage), sb = sa + kBxABytes;
#pragma unroll
            for (int kk = 0; kk < kSplitBK / 16; ++kk) {
              if (PAIR)
                umma_pair(dt, umma_desc_sw128(sa + kk * 32), umma_desc_sw128(sb + kk * 32), idesc,
                          (kb > c0 || kk > 0) ? 1u : 0u);
              else
                umma_bf16(dt, umma_desc_sw128(sa + kk * 32), umma_desc_sw128(sb + kk * 32),
                          idesc, (kb > c0 || kk > 0) ? 1u : 0u);
            }
            if (PAIR)
              umma_commit_pair(&empty[s], 0x3);  // both CTAs' stage s is free
            else
              umma_commit(&empty[s]);
          }
          if (ok) {
            if (PAIR)
              umma_commit_pair(&accf[b], 0x3);
            else
              umma_commit(&accf[b]);
          }
          c0 = c1;
          if (c0 == rend) ++rn;
        }
      }
      // every issued MMA has completed before TMEM is released
      if (PAIR)
        umma_commit_pair(done, 0x1);
      else
        umma_commit(done);
      mbar_wait(done, 0, p.err, kErrTimeoutMma, nullptr);
    }
  } else {
    const int q = warp & 3;             // TMEM lane quarter this warp may access
    const int h = (warp - 2) >> 2;      // column block of the tile
    const int row_in_tile = q * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16) + h * kBxColsPerWarp;
    // CS: column block h's slot holds half of its columns at a time.  Its
    // barriers move two phases a tile (first half, second half), and every
    // wait comes after the block's own arrival on the phase before, so the
    // parities are fixed: no waiter can be two phases ahead.
    float *cs_c = reinterpret_cast<float *>(cslot + h * kCsSlotBytes);
    const bool cs_loader = CS && q == 0 && lane == 0;
    int cs_pending = -1;  // the half whose load this thread issued and the block has not read
    auto cs_load = [&](const Bf16xParams &pq, int tm, int tn, int half) {
      mbar_arrive_expect_tx(&cfull[h], kCsSlotBytes);
      tma_load_2d_hint(cs_c, &pq.tmC, tm * kSplitBM, tn * BN + h * 64 + half * 32, &cfull[h],
                       l2_evict_first());
      cs_pending = half;
    };
    uint32_t chunk = 0;
    bool ok = true;
    for (int u = first; u < nunits && ok; u += stride) {
      const int pi = prob_of(u);
      const Bf16xParams &pq = *prm(pi);
      const int nchunks = GR ? nchunks_of(pq) : nchunks1;
      int tm, tn;
      unit_tile(u, pi, tm, tn);
      if (CS) {  // the first half of the block's C, under the MMAs, once the slot is free
        if (!mbar_wait(&crel[h], 1u, p.err, kErrTimeoutAcc, abort_flag)) { ok = false; break; }
        if (cs_loader) cs_load(pq, tm, tn, 0);
      }
      float run[kBxColsPerWarp];
#pragma unroll
      for (int j = 0; j < kBxColsPerWarp; ++j) run[j] = 0.f;
      for (int c = 0; c < nchunks; ++c, ++chunk) {
        const int b = chunk & 1;
        const uint32_t u = chunk >> 1;
        if (!mbar_wait(&accf[b], u & 1, p.err, kErrTimeoutAcc, abort_flag)) { ok = false; break; }
        tc_fence_after();
        if (F16 && c == pq.rescale_chunk) {  // the hi*lo segments end: scale them by 2^-11 (exact)
#pragma unroll
          for (int j = 0; j < kBxColsPerWarp; ++j) run[j] *= pq.rescale;
        }
#pragma unroll
        for (int g = 0; g < kBxColsPerWarp / 16; ++g) {
          uint32_t v[16];
          tmem_ld16(lane_base + b * BN + g * 16, v);
          tmem_ld_wait();
#pragma unroll
          for (int j = 0; j < 16; ++j) run[g * 16 + j] += __uint_as_float(v[j]);
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) {
          if (PAIR)
            mbar_arrive_cluster<false>(&acce[b], 0);  // the even CTA issues the MMAs of both
          else
            mbar_arrive(&acce[b]);
        }
      }
      if (!ok) break;
      const int row = tm * kSplitBM + row_in_tile;
      const int col0 = tn * BN + h * kBxColsPerWarp;
      // scaled FP16 form: the row and column scales come off here (a non-finite
      // row or column is NaN already; its marker exponent is capped)
      const int ea = (F16 && row < pq.m) ? min(pq.expA[row], 1024) - 30 : 0;
      // beta C + alpha v for the columns [c0, c1) of the warp, rounded as
      // written (no contraction: every instantiation and the grouped launch
      // round alike); C from the slot (CS) or from memory in batches of 8
      // columns, all loads of a batch before its stores
      auto update = [&](int c0, int c1) {
#pragma unroll
        for (int jb = c0; jb < c1; jb += 8) {
          float cv[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int col = col0 + jb + j;
            if (CS)  // the slot holds 32 columns x 128 rows, column-major
              cv[j] = cs_c[(jb - c0 + j) * kSplitBM + row_in_tile];
            else
              cv[j] = (col < pq.n) ? pq.C[(int64_t)col * pq.ldc + row] : 0.f;
          }
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int col = col0 + jb + j;
            if (col < pq.n) {
              const float v =
                  F16 ? scale_pow2f(run[jb + j], ea + min(pq.expB[col], 1024)) : run[jb + j];
              const float cb = (pq.beta == 1.0f) ? cv[j] : __fmul_rn(cv[j], pq.beta);
              const float r = __fadd_rn(cb, __fmul_rn(pq.alpha, v));
              if (CS)
                cs_c[(jb - c0 + j) * kSplitBM + row_in_tile] = r;
              else
                pq.C[(int64_t)col * pq.ldc + row] = r;
            }
          }
        }
      };
      if constexpr (CS) {
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          // the second half's load follows the first half's store (crel phase 0)
          if (half == 1 && !mbar_wait(&crel[h], 0u, p.err, kErrTimeoutAcc, abort_flag)) {
            ok = false;
            break;
          }
          if (!mbar_wait(&cfull[h], (uint32_t)half, p.err, kErrTimeoutAcc, abort_flag)) {
            ok = false;
            break;
          }
          cs_pending = -1;
          if (row < pq.m) update(half * 32, half * 32 + 32);
          // the results are in the slot (visible to the async proxy): one
          // thread stores them, frees the slot once the store has read it and
          // loads the second half
          fence_proxy_async();
          __syncwarp();
          if (lane == 0) mbar_arrive(&cwr[h]);
          if (cs_loader) {
            if (mbar_wait(&cwr[h], (uint32_t)half, p.err, kErrTimeoutAcc, abort_flag)) {
              tma_store_2d_hint(&pq.tmC, cs_c, tm * kSplitBM, tn * BN + h * 64 + half * 32,
                                l2_evict_first());
              bulk_commit();
              bulk_wait_read0();
              mbar_arrive(&crel[h]);
              if (half == 0) cs_load(pq, tm, tn, 1);
            } else {
              ok = false;
              mbar_arrive(&crel[h]);
              break;
            }
          }
        }
      } else {
        if (row < pq.m) update(0, kBxColsPerWarp);
      }
    }
    // a load still in flight after a time-out lands before the CTA exits, and
    // the last stores are complete
    if (cs_pending >= 0)
      mbar_wait_limit(&cfull[h], (uint32_t)cs_pending, GB300_SPIN_LIMIT, nullptr, 0);
    if (CS && cs_loader) bulk_wait0();
  }
  tc_fence_before();
  __syncthreads();
  if (PAIR) cluster_sync();  // both CTAs are done with the pair's TMEM
  if (warp == 1) {
    tc_fence_after();
    if (PAIR)
      tmem_dealloc_pair(tmem, 512);
    else
      tmem_dealloc(tmem, 512);
  }
  if (PAIR) cluster_sync();  // no peer commit or arrive can still target this CTA
}

// ===========================================================================
// Ozaki GEMM: persistent, 128 x 256 tiles, exact integer slice products.
// TMEM: [0,256) and [256,512) chunk accumulators (FP32).  The tile's FP64
// result accumulates in a global scratch (Mp x Np, column-major) that only
// this tile's threads touch: each slice group is folded into it once, so its
// traffic is small next to the operand stream, and TMEM holds two full-width
// accumulators (128-column tiles reach only ~55% of the tensor pipe here).
// ===========================================================================
struct OzakiParams {
  int m, n, tiles_m, tiles_n;
  int S, KB;   // slices (mode 0) or moduli (mode 1), K blocks of 64 per pair
  int mode;    // 0: slice products folded into FP64; 1: residues mod mods[g] (CRT form)
  int Mp, Np;  // rows per slice block of A and B
  double alpha, beta;
  double *C;
  int ldc;
  const int *expA, *expB;  // per-row / per-column scale exponents
  double *res;             // Mp x Np FP64 result scratch (ld = Mp)
  uint8_t *rres;           // mode 1: S planes of Mp x Np residues in [0, mods[g]), each in
                           // words of 4 columns: byte (col / 4) * 4 Mp + 4 row + col % 4
  int mods[kCrtMaxModuli];
  unsigned mods_mg[kCrtMaxModuli];  // floor(2^32 / mods[g]) for the Barrett reduction
  float mods_f[kCrtMaxModuli], mods_inv[kCrtMaxModuli];  // mods[g] and 1 / mods[g] in FP32
  unsigned *err;
  // work units per tile: the S groups in gsplit ranges (CRT form only, whose
  // moduli are independent GEMMs; 1 in the slice form, which sums its groups)
  int gsplit;
  // first row of op(A) / column of op(B) in each operand block (a sub-block
  // of a larger problem's workspace; 0 for a whole problem)
  int row0, col0;
  // grouped launches (kernel GR = true): the table of GOzProblem, its length
  // and the total number of work units (whole tiles) over all problems
  const void *grp;
  int nprob, total_units;
};

// One problem of a grouped launch of ozaki_gemm_kernel (CRT mode, one CTA per
// tile, whole-tile units): its tensor maps, parameters and first unit.
struct alignas(128) GOzProblem {
  CUtensorMap tmA, tmB;
  OzakiParams prm;
  int unit0;
};

constexpr int kOzEpiWarps = 16;  // 4 per TMEM lane quarter, BN / 4 columns each
constexpr int kOzThreads = (2 + kOzEpiWarps) * 32;
constexpr int kOzABytes = kSplitBM * 128;
// 16 x 64 = 1024 K-steps per exact chunk: |partial sum| <= 1024 * 127^2 =
// 16,516,096 < 2^24, so every partial sum is an exactly representable FP32 integer.
constexpr int kOzChunkStages = 16;
// int32 running sums are folded into FP64 at least every 128 chunks:
// 128 * 16,516,096 < 2^31.
constexpr int kOzRunChunks = 128;

// pairs of slice group t: sa in [lo, hi], sb = t - sa
__device__ __forceinline__ void group_pairs(int t, int S, int &lo, int &np) {
  lo = max(1, t - S);
  const int hi = min(S, t - 1);
  np = hi - lo + 1;
}

// Group gi (0-based) of the K sequence.  Mode 0: slice order t = S + 1 - gi,
// pairs sa in [lo, lo + np), sb = t - sa.  Mode 1: modulus gi, the single pair
// (gi + 1, gi + 1) of residue blocks (t = 2 gi + 2 makes sb = t - sa hold).
__device__ __forceinline__ void group_of(int mode, int gi, int S, int &t, int &lo, int &np) {
  if (mode) {
    lo = gi + 1;
    np = 1;
    t = 2 * gi + 2;
  } else {
    t = S + 1 - gi;
    group_pairs(t, S, lo, np);
  }
}
// mode 1: int32 running sums are reduced mod p at least every 64 chunks:
// 64 * 1024 * 127^2 < 2^31.
constexpr int kCrtRunChunks = 64;

// CL: the cluster mode of bf16x_gemm_kernel (0: one CTA per tile; 2: pair
// MMAs over the row tiles 2u and 2u + 1, each CTA loading its A tile and half
// of the B tile, the even CTA issuing the MMAs of both).  In mode 2 a row tile
// past the end (odd tile rows) still takes part in the pipeline (its A loads
// fetch rows of the next block, or zeros past the last, and its sums are
// discarded) but writes nothing.
// MODE: 0 = slice products folded into FP64, 1 = the CRT form's residue GEMMs
// (p.mode holds the same value; the template keeps the two epilogues' register
// allocations apart).
// GR: a grouped launch over the problems of p.grp (CRT mode, one CTA per tile,
// each unit a whole tile of one problem with all its moduli).
template <int CL, int BN, int MODE, bool GR = false>
__global__ void __launch_bounds__(kOzThreads, 1)
ozaki_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                  const __grid_constant__ OzakiParams p) {
  using T = TileN<BN>;
  using CT = ClusterTile<CL, BN>;
  static_assert(CL == 0 || CL == 2, "cluster modes: 0 (one CTA per tile) or 2 (pair MMAs)");
  static_assert(!GR || (CL == 0 && MODE == 1), "grouped launches: CRT mode, one CTA per tile");
  constexpr bool PAIR = CT::kPair;
  constexpr int kOzStages = CT::kStages, kOzStage = CT::kStage;
  constexpr int kOzCols = T::kCols;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                              ~uintptr_t(1023));
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + kOzStages * kOzStage);
  uint64_t *empty = full + kOzStages;
  uint64_t *accf = empty + kOzStages;
  uint64_t *acce = accf + 2;
  uint64_t *done = acce + 2;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kOzStages; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], PAIR ? 2 * kOzEpiWarps : kOzEpiWarps);  // pair: both CTAs drain
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    fence_barrier_init();
    if (!GR) {
      tma_prefetch_desc(&tmA);
      tma_prefetch_desc(&tmB);
    }
  }
  if (warp == 1) {
    if (PAIR) { tmem_alloc_pair(tmem_slot, 512); tmem_relinquish_pair(); }
    else { tmem_alloc(tmem_slot, 512); tmem_relinquish(); }
  }
  tc_fence_before();
  __syncthreads();
  if (PAIR) cluster_sync();  // the peer's barriers are initialised before any remote arrive
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  // work units: tiles, or (PAIR) row-tile pairs whose rank-th row tile is this CTA's
  const uint32_t rank = PAIR ? cluster_ctarank() : 0u;
  const int pm = PAIR ? (p.tiles_m + 1) / 2 : p.tiles_m;
  // units: (group range, tile), group-range major so that neighbouring units
  // share the residue planes of their moduli in L2
  const int ntu = pm * p.tiles_n;
  const int nunits = GR ? p.total_units : ntu * p.gsplit;
  const int first = PAIR ? (int)(blockIdx.x >> 1) : (int)blockIdx.x;
  const int stride = PAIR ? (int)(gridDim.x >> 1) : (int)gridDim.x;
  const GOzProblem *grp = static_cast<const GOzProblem *>(p.grp);
  // grouped: the problem of unit u (the last whose unit0 <= u) and its parameters
  auto prob_of = [&](int u) -> int {
    if constexpr (!GR) return 0;
    int lo = 0, hi = p.nprob - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (grp[mid].unit0 <= u) lo = mid; else hi = mid - 1;
    }
    return lo;
  };
  auto prm = [&](int i) -> const OzakiParams * {
    if constexpr (GR) return &grp[i].prm;
    else return &p;
  };
  auto map_a = [&](int i) -> const void * {
    if constexpr (GR) return &grp[i].tmA;
    else return &tmA;
  };
  auto map_b = [&](int i) -> const void * {
    if constexpr (GR) return &grp[i].tmB;
    else return &tmB;
  };
  auto unit_tile = [&](int u, int i, int &tm, int &tn) {
    if constexpr (GR) {
      const OzakiParams &q = grp[i].prm;
      tile_coords(u - grp[i].unit0, q.tiles_m, q.tiles_n, kSplitGroupM, tm, tn);
    } else {
      int um;
      tile_coords(u % ntu, pm, p.tiles_n, PAIR ? kSplitGroupM / 2 : kSplitGroupM, um, tn);
      tm = PAIR ? 2 * um + (int)rank : um;
    }
  };
  auto unit_groups = [&](int u, const OzakiParams &q, int &g0, int &g1) {
    if constexpr (GR) {
      g0 = 0;
      g1 = q.S;
    } else {
      const int gp = u / ntu;
      g0 = gp * q.S / q.gsplit;
      g1 = (gp + 1) * q.S / q.gsplit;
    }
  };

  if (warp == 0) {
    if (lane == 0) {
      uint32_t L = 0;
      bool ok = true;
      for (int u = first; u < nunits && ok; u += stride) {
        const int pi = prob_of(u);
        const OzakiParams &q = *prm(pi);
        const int S = q.S, KB = q.KB;
        const void *mA = map_a(pi), *mB = map_b(pi);
        int tm, tn, g0, g1;
        unit_tile(u, pi, tm, tn);
        unit_groups(u, q, g0, g1);
        for (int gi = g0; gi < g1 && ok; ++gi) {
          int t, lo, np;
          group_of(MODE, gi, S, t, lo, np);
          const int G = np * KB;
          for (int idx = 0; idx < G; ++idx, ++L) {
            const int kb = idx / np, sa = lo + idx % np, sb = t - sa;
            const int s = L % kOzStages;
            const uint32_t r = L / kOzStages;
            if (!mbar_wait(&empty[s], (r & 1) ^ 1, p.err, kErrTimeoutEmpty, abort_flag)) {
              ok = false;
              break;
            }
            uint8_t *sa_ptr = smem + s * kOzStage;
            const int arow = q.row0 + tm * kSplitBM;  // in block sa - 1 of A
            if (PAIR) {
              // both CTAs' A rows and B halves land on the even CTA's full barrier
              if (rank == 0) mbar_arrive_expect_tx(&full[s], 2 * kOzStage);
              const uint32_t fb = cluster_addr(&full[s], 0);
              tma_load_3d_pair(sa_ptr, mA, kb * kSplitBK, arow, sa - 1, fb);
              tma_load_3d_pair(sa_ptr + kOzABytes, mB, kb * kSplitBK,
                               q.col0 + tn * BN + (int)rank * (BN / 2), sb - 1, fb);
              continue;
            }
            mbar_arrive_expect_tx(&full[s], kOzStage);
            tma_load_3d(sa_ptr, mA, kb * kSplitBK, arow, sa - 1, &full[s]);
            tma_load_3d(sa_ptr + kOzABytes, mB, kb * kSplitBK, q.col0 + tn * BN, sb - 1,
                        &full[s]);
          }
        }
      }
    }
  } else if (warp == 1 && PAIR && rank == 1) {
    // odd CTA of a pair: the even CTA issues the MMAs of both
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16_f32(PAIR ? 2 * kSplitBM : kSplitBM, BN);
      uint32_t L = 0, chunk = 0;
      bool ok = true;
      for (int u = first; u < nunits && ok; u += stride) {
        const OzakiParams &q = *prm(prob_of(u));
        const int S = q.S, KB = q.KB;
        int g0, g1;
        unit_groups(u, q, g0, g1);
        for (int gi = g0; gi < g1 && ok; ++gi) {
          int t, lo, np;
          group_of(MODE, gi, S, t, lo, np);
          const int G = np * KB;
          for (int c0 = 0; c0 < G && ok; c0 += kOzChunkStages, ++chunk) {
            const int b = chunk & 1;
            const uint32_t u = chunk >> 1;
            if (!mbar_wait(&acce[b], (u & 1) ^ 1, p.err, kErrTimeoutMma, abort_flag)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t dt = tmem + b * BN;
            const int c1 = min(G, c0 + kOzChunkStages);
            for (int idx = c0; idx < c1; ++idx, ++L) {
              const int s = L % kOzStages;
              const uint32_t r = L / kOzStages;
              if (!mbar_wait(&full[s], r & 1, p.err, kErrTimeoutFull, abort_flag)) {
                ok = false;
                break;
              }
              tc_fence_after();
              const uint32_t sa = smem_u32(smem + s * kOzStage), sb = sa + kOzABytes;
#pragma unroll
              for (int kk = 0; kk < kSplitBK / 16; ++kk) {
                if (PAIR)
                  umma_pair(dt, umma_desc_sw128(sa + kk * 32), umma_desc_sw128(sb + kk * 32),
                            idesc, (idx > c0 || kk > 0) ? 1u : 0u);
                else
                  umma_bf16(dt, umma_desc_sw128(sa + kk * 32), umma_desc_sw128(sb + kk * 32),
                            idesc, (idx > c0 || kk > 0) ? 1u : 0u);
              }
              if (PAIR)
                umma_commit_pair(&empty[s], 0x3);  // both CTAs' stage s is free
              else
                umma_commit(&empty[s]);
            }
            if (ok) {
              if (PAIR)
                umma_commit_pair(&accf[b], 0x3);
              else
                umma_commit(&accf[b]);
            }
          }
        }
      }
      // every issued MMA has completed before TMEM is released
      if (PAIR)
        umma_commit_pair(done, 0x1);
      else
        umma_commit(done);
      mbar_wait(done, 0, p.err, kErrTimeoutMma, nullptr);
    }
  } else {
    // 16 epilogue warps: lane quarter q = warp % 4, column block h (64 columns each)
    const int q = warp & 3;
    const int h = (warp - 2) >> 2;
    const int row_in_tile = q * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16) + h * kOzCols;
    uint32_t chunk = 0;
    bool ok = true;
    for (int u = first; u < nunits && ok; u += stride) {
      const int pi = prob_of(u);
      const OzakiParams &pq = *prm(pi);
      const int S = pq.S, KB = pq.KB;
      int tm, tn, g0, g1;
      unit_tile(u, pi, tm, tn);
      unit_groups(u, pq, g0, g1);
      const bool real = tm < pq.tiles_m;  // PAIR: a row tile past the end writes nothing
      const int row = tm * kSplitBM + row_in_tile;          // < Mp when real
      const int col0 = tn * BN + h * kOzCols;          // first of this warp's columns
      double *res = pq.res + (int64_t)col0 * pq.Mp + row;      // res[j * Mp] is column col0 + j
      bool res_init = false;
      const int run_limit = MODE ? kCrtRunChunks : kOzRunChunks;
      for (int gi = g0; gi < g1 && ok; ++gi) {
        int t, lo, np;
        group_of(MODE, gi, S, t, lo, np);
        const int G = np * KB;
        const int nch = (G + kOzChunkStages - 1) / kOzChunkStages;
        // residue plane of modulus gi: words of 4 consecutive columns,
        // word (col / 4) * Mp + row (the reconstruction reads one word per
        // modulus for 4 columns of a row; a warp's 32 rows store 128 bytes)
        uint32_t *plane = MODE ? reinterpret_cast<uint32_t *>(pq.rres + (int64_t)gi * pq.Mp * pq.Np) +
                                     (int64_t)(col0 >> 2) * pq.Mp + row
                               : nullptr;
        if (MODE && nch == 1) {
          // CRT form, K of this modulus in one chunk (k <= 1024): each chunk
          // sum x is an integer with |x| <= 1024 * 127^2 < 2^24, exact in FP32.
          // x mod p in FP32: q = rint(x / p) from x * (1 / p) (rounded to an
          // integer by the 1.5 * 2^23 constant; |x / p| < 2^17 and the product's
          // error below 0.01 leave q the nearest integer or its neighbour),
          // r = x - q p exact by one FMA (|r| < p), then r in [0, p).
          const int b = chunk & 1;
          const uint32_t uph = chunk >> 1;
          ++chunk;
          if (!mbar_wait(&accf[b], uph & 1, p.err, kErrTimeoutAcc, abort_flag)) { ok = false; break; }
          tc_fence_after();
          const float pf = pq.mods_f[gi], ip = pq.mods_inv[gi];
          // two halves of the warp's columns: the second half's TMEM loads
          // release the accumulator, the first half is stored meanwhile
          constexpr int kHalf = kOzCols / 2;
#pragma unroll
          for (int hf = 0; hf < 2; ++hf) {
            uint32_t v[kHalf];
#pragma unroll
            for (int g = 0; g < kHalf / 16; ++g) {
              uint32_t t16[16];
              tmem_ld16(lane_base + b * BN + hf * kHalf + g * 16, t16);
#pragma unroll
              for (int j = 0; j < 16; ++j) v[g * 16 + j] = t16[j];
            }
            tmem_ld_wait();
            if (hf == 1) {
              tc_fence_before();
              __syncwarp();
              if (lane == 0) {
                if (PAIR)
                  mbar_arrive_cluster<false>(&acce[b], 0);  // the even CTA issues the MMAs of both
                else
                  mbar_arrive(&acce[b]);
              }
            }
            if (real) {
#pragma unroll
              for (int qd = 0; qd < kHalf / 4; ++qd) {
                uint32_t w = 0;
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                  const float x = __uint_as_float(v[4 * qd + e]);
                  const float qf = fmaf(x, ip, 12582912.0f) - 12582912.0f;
                  float r = fmaf(-qf, pf, x);
                  r = r < 0.0f ? r + pf : r;
                  // r + 2^23 holds r in its low mantissa bits (0 <= r < 256)
                  w |= (__float_as_uint(r + 8388608.0f) & 0xffu) << (8 * e);
                }
                plane[(int64_t)(hf * kHalf / 4 + qd) * pq.Mp] = w;
              }
            }
          }
          continue;
        }
        const double wt = ldexp(1.0, -7 * t);
        int run[kOzCols];
#pragma unroll
        for (int j = 0; j < kOzCols; ++j) run[j] = 0;
        int since_fold = 0;
        for (int c = 0; c < nch; ++c, ++chunk) {
          const int b = chunk & 1;
          const uint32_t u = chunk >> 1;
          if (!mbar_wait(&accf[b], u & 1, p.err, kErrTimeoutAcc, abort_flag)) { ok = false; break; }
          tc_fence_after();
#pragma unroll
          for (int g = 0; g < kOzCols / 16; ++g) {
            uint32_t v[16];
            tmem_ld16(lane_base + b * BN + g * 16, v);
            tmem_ld_wait();
#pragma unroll
            for (int j = 0; j < 16; ++j)
              // integer-valued with |v| < 2^24: round-to-nearest conversion is exact
              run[g * 16 + j] += __float2int_rn(__uint_as_float(v[j]));
          }
          tc_fence_before();
          __syncwarp();
          if (lane == 0) {
            if (PAIR)
              mbar_arrive_cluster<false>(&acce[b], 0);  // the even CTA issues the MMAs of both
            else
              mbar_arrive(&acce[b]);
          }
          const bool last = (c == nch - 1);
          if (MODE && (++since_fold == run_limit || last)) {
            // CRT form: reduce the exact sums mod p; at the modulus' end store
            // the residue in [0, p) for the reconstruction kernel
            // |run| < 64 chunks x 2^24 = 2^30 < 149 * 2^23, so run + pm * 2^23 is in
            // [0, 2^32): one Barrett step (q = the quotient or one less) and an
            // unsigned-min correction give run mod pm in [0, pm)
            const unsigned pm = (unsigned)pq.mods[gi], mg = pq.mods_mg[gi], off = pm << 23;
#pragma unroll
            for (int j = 0; j < kOzCols; ++j) {
              const unsigned x = (unsigned)run[j] + off;
              const unsigned r = x - __umulhi(x, mg) * pm;
              run[j] = (int)min(r, r - pm);
            }
            if (last && real) {
#pragma unroll
              for (int qd = 0; qd < kOzCols / 4; ++qd)
                plane[(int64_t)qd * pq.Mp] = (uint32_t)run[4 * qd] |
                                            ((uint32_t)run[4 * qd + 1] << 8) |
                                            ((uint32_t)run[4 * qd + 2] << 16) |
                                            ((uint32_t)run[4 * qd + 3] << 24);
            }
            since_fold = 0;
          } else if (!MODE && (++since_fold == kOzRunChunks || last)) {
            // fold the exact group sum into the FP64 result: res += run * 2^-7t
#pragma unroll
            for (int g = 0; g < kOzCols && real; g += 8) {
              double prev[8];
#pragma unroll
              for (int j = 0; j < 8; ++j) prev[j] = res_init ? res[(int64_t)(g + j) * pq.Mp] : 0.0;
#pragma unroll
              for (int j = 0; j < 8; ++j) {
                res[(int64_t)(g + j) * pq.Mp] = fma((double)run[g + j], wt, prev[j]);
                run[g + j] = 0;
              }
            }
            res_init = true;
            since_fold = 0;
          }
        }
      }
      if (!ok) break;
      // final epilogue: C = alpha * 2^(E_i + F_j) * res + beta * C (slice form;
      // the CRT form's C update is the reconstruction kernel's)
      if (!MODE && real && row < pq.m) {
        const int ea = pq.expA[row];
#pragma unroll 1
        for (int g = 0; g < kOzCols; g += 8) {
          double rv[8], cv[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int col = col0 + g + j;
            rv[j] = res[(int64_t)(g + j) * pq.Mp];
            cv[j] = (col < pq.n) ? pq.C[(int64_t)col * pq.ldc + row] : 0.0;
          }
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int col = col0 + g + j;
            if (col < pq.n) {
              const int eb = pq.expB[col];
              const double v = (ea == kNonFiniteExp || eb == kNonFiniteExp)
                                   ? __longlong_as_double(0x7ff8000000000000LL)
                                   : scale_pow2(rv[j], ea + eb);
              const double cb = (pq.beta == 1.0) ? cv[j] : __dmul_rn(cv[j], pq.beta);
              pq.C[(int64_t)col * pq.ldc + row] = __dadd_rn(cb, __dmul_rn(pq.alpha, v));
            }
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (PAIR) cluster_sync();  // both CTAs are done with the pair's TMEM
  if (warp == 1) {
    tc_fence_after();
    if (PAIR)
      tmem_dealloc_pair(tmem, 512);
    else
      tmem_dealloc(tmem, 512);
  }
  if (PAIR) cluster_sync();  // no peer commit or arrive can still target this CTA
}

// ===========================================================================
// host side
// ===========================================================================
static int sm_count() {
  static int n = 0;
  if (!n) {
    int d = 0;
    cudaGetDevice(&d);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, d);
    if (n <= 0) n = 148;
  }
  return n;
}

static SegMap seg_map(int products, bool is_a) {
  SegMap s{};
  if (products == 3) {
    // products (lo*hi), (hi*lo), (hi*hi): small terms accumulate first
    const int a[3] = {1, 0, 0}, b[3] = {0, 1, 0};
    s.nseg = 3;
    for (int i = 0; i < 3; ++i) s.term[i] = is_a ? a[i] : b[i];
  } else {
    // all (i, j) with i + j <= 2 over terms (hi, mid, lo), smallest order first
    const int a[6] = {2, 1, 0, 1, 0, 0}, b[6] = {0, 1, 2, 0, 1, 0};
    s.nseg = 6;
    for (int i = 0; i < 6; ++i) s.term[i] = is_a ? a[i] : b[i];
  }
  return s;
}

size_t split_workspace_bytes(int kind, int m, int n, int k, int param) {
  if (m <= 0 || n <= 0 || k <= 0) return 0;
  if (kind == 2) return crt_workspace_bytes(m, n, k, param);
  const int64_t Kp = round_up(k, kSplitBK);
  if (kind == 0) {
    if (param == 0) {
      int c = 0;
      bf16x_resolve(m, n, k, &param, &c);
    }
    if (!split_products_ok(param)) return 0;
    const int64_t Mp = round_up(m, kSplitBM), Np = round_up(n, kBf16xBN);
    // scaled FP16 form: + the max |.| bit patterns and exponents of rows / columns
    const int64_t scales = param == kFp16x3 ? (Mp + Np) * 8 + 512 : 0;
    return (size_t)((Mp + Np) * split_terms(param) * Kp * 2 + 1024 + scales);
  }
  int S = param > 0 ? param : ozaki_default_slices(m, n, k);
  if (S < 2 || S > kOzakiMaxSlices) return 0;
  const int64_t Mp = round_up(m, kSplitBM), Np = round_up(n, kOzakiBN);
  return (size_t)((Mp + Np) * S * Kp * 2 + (Mp + Np) * 12 + Mp * Np * 8 + 4096);
}

int ozaki_default_slices(int m, int n, int k) {
  int S = 0;
  return tune_lookup(1, m, n, k, &S, nullptr) ? S : 8;
}

void bf16x_resolve(int m, int n, int k, int *products, int *chunk) {
  int P = 0, c = 0;
  if (!tune_lookup(0, m, n, k, &P, &c)) { P = 6; c = 0; }
  *products = P;
  *chunk = c;
}

// K blocks per TMEM accumulation chunk of the BF16xP GEMM (0 = default).
static int g_bf16x_chunk = 0;
int bf16x_chunk_kblocks() { return g_bf16x_chunk; }
void set_bf16x_chunk_kblocks(int c) { g_bf16x_chunk = c < 0 ? 0 : c; }

// Grid of the max pass over one operand (R rows of op(X), k long): one warp
// (k-contiguous rows) or one thread (row-contiguous columns) per row and k
// range; the k range doubles until the grid's y extent fits.
static void absmax_grid(bool kc, int R, int k, int *span, unsigned *gx, unsigned *gy) {
  int64_t sp = kc ? kAmaxSpanK : kAmaxSpanR;
  while ((k + sp - 1) / sp > 65535) sp *= 2;
  *span = (int)sp;
  *gx = (unsigned)(kc ? (R + 7) / 8 : (R + 255) / 256);
  *gy = (unsigned)((k + sp - 1) / sp);
}

// Per-row max |.| of op(A) and per-column max |.| of op(B), then their scale
// exponents.  amax / ex hold Mp entries for the rows of op(A), then Np for
// the columns of op(B); padding entries get exponent 0.  The completion
// counter sits in the 16 bytes after amax and is zeroed with it: one memset
// and one launch.
template <typename T>
static int scale_exponents(char ta, char tb, int m, int n, int k, const T *A, int lda, const T *B,
                           int ldb, typename AbsBits<T>::U *amax, int *ex, int64_t Mp, int64_t Np,
                           cudaStream_t st) {
  const bool an = notrans(ta), bn = notrans(tb);
  using U = typename AbsBits<T>::U;
  if (cudaMemsetAsync(amax, 0, (size_t)(Mp + Np) * sizeof(U) + 16, st) != cudaSuccess)
    return GB300_ERR_CUDA;
  AbsmaxArgs<T> p;
  // A rows are k-contiguous when transposed, B columns when not.
  p.X0 = A; p.ld0 = lda; p.R0 = m; p.kc0 = an ? 0 : 1;
  p.X1 = B; p.ld1 = ldb; p.R1 = n; p.kc1 = bn ? 1 : 0;
  unsigned gx = 1, gy = 1;
  for (int z = 0; z < 2; ++z) {
    unsigned x, y;
    absmax_grid((z ? p.kc1 : p.kc0) != 0, z ? n : m, k, z ? &p.span1 : &p.span0, &x, &y);
    gx = x > gx ? x : gx;
    gy = y > gy ? y : gy;
  }
  p.K = k; p.Mp = (int)Mp; p.first = 0; p.total = (int)(Mp + Np); p.zbase = 0;
  p.amax = amax; p.ex = ex;
  p.counter = reinterpret_cast<unsigned *>(amax + Mp + Np);
  p.nblocks = gx * gy * 2;
  row_absmax_kernel<T><<<dim3(gx, gy, 2), 256, 0, st>>>(p);
  return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
}

// The same over one operand part: rows [r0, r0 + R) of op(A) (z = 0) or
// columns of op(B) (z = 1), X pointing at the part's first row; the entries
// [r0, r0 + Rpart) of the operand's amax / ex range are written.  The counter
// (after all Mp + Np entries) is zeroed for this launch: parts on one stream
// run one after another.
template <typename T>
static int scale_exponents_part(int z, bool kc, int R, int Rpart, int r0, int k, const T *X,
                                int ldx, typename AbsBits<T>::U *amax, int *ex, int64_t Mp,
                                int64_t Np, cudaStream_t st) {
  using U = typename AbsBits<T>::U;
  U *mine = amax + (z ? Mp : 0) + r0;
  unsigned *counter = reinterpret_cast<unsigned *>(amax + Mp + Np);
  if (cudaMemsetAsync(mine, 0, (size_t)Rpart * sizeof(U), st) != cudaSuccess ||
      cudaMemsetAsync(counter, 0, sizeof(unsigned), st) != cudaSuccess)
    return GB300_ERR_CUDA;
  AbsmaxArgs<T> p;
  p.X0 = p.X1 = X; p.ld0 = p.ld1 = ldx; p.R0 = p.R1 = R; p.kc0 = p.kc1 = kc ? 1 : 0;
  unsigned gx, gy;
  absmax_grid(kc, R, k, &p.span0, &gx, &gy);
  p.span1 = p.span0;
  p.K = k; p.Mp = (int)Mp; p.zbase = z;
  p.amax = amax + r0; p.ex = ex + r0;  // z = 1 adds Mp in the kernel
  p.first = z ? (int)Mp : 0; p.total = Rpart;
  p.counter = counter;
  p.nblocks = gx * gy;
  row_absmax_kernel<T><<<dim3(gx, gy, 1), 256, 0, st>>>(p);
  return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
}

int row_scale_exponents_part(int z, bool kc, int R, int Rpart, int r0, int k, const double *X,
                             int ldx, unsigned long long *amax, int *ex, int64_t Mp, int64_t Np,
                             cudaStream_t st) {
  return scale_exponents_part<double>(z, kc, R, Rpart, r0, k, X, ldx, amax, ex, Mp, Np, st);
}

int row_scale_exponents(char ta, char tb, int m, int n, int k, const double *A, int lda,
                        const double *B, int ldb, unsigned long long *amax, int *ex, int64_t Mp,
                        int64_t Np, cudaStream_t st) {
  return scale_exponents<double>(ta, tb, m, n, k, A, lda, B, ldb, amax, ex, Mp, Np, st);
}

// ----------------------------------------------------------------- BF16xP
struct Bf16xLayout {
  int64_t Kp, Kld, Mp, Np;
  __nv_bfloat16 *Ap, *Bp;  // 16-bit terms (FP16 bit patterns in the scaled FP16 form)
  unsigned *amax;          // scaled FP16 form: max |.| of rows of op(A), columns of op(B)
  int *ex;                 //   and their scale exponents (Mp then Np entries)
};
static Bf16xLayout bf16x_layout(int m, int n, int k, int products, void *ws) {
  Bf16xLayout L;
  L.Kp = round_up(k, kSplitBK);
  L.Kld = L.Kp * split_terms(products);  // each term once
  L.Mp = round_up(m, kSplitBM);
  L.Np = round_up(n, kBf16xBN);
  L.Ap = reinterpret_cast<__nv_bfloat16 *>((reinterpret_cast<uintptr_t>(ws) + 1023) &
                                           ~uintptr_t(1023));
  L.Bp = L.Ap + L.Mp * L.Kld;
  L.amax = reinterpret_cast<unsigned *>(
      (reinterpret_cast<uintptr_t>(L.Bp + L.Np * L.Kld) + 255) & ~uintptr_t(255));
  // 16 bytes after amax: the max pass's completion counter
  L.ex = reinterpret_cast<int *>(reinterpret_cast<uint8_t *>(L.amax + L.Mp + L.Np) + 16);
  return L;
}

int split_sgemm_prepare(char ta, char tb, int m, int n, int k, const float *A, int lda,
                        const float *B, int ldb, int products, void *ws, size_t ws_bytes,
                        cudaStream_t st) {
  if (products == 0) {
    int c = 0;
    bf16x_resolve(m, n, k, &products, &c);
  }
  const int ck = check_args(ta, tb, m, n, k, lda, ldb, m > 1 ? m : 1);
  if (ck == GB300_ERR_ARG || !split_products_ok(products)) return GB300_ERR_ARG;
  if (ck < 0 || k == 0) return GB300_OK;
  const size_t need = split_workspace_bytes(0, m, n, k, products);
  if (!ws || ws_bytes < need) return GB300_ERR_WORKSPACE;
  const Bf16xLayout L = bf16x_layout(m, n, k, products, ws);
  if (L.Kld > 0x7fffffff || L.Mp > 0x7fffffff || L.Np > 0x7fffffff) return GB300_ERR_ARG;
  const bool an = notrans(ta), bn = notrans(tb);
  const bool f16 = products == kFp16x3;
  SplitArgs sa;
  sa.X0 = A; sa.ld0 = lda; sa.R0 = m; sa.kc0 = an ? 0 : 1; sa.Rp0 = (int)L.Mp;
  sa.X1 = B; sa.ld1 = ldb; sa.R1 = n; sa.kc1 = bn ? 1 : 0; sa.Rp1 = (int)L.Np;
  sa.ex0 = f16 ? L.ex : nullptr;
  sa.ex1 = f16 ? L.ex + L.Mp : nullptr;
  sa.out0 = L.Ap; sa.out1 = L.Bp;
  sa.K = k; sa.Kp = (int)L.Kp; sa.nterms = products == 6 ? 3 : 2;
  sa.ldo = L.Kld;
  sa.zbase = 0;
  const unsigned rb = row_blocks(L.Mp > L.Np ? L.Mp : L.Np);
  const dim3 grid((unsigned)(L.Kp / 64), rb, 2);
  const int vpt = f16 ? row_split_vpt(k) : 0;
  const bool fz[2] = {vpt && sa.kc0, vpt && sa.kc1};  // operands for the fused row split
  if (f16 && (fz[0] || fz[1])) {
    RowSplitArgs ra;
    ra.X0 = A; ra.X1 = B; ra.ld0 = lda; ra.ld1 = ldb; ra.R0 = m; ra.R1 = n;
    ra.Rp0 = (int)L.Mp; ra.Rp1 = (int)L.Np;
    ra.ex0 = L.ex; ra.ex1 = L.ex + L.Mp; ra.out0 = L.Ap; ra.out1 = L.Bp;
    ra.K = k; ra.Kp = (int)L.Kp; ra.ldo = L.Kld;
    ra.vec = (reinterpret_cast<uintptr_t>(A) % 16 == 0 && lda % 4 == 0 || !fz[0]) &&
             (reinterpret_cast<uintptr_t>(B) % 16 == 0 && ldb % 4 == 0 || !fz[1]);
    if (fz[0] && fz[1]) {
      ra.zbase = 0;
      row_split_launch(ra, vpt, (unsigned)(L.Mp > L.Np ? L.Mp : L.Np), 2, st);
    } else {
      // one operand fused, the other through the max pass and the tile split
      const int zf = fz[0] ? 0 : 1, zo = 1 - zf;
      ra.zbase = zf;
      row_split_launch(ra, vpt, (unsigned)(zf ? L.Np : L.Mp), 1, st);
      const int rc = scale_exponents_part<float>(
          zo, zo ? sa.kc1 != 0 : sa.kc0 != 0, zo ? n : m, (int)(zo ? L.Np : L.Mp), 0, k,
          zo ? B : A, zo ? ldb : lda, L.amax, L.ex, L.Mp, L.Np, st);
      if (rc != GB300_OK) return rc;
      sa.zbase = zo;
      split_bf16_kernel<true><<<dim3((unsigned)(L.Kp / 64), row_blocks(zo ? L.Np : L.Mp), 1), 256,
                                 0, st>>>(sa);
    }
  } else if (f16) {
    const int rc = scale_exponents<float>(ta, tb, m, n, k, A, lda, B, ldb, L.amax, L.ex, L.Mp,
                                          L.Np, st);
    if (rc != GB300_OK) return rc;
    split_bf16_kernel<true><<<grid, 256, 0, st>>>(sa);
  } else {
    split_bf16_kernel<false><<<grid, 256, 0, st>>>(sa);
  }
  return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
}

int split_sgemm_prepare_part(int z, char t, int m, int n, int k, const float *X, int ldx, int r0,
                             int rows, int products, void *ws, size_t ws_bytes, cudaStream_t st) {
  if (products == 0) {
    int c = 0;
    bf16x_resolve(m, n, k, &products, &c);
  }
  const int align = z ? kBf16xBN : kSplitBM, R = z ? n : m;
  if (!split_products_ok(products) || m <= 0 || n <= 0 || k <= 0 || r0 < 0 || rows <= 0 ||
      r0 % align || r0 + rows > R || ldx < 1)
    return GB300_ERR_ARG;
  const size_t need = split_workspace_bytes(0, m, n, k, products);
  if (!ws || ws_bytes < need) return GB300_ERR_WORKSPACE;
  const Bf16xLayout L = bf16x_layout(m, n, k, products, ws);
  // op(A) rows are k-contiguous when A is transposed, op(B) columns when B is not
  const bool kc = z ? notrans(t) : !notrans(t);
  const float *Xp = kc ? X + (int64_t)r0 * ldx : X + r0;
  const int Rpart = (int)round_up(rows, align);
  const bool f16 = products == kFp16x3;
  SplitArgs sa;
  sa.X0 = sa.X1 = Xp; sa.ld0 = sa.ld1 = ldx; sa.R0 = sa.R1 = rows;
  sa.kc0 = sa.kc1 = kc ? 1 : 0; sa.Rp0 = sa.Rp1 = Rpart;
  int *ex = f16 ? L.ex + (z ? L.Mp : 0) + r0 : nullptr;
  sa.ex0 = sa.ex1 = ex;
  __nv_bfloat16 *out = (z ? L.Bp : L.Ap) + (int64_t)r0 * L.Kld;
  sa.out0 = sa.out1 = out;
  sa.K = k; sa.Kp = (int)L.Kp; sa.nterms = products == 6 ? 3 : 2;
  sa.ldo = L.Kld;
  sa.zbase = z;
  const dim3 grid((unsigned)(L.Kp / 64), row_blocks(Rpart), 1);
  const int vpt = f16 && kc ? row_split_vpt(k) : 0;
  if (vpt) {  // k-contiguous rows: the fused max pass and split
    RowSplitArgs ra;
    ra.X0 = ra.X1 = Xp; ra.ld0 = ra.ld1 = ldx; ra.R0 = ra.R1 = rows; ra.Rp0 = ra.Rp1 = Rpart;
    ra.ex0 = ra.ex1 = ex; ra.out0 = ra.out1 = out;
    ra.K = k; ra.Kp = (int)L.Kp; ra.ldo = L.Kld; ra.zbase = z;
    ra.vec = reinterpret_cast<uintptr_t>(Xp) % 16 == 0 && ldx % 4 == 0;
    row_split_launch(ra, vpt, (unsigned)Rpart, 1, st);
  } else if (f16) {
    const int rc = scale_exponents_part<float>(z, kc, rows, Rpart, r0, k, Xp, ldx, L.amax, L.ex,
                                               L.Mp, L.Np, st);
    if (rc != GB300_OK) return rc;
    split_bf16_kernel<true><<<grid, 256, 0, st>>>(sa);
  } else {
    split_bf16_kernel<false><<<grid, 256, 0, st>>>(sa);
  }
  return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
}

// Persistent launch of a tile kernel: one CTA per SM (plain), or 2-CTA
// clusters running pair MMAs on row-tile pairs (pair).
template <typename P>
static int persistent_launch(void (*plain)(const CUtensorMap, const CUtensorMap, P),
                             void (*clustered)(const CUtensorMap, const CUtensorMap, P),
                             int threads, int smem, const CUtensorMap &tA, const CUtensorMap &tB,
                             const P &p, int tiles_m, int tiles_n, bool pair, cudaStream_t st) {
  if (!pair) {
    if (cudaFuncSetAttribute(plain, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
        cudaSuccess)
      return GB300_ERR_CUDA;
    const int ntiles = tiles_m * tiles_n;
    const int grid = ntiles < sm_count() ? ntiles : sm_count();
    plain<<<grid, threads, smem, st>>>(tA, tB, p);
    return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
  }
  if (cudaFuncSetAttribute(clustered, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
      cudaSuccess)
    return GB300_ERR_CUDA;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const int npairs = ((tiles_m + 1) / 2) * tiles_n;
  int max_clusters = sm_count() / 2;
  cfg.gridDim = dim3((unsigned)(2 * max_clusters));
  int occ = 0;
  if (cudaOccupancyMaxActiveClusters(&occ, clustered, &cfg) == cudaSuccess && occ > 0 &&
      occ < max_clusters)
    max_clusters = occ;
  cfg.gridDim = dim3((unsigned)(2 * (npairs < max_clusters ? npairs : max_clusters)));
  if (cudaLaunchKernelEx(&cfg, clustered, tA, tB, p) != cudaSuccess) return GB300_ERR_CUDA;
  return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
}

// Tile width of the split GEMMs: 128 for outputs at most 128 columns wide
// (the grouped batches' small shapes: a 256-wide tile would be at most half
// used), else 256.  128-wide tiles run 1.4-1.6x longer per column (measured
// from 2048 to 8192, all split forms), so they pay only where they halve the
// padding.  A tuned width of the shape class, or GB300_TUNE_TILE_N, wins.
static int g_tile_n = 0;
int split_tile_n(int kind, int m, int n, int k) {
  if (g_tile_n == 128 || g_tile_n == 256) return g_tile_n;
  const int tuned = tune_tile_n(kind, m, n, k);
  if (tuned) return tuned;
  (void)m;
  return n <= 128 ? 128 : 256;
}
void set_split_tile_n(int v) { g_tile_n = v; }
int split_tile_override() { return g_tile_n; }

// Cluster mode of the tensor-core GEMMs (BF16xP and Ozaki / CRT) with two or
// more row tiles: pair MMAs on 2-CTA clusters (kernel mode 2) or one CTA per
// tile (mode 0).  Same results bit for bit, so the autotuner times both per
// shape class.  Order: GB300_TUNE_PAIR_MMA, the tuned mode of the shape
// class, pair MMAs.
static int g_pair_mma = 0;  // 0: none, 1: pair MMAs, 2: one CTA per tile
void set_pair_mma(int v) { g_pair_mma = v; }
int pair_mma_override() { return g_pair_mma; }
// Work units of the CRT GEMM: 0 = by shape, 1 = whole tiles (all moduli),
// 2 = one modulus of one tile.  Same results bit for bit.
static int g_modulus_split = 0;
void set_modulus_split(int v) { g_modulus_split = v; }
int modulus_split_override() { return g_modulus_split; }
static bool use_pair_mma(int kind, int m, int n, int k) {
  const int v = g_pair_mma ? g_pair_mma : tune_pair_mma(kind, m, n, k);
  return v != 2;
}

// The split GEMM's operand maps over the rows / columns of L: k x T x rows
// (K within a term block, the term, the row; T = Kld / Kp terms), so rows
// past h (w) and K past k read as zeros and the padding is never read.
static bool bf16x_maps(const Bf16xLayout &L, int h, int w, int k, CUtensorMap *tA,
                       CUtensorMap *tB, int box_b) {
  const int64_t T = L.Kld / L.Kp;
  return encode_3d(tA, L.Ap, 2, k, T, h, L.Kp, L.Kld, kSplitBK, 1, kSplitBM) &&
         encode_3d(tB, L.Bp, 2, k, T, w, L.Kp, L.Kld, kSplitBK, 1, box_b);
}

// The map of C in 128 x 32 boxes (L2 prefetch, staged C), where C's base and column
// stride are 16-byte multiples (a tensor map's rule); else no prefetch.
static void bf16x_c_prefetch(Bf16xParams &p) {
  p.c_pf = ((uintptr_t)p.C % 16 == 0 && p.ldc % 4 == 0 &&
            encode_2d(&p.tmC, p.C, 4, p.m, p.n, p.ldc, kSplitBM, 32, false))
               ? 1
               : 0;
}

// L: the layout of the rows / columns this launch covers; (tm, tn, k): the
// problem whose shape class picks the cluster mode.
template <bool F16, int BN>
static int bf16x_launch(const Bf16xLayout &L, Bf16xParams p, int tm, int tn, int k,
                        cudaStream_t st) {
  // pair MMAs on row-tile pairs (2-CTA clusters) when there are two or more row tiles
  const bool pair = L.Mp / kSplitBM >= 2 && use_pair_mma(0, tm, tn, k);
  CUtensorMap tA{}, tB{};
  if (!bf16x_maps(L, p.m, p.n, k, &tA, &tB, pair ? BN / 2 : BN)) return GB300_ERR_CUDA;
  p.tiles_n = (p.n + BN - 1) / BN;
  bf16x_c_prefetch(p);
  if constexpr (BN == 256) {
    // short K: staged C; m a multiple of 4, because the TMA store of a box
    // clips the rows at 16 bytes (an m x n map with m = 170 wrote rows 170 and
    // 171 of the ld padding), while the plain epilogue stores row by row
    if (pair && p.c_pf && p.m % 4 == 0 && p.kblocks <= kBxStagedMaxKBlocks)
      return persistent_launch<Bf16xParams>(
          bf16x_gemm_kernel<0, F16, BN>, bf16x_gemm_kernel<2, F16, BN, false, true>, kBxThreads,
          BxSmem<2, BN, true>::kBytes, tA, tB, p, p.tiles_m, p.tiles_n, true, st);
  }
  return persistent_launch<Bf16xParams>(
      bf16x_gemm_kernel<0, F16, BN>, bf16x_gemm_kernel<2, F16, BN>, kBxThreads,
      pair ? ClusterTile<2, BN>::kSmem : ClusterTile<0, BN>::kSmem, tA, tB, p, p.tiles_m,
      p.tiles_n, pair, st);
}

int split_sgemm_run(int m, int n, int k, float alpha, float beta, float *C, int ldc, int products,
                    const void *ws, size_t ws_bytes, cudaStream_t st, unsigned *err, int chunk0) {
  return split_sgemm_run_block(m, n, k, 0, m, 0, n, alpha, beta, C, ldc, products, ws, ws_bytes,
                               st, err, chunk0);
}

// The layout and kernel parameters of the C block (i0, h) x (j0, w) of a
// prepared problem (the tile width is set by the launch).  products and
// chunk0 as resolved by the caller.
static int bf16x_block_setup(int m, int n, int k, int i0, int h, int j0, int w, float alpha,
                             float beta, float *C, int ldc, int products, int chunk0,
                             const void *ws, size_t ws_bytes, unsigned *err, Bf16xLayout &L,
                             Bf16xParams &p) {
  const size_t need = split_workspace_bytes(0, m, n, k, products);
  if (!ws || ws_bytes < need) return GB300_ERR_WORKSPACE;
  const Bf16xLayout Lf = bf16x_layout(m, n, k, products, const_cast<void *>(ws));
  // the block's rows of A' and columns of B' (tile-aligned offsets)
  L = Lf;
  L.Ap = Lf.Ap + (int64_t)i0 * Lf.Kld;
  L.Bp = Lf.Bp + (int64_t)j0 * Lf.Kld;
  L.Mp = round_up(h, kSplitBM);
  L.Np = round_up(w, kBf16xBN);
  std::memset(&p, 0, sizeof(p));
  p.m = h; p.n = w;
  p.tiles_m = (int)(L.Mp / kSplitBM);
  p.tiles_n = 0;  // set by the launch for its tile width
  const int skb = (int)(L.Kp / kSplitBK);  // K blocks of one segment
  p.kblocks = split_segments(products) * skb;
  p.skb = skb;
  {
    const SegMap sa = seg_map(products == kFp16x3 ? 3 : products, true),
                 sb = seg_map(products == kFp16x3 ? 3 : products, false);
    p.segA = p.segB = 0u;
    for (int sg = 0; sg < sa.nseg; ++sg) {
      p.segA |= (unsigned)sa.term[sg] << (4 * sg);
      p.segB |= (unsigned)sb.term[sg] << (4 * sg);
    }
  }
  {
    // segments by order (i + j) of their cross product, see seg_map():
    // P = 6: 2 2 2 1 1 0; P = 3 and the scaled FP16 form: 1 1 0.  Segments
    // of one order share chunks, so short K (k = 256: 4 blocks a segment)
    // gets few TMEM drains per tile.
    const int c0 = chunk0 > 0                  ? chunk0
                   : bf16x_chunk_kblocks() > 0 ? bf16x_chunk_kblocks()
                                               : kBxDefaultChunk;
    // order-1 products weigh 2^-8 of the result with BF16 terms, 2^-11 with the
    // scaled FP16 terms: the latter tolerate 8x longer chunks at the same error
    const int c1 = (products == kFp16x3 ? 32 : 4) * c0;
    if (split_segments(products) == 6) {
      p.nruns = 3;
      p.run_end0 = 3 * skb; p.run_chunk0 = 0;   // order 2: unchunked
      p.run_end1 = 5 * skb; p.run_chunk1 = c1;  // order 1
      p.run_end2 = 6 * skb; p.run_chunk2 = c0;  // hi*hi
    } else {
      p.nruns = 2;
      p.run_end0 = 2 * skb; p.run_chunk0 = c1;
      p.run_end1 = 3 * skb; p.run_chunk1 = c0;
      p.run_end2 = 3 * skb; p.run_chunk2 = c0;
    }
  }
  p.alpha = alpha; p.beta = beta; p.C = C + i0 + (int64_t)j0 * ldc; p.ldc = ldc; p.err = err;
  p.rescale_chunk = -1;
  p.rescale = 1.0f;
  p.expA = p.expB = nullptr;
  if (products == kFp16x3) {
    // segments 0 and 1 (lo*hi, hi*lo, run 0) carry 2^11 x their value; their
    // chunks come first, so the running sums are scaled once when run 1 starts
    p.rescale_chunk = (p.run_end0 + p.run_chunk0 - 1) / p.run_chunk0;
    p.rescale = 1.0f / 2048.0f;
    p.expA = Lf.ex + i0;
    p.expB = Lf.ex + Lf.Mp + j0;
  }
  return GB300_OK;
}

int split_sgemm_run_block(int m, int n, int k, int i0, int h, int j0, int w, float alpha,
                          float beta, float *C, int ldc, int products, const void *ws,
                          size_t ws_bytes, cudaStream_t st, unsigned *err, int chunk0) {
  if (products == 0) {
    int c = 0;
    bf16x_resolve(m, n, k, &products, &c);
    if (chunk0 == 0) chunk0 = c;
  }
  if (m < 0 || n < 0 || k < 0 || ldc < (m > 1 ? m : 1) || !split_products_ok(products) ||
      i0 < 0 || j0 < 0 || h < 0 || w < 0 || i0 % kSplitBM || j0 % kBf16xBN || i0 + h > m ||
      j0 + w > n)
    return GB300_ERR_ARG;
  if (h == 0 || w == 0) return GB300_OK;
  if (alpha == 0.0f || k == 0)
    return plain_sgemm('N', 'N', h, w, 0, alpha, nullptr, h > 1 ? h : 1, nullptr, 1, beta,
                       C + i0 + (int64_t)j0 * ldc, ldc, st, err);
  Bf16xLayout L;
  Bf16xParams p;
  const int rc = bf16x_block_setup(m, n, k, i0, h, j0, w, alpha, beta, C, ldc, products, chunk0,
                                   ws, ws_bytes, err, L, p);
  if (rc != GB300_OK) return rc;
  const int bn = split_tile_n(0, m, n, k);
  if (products == kFp16x3)
    return bn == 128 ? bf16x_launch<true, 128>(L, p, m, n, k, st)
                     : bf16x_launch<true, 256>(L, p, m, n, k, st);
  return bn == 128 ? bf16x_launch<false, 128>(L, p, m, n, k, st)
                   : bf16x_launch<false, 256>(L, p, m, n, k, st);
}

// ---------------------------------------------------------- grouped launches
// The grouped batch's GEMMs in one persistent launch per kind: every problem's
// operands are prepared in its own workspace first, then one launch runs the
// concatenated tiles of all problems (128 x 128 tiles, one CTA per tile), each
// tile with its problem's tensor maps and parameters from a device table.
// The tiles of a problem are computed exactly as by its own call (same K
// order and chunks), so results are bit-identical to the per-problem calls.
constexpr int kGroupBN = 128;  // tile width of grouped launches (least padding)
size_t bf16x_group_entry_bytes() { return sizeof(GBxProblem); }
size_t ozaki_group_entry_bytes() { return sizeof(GOzProblem); }

int bf16x_group_entry(int m, int n, int k, float alpha, float beta, float *C, int ldc,
                      int products, const void *ws, size_t ws_bytes, unsigned *err, int unit0,
                      void *entry, int *units) {
  if (m <= 0 || n <= 0 || k <= 0 || alpha == 0.0f || ldc < m ||
      (products != 6 && products != 3))
    return GB300_ERR_ARG;
  Bf16xLayout L;
  GBxProblem e;
  std::memset(&e, 0, sizeof(e));
  const int rc = bf16x_block_setup(m, n, k, 0, m, 0, n, alpha, beta, C, ldc, products, 0, ws,
                                   ws_bytes, err, L, e.prm);
  if (rc != GB300_OK) return rc;
  if (!bf16x_maps(L, m, n, k, &e.tmA, &e.tmB, kGroupBN)) return GB300_ERR_CUDA;
  e.prm.tiles_n = (n + kGroupBN - 1) / kGroupBN;
  bf16x_c_prefetch(e.prm);
  e.unit0 = unit0;
  *units = e.prm.tiles_m * e.prm.tiles_n;
  std::memcpy(entry, &e, sizeof(e));
  return GB300_OK;
}

// table: nprob entries in device memory, in the order of their unit0.
template <typename P>
static int group_launch(void (*kern)(const CUtensorMap, const CUtensorMap, P), int threads,
                        int smem, const P &p, cudaStream_t st) {
  if (p.total_units <= 0) return GB300_OK;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
      cudaSuccess)
    return GB300_ERR_CUDA;
  const CUtensorMap unused{};  // each problem's maps come from the table
  const int grid = p.total_units < sm_count() ? p.total_units : sm_count();
  kern<<<grid, threads, smem, st>>>(unused, unused, p);
  return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
}

int bf16x_group_launch(const void *table, int nprob, int total_units, cudaStream_t st,
                       unsigned *err) {
  Bf16xParams p;
  std::memset(&p, 0, sizeof(p));
  p.grp = table; p.nprob = nprob; p.total_units = total_units; p.err = err;
  return group_launch<Bf16xParams>(bf16x_gemm_kernel<0, false, kGroupBN, true>, kBxThreads,
                                   ClusterTile<0, kGroupBN>::kSmem, p, st);
}

int split_sgemm(char ta, char tb, int m, int n, int k, float alpha, const float *A, int lda,
                const float *B, int ldb, float beta, float *C, int ldc, int products, void *ws,
                size_t ws_bytes, cudaStream_t st, unsigned *err, int chunk0) {
  if (products == 0) {
    int c = 0;
    bf16x_resolve(m, n, k, &products, &c);
    if (chunk0 == 0) chunk0 = c;
  }
  const int ck = check_args(ta, tb, m, n, k, lda, ldb, ldc);
  if (ck == GB300_ERR_ARG || !split_products_ok(products)) return GB300_ERR_ARG;
  if (ck < 0) return GB300_OK;
  if (alpha == 0.0f || k == 0)  // no products to form: the plain path's beta handling
    return plain_sgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, st, err);
  int rc = split_sgemm_prepare(ta, tb, m, n, k, A, lda, B, ldb, products, ws, ws_bytes, st);
  if (rc != GB300_OK) return rc;
  return split_sgemm_run(m, n, k, alpha, beta, C, ldc, products, ws, ws_bytes, st, err, chunk0);
}

// ----------------------------------------------------------------- Ozaki
struct OzakiLayout {
  int64_t Kp, Mp, Np;
  __nv_bfloat16 *As, *Bs;
  unsigned long long *amaxA, *amaxB;
  int *expA, *expB;
  double *res;
};
static OzakiLayout ozaki_layout(int m, int n, int k, int S, void *ws) {
  OzakiLayout L;
  L.Kp = round_up(k, kSplitBK);
  L.Mp = round_up(m, kSplitBM);
  L.Np = round_up(n, kOzakiBN);
  uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(ws) + 1023) &
                                              ~uintptr_t(1023));
  L.As = reinterpret_cast<__nv_bfloat16 *>(base);
  L.Bs = L.As + S * L.Mp * L.Kp;
  L.amaxA = reinterpret_cast<unsigned long long *>(L.Bs + S * L.Np * L.Kp);
  L.amaxB = L.amaxA + L.Mp;
  // 16 bytes after amaxB: the max pass's completion counter
  L.expA = reinterpret_cast<int *>(reinterpret_cast<uint8_t *>(L.amaxB + L.Np) + 16);
  L.expB = L.expA + L.Mp;
  L.res = reinterpret_cast<double *>(
      (reinterpret_cast<uintptr_t>(L.expB + L.Np) + 255) & ~uintptr_t(255));
  return L;
}


int ozaki_prepare(char ta, char tb, int m, int n, int k, const double *A, int lda, const double *B,
                  int ldb, int slices, void *ws, size_t ws_bytes, cudaStream_t st) {
  const int ck = check_args(ta, tb, m, n, k, lda, ldb, m > 1 ? m : 1);
  const int S = slices > 0 ? slices : ozaki_default_slices(m, n, k);
  if (ck == GB300_ERR_ARG || S < 2 || S > kOzakiMaxSlices) return GB300_ERR_ARG;
  if (ck < 0 || k == 0) return GB300_OK;
  const size_t need = split_workspace_bytes(1, m, n, k, S);
  if (!ws || ws_bytes < need) return GB300_ERR_WORKSPACE;
  const OzakiLayout L = ozaki_layout(m, n, k, S, ws);
  if (S * L.Mp > 0x7fffffff || S * L.Np > 0x7fffffff || L.Kp > 0x7fffffff) return GB300_ERR_ARG;
  const bool an = notrans(ta), bn = notrans(tb);
  const int rc = row_scale_exponents(ta, tb, m, n, k, A, lda, B, ldb, L.amaxA, L.expA, L.Mp,
                                     L.Np, st);
  if (rc != GB300_OK) return rc;
  OperandPair op;
  op.X0 = A; op.ld0 = lda; op.R0 = m; op.kc0 = an ? 0 : 1; op.Rp0 = (int)L.Mp;
  op.X1 = B; op.ld1 = ldb; op.R1 = n; op.kc1 = bn ? 1 : 0; op.Rp1 = (int)L.Np;
  op.ex0 = L.expA; op.ex1 = L.expB; op.out0 = L.As; op.out1 = L.Bs;
  op.K = k; op.Kp = (int)L.Kp;
  ozaki_slice_kernel<<<dim3((unsigned)(L.Kp / 64), row_blocks(L.Mp > L.Np ? L.Mp : L.Np), 2), 256,
                       0, st>>>(op, S);
  return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
}

int ozaki_run(int m, int n, int k, double alpha, double beta, double *C, int ldc, int slices,
              const void *ws, size_t ws_bytes, cudaStream_t st, unsigned *err) {
  const int S = slices > 0 ? slices : ozaki_default_slices(m, n, k);
  if (m < 0 || n < 0 || k < 0 || ldc < (m > 1 ? m : 1) || S < 2 || S > kOzakiMaxSlices)
    return GB300_ERR_ARG;
  if (m == 0 || n == 0) return GB300_OK;
  if (alpha == 0.0 || k == 0)
    return plain_dgemm('N', 'N', m, n, 0, alpha, nullptr, m > 1 ? m : 1, nullptr, 1, beta, C, ldc,
                       st, err);
  const size_t need = split_workspace_bytes(1, m, n, k, S);
  if (!ws || ws_bytes < need) return GB300_ERR_WORKSPACE;
  const OzakiLayout L = ozaki_layout(m, n, k, S, const_cast<void *>(ws));
  OzakiGemmArgs a;
  a.m = m; a.n = n; a.k = k; a.S = S; a.mode = 0;
  a.m_all = m; a.n_all = n;
  a.Mp = L.Mp; a.Np = L.Np; a.Kp = L.Kp;
  a.As = L.As; a.Bs = L.Bs;
  a.alpha = alpha; a.beta = beta; a.C = C; a.ldc = ldc;
  a.expA = L.expA; a.expB = L.expB; a.res = L.res; a.rres = nullptr; a.mods = nullptr;
  return ozaki_gemm_launch(a, st, err);
}

// The slice / residue GEMM's operand maps: S blocks of Mp (Np) rows x Kp, of
// which rows [0, m_all) ([0, n_all)) and K [0, k) hold data; everything past
// them reads as zeros, so the padding is never read from memory.
static bool ozaki_maps(const OzakiGemmArgs &a, CUtensorMap *tA, CUtensorMap *tB, int box_b) {
  const int64_t ma = a.m_all > 0 ? a.m_all : a.Mp, na = a.n_all > 0 ? a.n_all : a.Np;
  return encode_3d(tA, a.As, 2, a.k, ma, a.S, a.Kp, a.Mp * a.Kp, kSplitBK, kSplitBM, 1) &&
         encode_3d(tB, a.Bs, 2, a.k, na, a.S, a.Kp, a.Np * a.Kp, kSplitBK, box_b, 1);
}

template <int BN>
static int ozaki_launch_bn(const OzakiGemmArgs &a, OzakiParams p, cudaStream_t st) {
  // pair MMAs on row-tile pairs (2-CTA clusters) when there are two or more row tiles
  const bool pair = p.tiles_m >= 2 && use_pair_mma(a.mode ? 2 : 1, a.m, a.n, a.k);
  CUtensorMap tA{}, tB{};
  if (!ozaki_maps(a, &tA, &tB, pair ? BN / 2 : BN)) return GB300_ERR_CUDA;
  p.tiles_n = (p.n + BN - 1) / BN;
  // CRT form: one modulus per work unit when the tiles alone fill fewer than
  // four waves (a 2048^2 output has 128 tiles for 152 SMs)
  const int stride = pair ? sm_count() / 2 : sm_count();
  const int ntu = (pair ? (p.tiles_m + 1) / 2 : p.tiles_m) * p.tiles_n;
  const int mode = modulus_split_override();
  p.gsplit = !p.mode || mode == 1 ? 1 : (mode == 2 || ntu < 4 * stride) ? p.S : 1;
  const int smem = pair ? ClusterTile<2, BN>::kSmem : ClusterTile<0, BN>::kSmem;
  if (p.mode)
    return persistent_launch<OzakiParams>(ozaki_gemm_kernel<0, BN, 1>,
                                          ozaki_gemm_kernel<2, BN, 1>, kOzThreads, smem, tA, tB,
                                          p, p.tiles_m, p.tiles_n * p.gsplit, pair, st);
  return persistent_launch<OzakiParams>(ozaki_gemm_kernel<0, BN, 0>, ozaki_gemm_kernel<2, BN, 0>,
                                        kOzThreads, smem, tA, tB, p, p.tiles_m,
                                        p.tiles_n * p.gsplit, pair, st);
}

static void ozaki_params(const OzakiGemmArgs &a, unsigned *err, OzakiParams &p) {
  std::memset(&p, 0, sizeof(p));
  p.m = a.m; p.n = a.n;
  p.tiles_m = (a.m + kSplitBM - 1) / kSplitBM;  // Mp / 128 for a whole problem
  p.row0 = a.row0; p.col0 = a.col0;
  p.tiles_n = 0;  // set by the launch for its tile width
  p.S = a.S; p.KB = (int)(a.Kp / kSplitBK);
  p.mode = a.mode;
  p.Mp = (int)a.Mp; p.Np = (int)a.Np;
  p.alpha = a.alpha; p.beta = a.beta; p.C = a.C; p.ldc = a.ldc;
  p.expA = a.expA; p.expB = a.expB; p.res = a.res; p.rres = a.rres; p.err = err;
  for (int i = 0; i < kCrtMaxModuli; ++i) {
    p.mods[i] = (a.mode && i < a.S) ? a.mods[i] : 1;
    p.mods_mg[i] = p.mods[i] > 1 ? (unsigned)((1ull << 32) / (unsigned)p.mods[i]) : 0u;
    p.mods_f[i] = (float)p.mods[i];
    p.mods_inv[i] = 1.0f / (float)p.mods[i];
  }
}

int ozaki_gemm_launch(const OzakiGemmArgs &a, cudaStream_t st, unsigned *err) {
  if (a.S < 1 || a.S > (a.mode ? kCrtMaxModuli : kOzakiMaxSlices)) return GB300_ERR_ARG;
  OzakiParams p;
  ozaki_params(a, err, p);
  return split_tile_n(a.mode ? 2 : 1, a.m, a.n, a.k) == 128 ? ozaki_launch_bn<128>(a, p, st)
                                                           : ozaki_launch_bn<256>(a, p, st);
}

// One CRT problem (mode 1, a whole problem) of a grouped launch: its table
// entry, whole-tile units (all moduli of a tile in one unit).
int ozaki_group_entry(const OzakiGemmArgs &a, unsigned *err, int unit0, void *entry, int *units) {
  if (a.mode != 1 || a.S < 2 || a.S > kCrtMaxModuli || a.row0 || a.col0 || a.m <= 0 || a.n <= 0)
    return GB300_ERR_ARG;
  GOzProblem e;
  std::memset(&e, 0, sizeof(e));
  ozaki_params(a, err, e.prm);
  if (!ozaki_maps(a, &e.tmA, &e.tmB, kGroupBN)) return GB300_ERR_CUDA;
  e.prm.tiles_n = (a.n + kGroupBN - 1) / kGroupBN;
  e.prm.gsplit = 1;
  e.unit0 = unit0;
  *units = e.prm.tiles_m * e.prm.tiles_n;
  std::memcpy(entry, &e, sizeof(e));
  return GB300_OK;
}

int ozaki_group_launch(const void *table, int nprob, int total_units, cudaStream_t st,
                       unsigned *err) {
  OzakiParams p;
  std::memset(&p, 0, sizeof(p));
  p.mode = 1; p.gsplit = 1;
  p.grp = table; p.nprob = nprob; p.total_units = total_units; p.err = err;
  return group_launch<OzakiParams>(ozaki_gemm_kernel<0, kGroupBN, 1, true>, kOzThreads,
                                   ClusterTile<0, kGroupBN>::kSmem, p, st);
}

int ozaki_dgemm(char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
                const double *B, int ldb, double beta, double *C, int ldc, int slices, void *ws,
                size_t ws_bytes, cudaStream_t st, unsigned *err) {
  const int ck = check_args(ta, tb, m, n, k, lda, ldb, ldc);
  const int S = slices > 0 ? slices : ozaki_default_slices(m, n, k);
  if (ck == GB300_ERR_ARG || S < 2 || S > kOzakiMaxSlices) return GB300_ERR_ARG;
  if (ck < 0) return GB300_OK;
  if (alpha == 0.0 || k == 0)
    return plain_dgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, st, err);
  int rc = ozaki_prepare(ta, tb, m, n, k, A, lda, B, ldb, S, ws, ws_bytes, st);
  if (rc != GB300_OK) return rc;
  return ozaki_run(m, n, k, alpha, beta, C, ldc, S, ws, ws_bytes, st, err);
}

}  // namespace gb300
