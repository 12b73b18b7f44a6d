// crt.cu -- the CRT (modular-integer) form of the FP64 GEMM on the BF16 tensor
// pipe: a tensor-core form of the reference's dgemm_ (wjc404/GEMM_AVX2
// src/gemm_driver.c:118; same operand semantics), after the published Ozaki
// scheme II (Ozaki, Uchino & Imamura 2025).
//
//   1. Rows of op(A) and columns of op(B) are scaled by powers of two and
//      truncated to integers of at most b bits: A'_ik = trunc(a_ik 2^(b-E_i)).
//   2. Their symmetric residues modulo N pairwise coprime odd moduli <= 255
//      (|r| <= 127: exact in BF16, products < 2^14 exact in FP32) are written
//      as N K-major BF16 blocks (crt_residue_kernel).
//   3. One exact integer GEMM per modulus on tcgen05 (the slice GEMM of
//      tc_gemm.cu in its CRT mode) gives P = A'B' mod p_i for every i.
//   4. crt_reconstruct_kernel rebuilds P in (-M/2, M/2), M = p_1 ... p_N, with
//      192-bit integer arithmetic (X = sum r_i w_i, then X mod M), converts it
//      to FP64 with one rounding and scales by 2^(E_i + F_j - 2b).
//   b is the largest integer with 2 k (2^b - 1)^2 < M.  The only errors are
//   the truncations of step 1 (b bits relative to the row / column maximum);
//   N moduli cost N tensor GEMMs where the slice form needs S(S+1)/2 for
//   about 7S bits.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>

#include "plain_gemm.h"
#include "split_gemm.h"
#include "split_tiles.cuh"

namespace gb300 {

namespace {

// pairwise coprime, odd, <= 255 (255 = 3*5*17, 253 = 11*23, 247 = 13*19,
// 217 = 7*31, the rest prime)
constexpr int kModuli[kCrtMaxModuli] = {255, 253, 251, 247, 241, 239, 233, 229,
                                        227, 223, 217, 211, 199, 197, 193, 191,
                                        181, 179, 173, 167, 163, 157, 151, 149};
constexpr int kCrtDefaultModuli = 16;

// ------------------------------------------------------------------ residues
struct CrtModParams {
  int N, b;
  unsigned p[kCrtMaxModuli];
  unsigned mg[kCrtMaxModuli];   // floor(2^32 / p)
  unsigned c21[kCrtMaxModuli];  // 2^21 mod p
  unsigned c42[kCrtMaxModuli];   // 2^42 mod p
  unsigned pw32[kCrtMaxModuli];  // 2^32 mod p
};

// x mod p for x < 2^32 (Barrett with mg = floor(2^32/p): q is the quotient or
// one less, so one correction suffices).
__device__ __forceinline__ unsigned mod32(unsigned x, unsigned p, unsigned mg) {
  const unsigned q = __umulhi(x, mg);
  const unsigned r = x - q * p;
  return r >= p ? r - p : r;
}

// BF16 bit patterns of two integers |v| < 2^22 packed in one word: 1.5 * 2^23
// + v is exact in FP32, so subtracting 1.5 * 2^23 leaves v exactly; |v| <= 127
// keeps the top 16 bits exact.
__device__ __forceinline__ unsigned bf16x2_of_small_ints(int v0, int v1) {
  const float f0 = __int_as_float(0x4B400000 + v0) - 12582912.0f;
  const float f1 = __int_as_float(0x4B400000 + v1) - 12582912.0f;
  return __byte_perm(__float_as_uint(f0), __float_as_uint(f1), 0x7632);
}

// The N residue blocks of one thread's 8 values.  s = y0 + y1 (2^21 mod p) +
// y2 (2^42 mod p) < 2^31 is y mod p up to multiples of p; Barrett with
// mg = floor(2^32 / p) leaves r in [0, 2p), and min(r, r - p) (unsigned) maps
// it into [0, p).  The symmetric residue of -y is minus that of y (p odd).
// SLOW: some value needs the factor 2^t mod p (b > 63, or a row whose largest
// value is subnormal).
template <bool SLOW>
__device__ __forceinline__ void residue_blocks(const unsigned (&y0)[8], const unsigned (&y1)[8],
                                               const unsigned (&y2)[8], const int (&tp)[8],
                                               const int (&sgn)[8], const CrtModParams &mp,
                                               uint4 *dst, int64_t step) {
  for (int i = 0; i < mp.N; ++i) {
    const unsigned p = mp.p[i], mg = mp.mg[i], c21 = mp.c21[i], c42 = mp.c42[i];
    const unsigned half = p >> 1;
    int v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const unsigned sm = y0[j] + y1[j] * c21 + y2[j] * c42;
      unsigned r = sm - __umulhi(sm, mg) * p;
      r = min(r, r - p);
      if (SLOW && tp[j] >= 0) {
        const int t = tp[j];
        unsigned p2 = mod32(1u << (t & 31), p, mg);
        for (int w32 = t >> 5; w32 > 0; --w32) p2 = mod32(p2 * mp.pw32[i], p, mg);
        r = mod32(r * p2, p, mg);
      }
      const int sym = (int)r - (r > half ? (int)p : 0);
      v[j] = (sym ^ sgn[j]) - sgn[j];
    }
    dst[i * step] = make_uint4(bf16x2_of_small_ints(v[0], v[1]), bf16x2_of_small_ints(v[2], v[3]),
                               bf16x2_of_small_ints(v[4], v[5]), bf16x2_of_small_ints(v[6], v[7]));
  }
}

// Symmetric residues of A' = trunc(x 2^(b - e)) for N moduli, 8 consecutive k
// of one row per thread, as BF16, block i at dst[i * step] (uint4 units).
// |x| = M 2^base with M the 53-bit significand, so |x| 2^(b-e) = M 2^t,
// t = b - e + base.  The integer y = M 2^t (right shift: truncation; left
// shift up to 10: exact, < 2^63) or, for t > 10, y = M with the factor
// 2^t mod p (2^(t mod 32) times t/32 factors of 2^32 mod p) applied after, is
// cut into 21-bit chunks y0 + y1 2^21 + y2 2^42;
// y mod p = (y0 + y1 (2^21 mod p) + y2 (2^42 mod p)) mod p, a sum below 2^31.
// Both operands in one launch (blockIdx.z).
__global__ void __launch_bounds__(256, 3)
    crt_residue_kernel(const __grid_constant__ OperandPair op,
                       const __grid_constant__ CrtModParams mp) {
  const int z = blockIdx.z + op.zbase;
  const double *__restrict__ X = z ? op.X1 : op.X0;
  const int ld = z ? op.ld1 : op.ld0, R = z ? op.R1 : op.R0, kcontig = z ? op.kc1 : op.kc0;
  const int Rp = z ? op.Rp1 : op.Rp0, K = op.K, Kp = op.Kp;
  const int *__restrict__ ex = z ? op.ex1 : op.ex0;
  __nv_bfloat16 *__restrict__ out = static_cast<__nv_bfloat16 *>(z ? op.out1 : op.out0);
  __shared__ double tile[32][65];
  const int k0 = blockIdx.x * 64;
  const int r = threadIdx.x >> 3, kq = (threadIdx.x & 7) * 8;
  const int64_t plane = z ? op.plane1 : op.plane0;
  const int64_t step = (plane ? plane : (int64_t)Rp * Kp) / 8;  // one residue block, in uint4
  // rows past R are never read (the GEMM's maps end at the problem's rows),
  // so only row blocks holding data are written
  for (int r0 = blockIdx.y * 32; r0 < R; r0 += gridDim.y * 32) {
    load_tile_32x64<double>(X, ld, R, K, kcontig != 0, r0, k0, tile);
    __syncthreads();
    const int gr = r0 + r;
    const int e = (gr < R) ? ex[gr] : 0;
    const bool bad = (e == kNonFiniteExp);  // row of Inf/NaN: zeros, the result is NaN
    uint4 *dst = reinterpret_cast<uint4 *>(out + (int64_t)gr * Kp + k0 + kq);
    unsigned y0[8], y1[8], y2[8];
    int tp[8];   // t when t > 10 (the 2^t factor), else -1
    int sgn[8];  // -1 for negative values, else 0
    bool slow = false;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const unsigned long long u = (unsigned long long)__double_as_longlong(tile[r][kq + j]);
      const int be = (int)((u >> 52) & 0x7ff);
      const unsigned long long M =
          bad ? 0ull : ((u & 0xfffffffffffffull) | (be ? (1ull << 52) : 0ull));
      const int t = mp.b - e + ((be ? be : 1) - 1075);
      const unsigned long long y =
          t < 0 ? (t > -64 ? M >> (-t) : 0ull) : (t <= 10 ? M << t : M);
      y0[j] = (unsigned)y & 0x1fffff;
      y1[j] = (unsigned)(y >> 21) & 0x1fffff;
      y2[j] = (unsigned)(y >> 42);
      tp[j] = t > 10 ? t : -1;
      slow |= t > 10;
      sgn[j] = -(int)(u >> 63);
    }
    if (slow)
      residue_blocks<true>(y0, y1, y2, tp, sgn, mp, dst, step);
    else
      residue_blocks<false>(y0, y1, y2, tp, sgn, mp, dst, step);
    __syncthreads();  // the tile is refilled for the next row block
  }
}

// ------------------------------------------------------------- reconstruction
constexpr int kLimbs = 6;  // 32-bit limbs of M and the weights (M < 2^188)
struct CrtRecParams {
  int N, m, n, Mp, Np, two_b;
  int topshift;  // bitlength(M) - 40
  float inv_mt;  // 2^30 / (M >> topshift)
  unsigned w[kCrtMaxModuli][kLimbs];  // CRT weights, little-endian 32-bit limbs
  unsigned M[kLimbs], half[kLimbs];   // M and (M - 1) / 2
  double alpha, beta;
  double *C;
  int ldc;
};

// The CRT reconstruction of one element from its residues r[0..N), then the C
// update: X = sum r_g w_g in carry-save 64-bit limb accumulators (r < 2^8,
// limbs < 2^32, at most 24 terms: no overflow), P = X - q M with q ~ X / M
// estimated from X's top bits in FP32 (floor(X / M) or one more), the symmetric
// residue from |P|, and one rounding to FP64.
// r_g is byte e of word[g]; the weights of unused moduli (g >= N) are zero.
// L = 32-bit limbs of M and the weights (M < 2^(32 L)); X needs L + 1.
template <int L>
__device__ __forceinline__ void crt_value(const unsigned (&word)[kCrtMaxModuli], int e,
                                          const CrtRecParams &rp, bool &negative,
                                          unsigned long long &top_out, int &pos_out) {
  unsigned long long acc[L];
#pragma unroll
  for (int l = 0; l < L; ++l) acc[l] = 0ull;
#pragma unroll
  for (int g = 0; g < kCrtMaxModuli; ++g) {
    if (g >= rp.N) break;  // uniform across the grid
    const unsigned r = __byte_perm(word[g], 0u, 0x4440u + (unsigned)e);
#pragma unroll
    for (int l = 0; l < L; ++l) acc[l] += (unsigned long long)r * rp.w[g][l];
  }
  unsigned X[L + 1];  // X < 2^13 M
  {
    unsigned long long c = 0;
#pragma unroll
    for (int l = 0; l < L; ++l) {
      c += acc[l];
      X[l] = (unsigned)c;
      c >>= 32;
    }
    X[L] = (unsigned)c;
  }
  // 53 bits of X from bit topshift (X >> topshift < 2^53)
  unsigned long long xt;
  {
    const int li = rp.topshift >> 5, o = rp.topshift & 31;
    unsigned long long lo = 0, hi = 0;
#pragma unroll
    for (int l = 0; l < L + 1; ++l) {
      if (l == li) lo = X[l];
      if (l == li + 1) lo |= (unsigned long long)X[l] << 32;
      if (l == li + 2) hi = X[l];
    }
    xt = o ? (lo >> o) | (hi << (64 - o)) : lo;
  }
  // q ~ X / M from the top 23 bits of xt (X >> (topshift + 30) < 2^23, exact in
  // FP32 by the 2^23 constant), rounded to an integer by the same constant:
  // the truncation costs < 2^-9 and the FP32 rounding < 2^-11 of a unit, so q
  // is floor(X / M) or one more; all on the FP32 / integer pipes (conversions
  // from 64-bit integers would occupy the FP64 pipe)
  const float xf = __uint_as_float(0x4B000000u | (unsigned)(xt >> 30)) - 8388608.0f;
  const unsigned q = __float_as_uint(fmaf(xf, rp.inv_mt, 8388608.0f)) & 0x7fffffu;
  // P = X - q M, two's complement over L + 1 limbs
  unsigned P[L + 1];
  {
    long long c = 0;
#pragma unroll
    for (int l = 0; l < L + 1; ++l) {
      const unsigned long long qm = l < L ? (unsigned long long)q * rp.M[l] : 0ull;
      c += (long long)X[l] - (long long)(qm & 0xffffffffull);
      P[l] = (unsigned)c;
      c = (c >> 32) - (long long)(qm >> 32);
    }
  }
  // q is floor(X / M) or one more (the estimate is within 0.0025 of X / M), so
  // P lies in [-M, M).  The symmetric residue Y of X mod M (in (-M/2, M/2],
  // where P_mod > (M - 1) / 2 stands for P_mod - M) then follows from a = |P|:
  // over = a > (M - 1) / 2; |Y| = over ? M - a : a; Y < 0 iff (P < 0) != over.
  const bool pneg = (int)P[L] < 0;
  unsigned a[L];
  {
    // a = pneg ? -P : P over L limbs (a <= M < 2^(32 L))
    unsigned long long c = pneg ? 1ull : 0ull;
    const unsigned flip = pneg ? 0xffffffffu : 0u;
#pragma unroll
    for (int l = 0; l < L; ++l) {
      c += (unsigned long long)(P[l] ^ flip);
      a[l] = (unsigned)c;
      c >>= 32;
    }
  }
  bool over = false;
#pragma unroll
  for (int l = L - 1; l >= 0; --l)
    if (a[l] != rp.half[l]) { over = a[l] > rp.half[l]; break; }
  unsigned mg[L];
  if (over) {
    long long c = 0;
#pragma unroll
    for (int l = 0; l < L; ++l) {
      c += (long long)rp.M[l] - (long long)a[l];
      mg[l] = (unsigned)c;
      c >>= 32;
    }
  } else {
#pragma unroll
    for (int l = 0; l < L; ++l) mg[l] = a[l];
  }
  negative = pneg != over;
  // magnitude -> FP64 with one rounding: the top 64 bits, the rest as a sticky bit
  int tl = -1;
#pragma unroll
  for (int l = L - 1; l >= 0; --l)
    if (tl < 0 && mg[l]) tl = l;
  unsigned long long top = 0;
  int pos = 0;
  if (tl >= 2) {
    unsigned a2 = 0, a1 = 0, a0 = 0;
    bool sticky = false;
#pragma unroll
    for (int l = 0; l < L; ++l) {
      if (l == tl) a2 = mg[l];
      else if (l == tl - 1) a1 = mg[l];
      else if (l == tl - 2) a0 = mg[l];
      else if (l < tl - 2 && mg[l]) sticky = true;
    }
    const int lz = __clz(a2);
    const unsigned long long w64 = ((unsigned long long)a2 << 32) | a1;
    top = lz ? (w64 << lz) | ((unsigned long long)a0 >> (32 - lz)) : w64;
    if ((lz ? (a0 << lz) : a0) != 0 || sticky) top |= 1ull;  // a0's bits below the window
    pos = 32 * (tl - 1) - lz;
  } else if (tl == 1) {
    top = ((unsigned long long)mg[1] << 32) | mg[0];
  } else if (tl == 0) {
    top = mg[0];
  }
  top_out = top;
  pos_out = pos;
}

// (-1)^neg * top * 2^e2 as FP64: round top to 53 bits (to nearest, ties to
// even; bit 0 may be a sticky bit) and assemble the bits when the result is a
// normal number, otherwise the same rounding through the FP64 pipe (which runs
// at 1 TFLOP/s here, so the common case stays on the integer pipe).
__device__ __forceinline__ double crt_compose(unsigned long long top, int e2, bool neg) {
  if (top == 0) return 0.0;
  const int lz = __clzll((long long)top);
  const unsigned long long t = top << lz;  // leading bit at 63
  int e = e2 + 63 - lz;                    // value = (t / 2^63) 2^e
  unsigned long long mant = t >> 11;
  const unsigned long long rem = t & 0x7ffull;
  if (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) {
    ++mant;
    if (mant >> 53) {
      mant >>= 1;
      ++e;
    }
  }
  if (e < -1022 || e > 1023) {
    const double v = scale_pow2(__ull2double_rn(top), e2);
    return neg ? -v : v;
  }
  const unsigned long long bits = (neg ? (1ull << 63) : 0ull) |
                                  ((unsigned long long)(e + 1023) << 52) |
                                  (mant & 0xfffffffffffffull);
  return __longlong_as_double((long long)bits);
}

// One row and 4 consecutive columns of C per thread: a residue plane holds
// words of 4 columns (word (col / 4) Mp + row), so one 32-bit load per
// modulus brings the thread's residues, and a warp's 32 rows load 128
// contiguous bytes and update 32 contiguous elements of each column of C.
// (m n / 4 threads in a 1-D grid: below 2^39 for every valid C.)
template <int L>
__global__ void __launch_bounds__(256)
    crt_reconstruct_kernel(const uint8_t *__restrict__ rres, const int *__restrict__ expA,
                           const int *__restrict__ expB, const __grid_constant__ CrtRecParams rp) {
  const int64_t plane_w = (int64_t)rp.Mp * rp.Np / 4;  // words per residue plane
  // thread t: row t % m of column group t / m, so a warp covers 32 rows of
  // one group (or, for m < 32, several groups) and small outputs fill whole
  // warps
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int ngroups = (rp.n + 3) / 4;
  if (t >= (int64_t)rp.m * ngroups) return;
  const int i = (int)(t % rp.m), jg = (int)(t / rp.m);
  const int ea = expA[i];
  const unsigned *base = reinterpret_cast<const unsigned *>(rres);
  {
    const unsigned *src = base + (int64_t)jg * rp.Mp + i;
    unsigned word[kCrtMaxModuli];
#pragma unroll
    for (int g = 0; g < kCrtMaxModuli; ++g) word[g] = g < rp.N ? src[g * plane_w] : 0u;
#pragma unroll 1
    for (int e = 0; e < 4; ++e) {
      const int j = 4 * jg + e;
      if (j >= rp.n) break;
      bool neg;
      unsigned long long top;
      int pos;
      crt_value<L>(word, e, rp, neg, top, pos);
      const int eb = expB[j];
      double v;
      if (ea == kNonFiniteExp || eb == kNonFiniteExp) {
        v = __longlong_as_double(0x7ff8000000000000LL);
      } else {
        v = crt_compose(top, pos + ea + eb - rp.two_b, neg);
      }
      double *c = rp.C + (int64_t)j * rp.ldc + i;
      // beta C + alpha v rounded as written, as the model in the oracle
      const double cb = (rp.beta == 1.0) ? *c : __dmul_rn(*c, rp.beta);
      *c = __dadd_rn(cb, __dmul_rn(rp.alpha, v));
    }
  }
}

// ------------------------------------------------------------------ host side
// Small fixed-width unsigned integers for the CRT constants (5 x 64 bits).
struct Big {
  uint64_t l[5] = {0, 0, 0, 0, 0};
};
Big big_from(uint64_t v) {
  Big b;
  b.l[0] = v;
  return b;
}
Big big_mul(const Big &a, uint64_t s) {
  Big r;
  unsigned __int128 c = 0;
  for (int i = 0; i < 5; ++i) {
    const unsigned __int128 t = (unsigned __int128)a.l[i] * s + c;
    r.l[i] = (uint64_t)t;
    c = t >> 64;
  }
  return r;
}
uint64_t big_divmod(Big &a, uint64_t d) {  // a /= d, returns the remainder
  unsigned __int128 rem = 0;
  for (int i = 4; i >= 0; --i) {
    const unsigned __int128 cur = (rem << 64) | a.l[i];
    a.l[i] = (uint64_t)(cur / d);
    rem = cur % d;
  }
  return (uint64_t)rem;
}
int big_cmp(const Big &a, const Big &b) {
  for (int i = 4; i >= 0; --i)
    if (a.l[i] != b.l[i]) return a.l[i] < b.l[i] ? -1 : 1;
  return 0;
}
Big big_sub(const Big &a, const Big &b) {
  Big r;
  uint64_t bo = 0;
  for (int i = 0; i < 5; ++i) {
    const uint64_t d = a.l[i] - b.l[i];
    const uint64_t b1 = a.l[i] < b.l[i];
    r.l[i] = d - bo;
    bo = b1 | (d < bo);
  }
  return r;
}
Big big_shl(const Big &a, int s) {
  Big r;
  const int w = s / 64, o = s % 64;
  for (int i = 4; i >= 0; --i) {
    uint64_t v = 0;
    if (i - w >= 0) v = a.l[i - w] << o;
    if (o && i - w - 1 >= 0) v |= a.l[i - w - 1] >> (64 - o);
    r.l[i] = v;
  }
  return r;
}
int big_bitlength(const Big &a) {
  for (int i = 4; i >= 0; --i)
    if (a.l[i]) return 64 * i + 64 - __builtin_clzll(a.l[i]);
  return 0;
}
Big modulus_product(int N) {
  Big M = big_from(1);
  for (int i = 0; i < N; ++i) M = big_mul(M, (uint64_t)kModuli[i]);
  return M;
}
int64_t inv_mod(int64_t a, int64_t p) {  // a^-1 mod p, gcd(a, p) = 1
  int64_t t = 0, nt = 1, r = p, nr = a % p;
  while (nr) {
    const int64_t q = r / nr;
    int64_t tmp = t - q * nt;
    t = nt;
    nt = tmp;
    tmp = r - q * nr;
    r = nr;
    nr = tmp;
  }
  return t < 0 ? t + p : t;
}

struct CrtLayout {
  int64_t Kp, Mp, Np;
  __nv_bfloat16 *As, *Bs;
  unsigned long long *amax;
  int *ex;
  uint8_t *rres;
};
CrtLayout crt_layout(int m, int n, int k, int N, void *ws) {
  CrtLayout L;
  L.Kp = (k + kSplitBK - 1) / kSplitBK * kSplitBK;
  L.Mp = (m + kSplitBM - 1) / kSplitBM * kSplitBM;
  L.Np = (n + kOzakiBN - 1) / kOzakiBN * kOzakiBN;
  uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(ws) + 1023) &
                                              ~uintptr_t(1023));
  L.As = reinterpret_cast<__nv_bfloat16 *>(base);
  L.Bs = L.As + N * L.Mp * L.Kp;
  L.amax = reinterpret_cast<unsigned long long *>(L.Bs + N * L.Np * L.Kp);
  // 16 bytes after amax: the max pass's completion counter
  L.ex = reinterpret_cast<int *>(reinterpret_cast<uint8_t *>(L.amax + L.Mp + L.Np) + 16);
  L.rres = reinterpret_cast<uint8_t *>(
      (reinterpret_cast<uintptr_t>(L.ex + L.Mp + L.Np) + 255) & ~uintptr_t(255));
  return L;
}

// Constants of the residue kernel for N moduli and b-bit scaled integers.
CrtModParams mod_params(int N, int b) {
  CrtModParams mp;
  std::memset(&mp, 0, sizeof(mp));
  mp.N = N;
  mp.b = b;
  for (int i = 0; i < kCrtMaxModuli; ++i) {
    const unsigned p = (unsigned)kModuli[i];
    mp.p[i] = p;
    mp.mg[i] = (unsigned)((1ull << 32) / p);
    mp.c21[i] = (unsigned)((1ull << 21) % p);
    mp.c42[i] = (unsigned)((1ull << 42) % p);
    mp.pw32[i] = (unsigned)((1ull << 32) % p);
  }
  return mp;
}

unsigned row_blocks(int64_t Rp) { return (unsigned)(Rp / 32 < 65535 ? Rp / 32 : 65535); }

// moduli 0: the autotuned count for the shape class, else the default
int resolve_moduli(int moduli, int m = 0, int n = 0, int k = 0) {
  if (moduli > 0) return moduli;
  int N = 0;
  if (m > 0 && n > 0 && k > 0 && tune_lookup(2, m, n, k, &N, nullptr)) return N;
  return kCrtDefaultModuli;
}

}  // namespace

int crt_default_moduli(int m, int n, int k) { return resolve_moduli(0, m, n, k); }

int crt_bits_for(int moduli, int k) {
  const int N = resolve_moduli(moduli);
  if (N < 1 || N > kCrtMaxModuli) return 0;
  const Big M = modulus_product(N);  // < 2^188
  const uint64_t twok = 2 * (uint64_t)(k > 1 ? k : 1);
  int b = 0;
  while (b < 120) {  // largest b with 2 k (2^b - 1)^2 < M
    const int nb = b + 1;
    // (2^nb - 1)^2 = 2^(2 nb) - 2^(nb + 1) + 1, at most 2^240: 2k times it fits 320 bits
    Big sq = big_sub(big_shl(big_from(1), 2 * nb), big_shl(big_from(1), nb + 1));
    uint64_t c = 1;
    for (int i = 0; i < 5 && c; ++i) {
      sq.l[i] += c;
      c = sq.l[i] == 0;
    }
    if (big_cmp(big_mul(sq, twok), M) >= 0) break;
    b = nb;
  }
  return b;
}

size_t crt_workspace_bytes(int m, int n, int k, int moduli) {
  if (m <= 0 || n <= 0 || k <= 0) return 0;
  const int N = resolve_moduli(moduli, m, n, k);
  if (N < 2 || N > kCrtMaxModuli) return 0;
  const int64_t Kp = (k + kSplitBK - 1) / kSplitBK * kSplitBK;
  const int64_t Mp = (m + kSplitBM - 1) / kSplitBM * kSplitBM;
  const int64_t Np = (n + kOzakiBN - 1) / kOzakiBN * kOzakiBN;
  return (size_t)((Mp + Np) * N * Kp * 2 + (Mp + Np) * 12 + N * Mp * Np + 2048);
}

int crt_prepare(char ta, char tb, int m, int n, int k, const double *A, int lda, const double *B,
                int ldb, int moduli, void *ws, size_t ws_bytes, cudaStream_t st) {
  const int ck = check_args(ta, tb, m, n, k, lda, ldb, m > 1 ? m : 1);
  const int N = resolve_moduli(moduli, m, n, k);
  if (ck == GB300_ERR_ARG || N < 2 || N > kCrtMaxModuli) return GB300_ERR_ARG;
  if (ck < 0 || k == 0) return GB300_OK;
  const int b = crt_bits_for(N, k);
  if (b < 1) return GB300_ERR_ARG;  // too few moduli for this k
  const size_t need = crt_workspace_bytes(m, n, k, N);
  if (!ws || ws_bytes < need) return GB300_ERR_WORKSPACE;
  const CrtLayout L = crt_layout(m, n, k, N, ws);
  if (N * L.Mp > 0x7fffffff || N * L.Np > 0x7fffffff || L.Kp > 0x7fffffff) return GB300_ERR_ARG;
  // 1. scale exponents of the rows of op(A) and columns of op(B)
  const int rc =
      row_scale_exponents(ta, tb, m, n, k, A, lda, B, ldb, L.amax, L.ex, L.Mp, L.Np, st);
  if (rc != GB300_OK) return rc;
  // 2. residues
  const CrtModParams mp = mod_params(N, b);
  const bool an = notrans(ta), bn = notrans(tb);
  OperandPair op;
  op.X0 = A; op.ld0 = lda; op.R0 = m; op.kc0 = an ? 0 : 1; op.Rp0 = (int)L.Mp;
  op.X1 = B; op.ld1 = ldb; op.R1 = n; op.kc1 = bn ? 1 : 0; op.Rp1 = (int)L.Np;
  op.ex0 = L.ex; op.ex1 = L.ex + L.Mp; op.out0 = L.As; op.out1 = L.Bs;
  op.K = k; op.Kp = (int)L.Kp;
  crt_residue_kernel<<<dim3((unsigned)(L.Kp / 64), row_blocks(L.Mp > L.Np ? L.Mp : L.Np), 2), 256,
                       0, st>>>(op, mp);
  return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
}

int crt_prepare_part(int z, char t, int m, int n, int k, const double *X, int ldx, int r0,
                     int rows, int moduli, void *ws, size_t ws_bytes, cudaStream_t st) {
  const int N = resolve_moduli(moduli, m, n, k);
  const int align = z ? kOzakiBN : kSplitBM, R = z ? n : m;
  if (N < 2 || N > kCrtMaxModuli || m <= 0 || n <= 0 || k <= 0 || r0 < 0 || rows <= 0 ||
      r0 % align || r0 + rows > R || ldx < 1)
    return GB300_ERR_ARG;
  const int b = crt_bits_for(N, k);
  if (b < 1) return GB300_ERR_ARG;
  const size_t need = crt_workspace_bytes(m, n, k, N);
  if (!ws || ws_bytes < need) return GB300_ERR_WORKSPACE;
  const CrtLayout L = crt_layout(m, n, k, N, ws);
  // op(A) rows are k-contiguous when A is transposed, op(B) columns when B is not
  const bool kc = z ? notrans(t) : !notrans(t);
  const double *Xp = kc ? X + (int64_t)r0 * ldx : X + r0;
  const int Rpart = (rows + align - 1) / align * align;
  int rc = row_scale_exponents_part(z, kc, rows, Rpart, r0, k, Xp, ldx, L.amax, L.ex, L.Mp, L.Np,
                                    st);
  if (rc != GB300_OK) return rc;
  OperandPair op;
  op.X0 = op.X1 = Xp; op.ld0 = op.ld1 = ldx; op.R0 = op.R1 = rows;
  op.kc0 = op.kc1 = kc ? 1 : 0; op.Rp0 = op.Rp1 = Rpart;
  op.ex0 = op.ex1 = L.ex + (z ? L.Mp : 0) + r0;
  op.out0 = op.out1 = (z ? L.Bs : L.As) + (int64_t)r0 * L.Kp;
  op.K = k; op.Kp = (int)L.Kp;
  op.zbase = z;
  op.plane0 = op.plane1 = (z ? L.Np : L.Mp) * L.Kp;
  crt_residue_kernel<<<dim3((unsigned)(L.Kp / 64), row_blocks(Rpart), 1), 256, 0, st>>>(
      op, mod_params(N, b));
  return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
}

int crt_run(int m, int n, int k, double alpha, double beta, double *C, int ldc, int moduli,
            const void *ws, size_t ws_bytes, cudaStream_t st, unsigned *err) {
  return crt_run_block(m, n, k, 0, m, 0, n, alpha, beta, C, ldc, moduli, ws, ws_bytes, st, err);
}

namespace {

// The residue GEMM's arguments for the C block (i0, h) x (j0, w) of a
// prepared problem (N moduli, b-bit scaled integers).
int crt_block_args(int m, int n, int k, int i0, int h, int j0, int w, double alpha, double beta,
                   double *C, int ldc, int N, const void *ws, size_t ws_bytes, OzakiGemmArgs &a,
                   int &b) {
  b = crt_bits_for(N, k);
  if (b < 1) return GB300_ERR_ARG;
  const size_t need = crt_workspace_bytes(m, n, k, N);
  if (!ws || ws_bytes < need) return GB300_ERR_WORKSPACE;
  const CrtLayout L = crt_layout(m, n, k, N, const_cast<void *>(ws));
  // the block's residues: plane g, column j0 + j, row i0 + i in the word
  // g Mp Np / 4 + ((j0 + j) / 4) Mp + i0 + i (j0 is a multiple of 256)
  a.m = h; a.n = w; a.k = k; a.S = N; a.mode = 1;
  a.m_all = m; a.n_all = n;
  a.Mp = L.Mp; a.Np = L.Np; a.Kp = L.Kp;
  a.As = L.As; a.Bs = L.Bs;
  a.row0 = i0; a.col0 = j0;
  a.alpha = alpha; a.beta = beta; a.C = C + i0 + (int64_t)j0 * ldc; a.ldc = ldc;
  a.expA = L.ex + i0; a.expB = L.ex + L.Mp + j0;
  a.res = nullptr;
  a.rres = L.rres + ((int64_t)(j0 >> 2) * L.Mp + i0) * 4;
  a.mods = kModuli;
  return GB300_OK;
}

// Reconstruction of the block of a (after its residue GEMM) and the C update.
int crt_reconstruct_launch(const OzakiGemmArgs &a, int b, cudaStream_t st) {
  const int N = a.S, h = a.m, w = a.n;
  CrtRecParams rp;
  std::memset(&rp, 0, sizeof(rp));
  rp.N = N; rp.m = h; rp.n = w; rp.Mp = (int)a.Mp; rp.Np = (int)a.Np; rp.two_b = 2 * b;
  const Big M = modulus_product(N);
  auto limbs32 = [](const Big &x, unsigned *out) {
    for (int l = 0; l < kLimbs; ++l) out[l] = (unsigned)(x.l[l / 2] >> (32 * (l % 2)));
  };
  for (int g = 0; g < N; ++g) {
    Big Mi = M;
    const uint64_t pg = (uint64_t)kModuli[g];
    big_divmod(Mi, pg);
    Big t = Mi;
    const uint64_t mi_mod = big_divmod(t, pg);
    const Big wg = big_mul(Mi, (uint64_t)inv_mod((int64_t)mi_mod, (int64_t)pg));  // < M
    limbs32(wg, rp.w[g]);
  }
  Big half = big_sub(M, big_from(1));
  big_divmod(half, 2);
  limbs32(M, rp.M);
  limbs32(half, rp.half);
  const int bl = big_bitlength(M);
  rp.topshift = bl - 40;
  {
    Big mt = M;
    for (int s = 0; s < rp.topshift; ++s) big_divmod(mt, 2);
    rp.inv_mt = (float)(1073741824.0 / (double)mt.l[0]);
  }
  rp.alpha = a.alpha; rp.beta = a.beta; rp.C = a.C; rp.ldc = a.ldc;
  const uint8_t *rres = a.rres;
  const int *expA = a.expA, *expB = a.expB;
  const int64_t threads = (int64_t)h * ((w + 3) / 4);
  const dim3 grid((unsigned)((threads + 255) / 256));
  // limbs of M: 4 up to 16 moduli, 5 up to 20, 6 up to 24
  const int limbs = (bl + 31) / 32 < 2 ? 2 : (bl + 31) / 32;
  switch (limbs) {
    case 2: crt_reconstruct_kernel<2><<<grid, 256, 0, st>>>(rres, expA, expB, rp); break;
    case 3: crt_reconstruct_kernel<3><<<grid, 256, 0, st>>>(rres, expA, expB, rp); break;
    case 4: crt_reconstruct_kernel<4><<<grid, 256, 0, st>>>(rres, expA, expB, rp); break;
    case 5: crt_reconstruct_kernel<5><<<grid, 256, 0, st>>>(rres, expA, expB, rp); break;
    default: crt_reconstruct_kernel<6><<<grid, 256, 0, st>>>(rres, expA, expB, rp); break;
  }
  return cudaGetLastError() == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
}

}  // namespace

int crt_run_block(int m, int n, int k, int i0, int h, int j0, int w, double alpha, double beta,
                  double *C, int ldc, int moduli, const void *ws, size_t ws_bytes,
                  cudaStream_t st, unsigned *err) {
  const int N = resolve_moduli(moduli, m, n, k);
  if (m < 0 || n < 0 || k < 0 || ldc < (m > 1 ? m : 1) || N < 2 || N > kCrtMaxModuli ||
      i0 < 0 || j0 < 0 || h < 0 || w < 0 || i0 % kSplitBM || j0 % kOzakiBN || i0 + h > m ||
      j0 + w > n)
    return GB300_ERR_ARG;
  if (h == 0 || w == 0) return GB300_OK;
  if (alpha == 0.0 || k == 0)
    return plain_dgemm('N', 'N', h, w, 0, alpha, nullptr, h > 1 ? h : 1, nullptr, 1, beta,
                       C + i0 + (int64_t)j0 * ldc, ldc, st, err);
  OzakiGemmArgs a;
  int b = 0;
  int rc = crt_block_args(m, n, k, i0, h, j0, w, alpha, beta, C, ldc, N, ws, ws_bytes, a, b);
  if (rc != GB300_OK) return rc;
  // 3. one exact integer GEMM per modulus
  rc = ozaki_gemm_launch(a, st, err);
  if (rc != GB300_OK) return rc;
  // 4. reconstruction and the C update
  return crt_reconstruct_launch(a, b, st);
}

// Grouped launches: the table entry of a prepared problem's residue GEMM, and
// its reconstruction once the grouped GEMM has run (alpha != 0, k > 0).
int crt_group_entry(int m, int n, int k, double alpha, double beta, double *C, int ldc,
                    int moduli, const void *ws, size_t ws_bytes, unsigned *err, int unit0,
                    void *entry, int *units) {
  const int N = resolve_moduli(moduli, m, n, k);
  if (m <= 0 || n <= 0 || k <= 0 || alpha == 0.0 || ldc < m || N < 2 || N > kCrtMaxModuli)
    return GB300_ERR_ARG;
  OzakiGemmArgs a;
  int b = 0;
  const int rc = crt_block_args(m, n, k, 0, m, 0, n, alpha, beta, C, ldc, N, ws, ws_bytes, a, b);
  if (rc != GB300_OK) return rc;
  return ozaki_group_entry(a, err, unit0, entry, units);
}

int crt_group_reconstruct(int m, int n, int k, double alpha, double beta, double *C, int ldc,
                          int moduli, const void *ws, size_t ws_bytes, cudaStream_t st) {
  const int N = resolve_moduli(moduli, m, n, k);
  if (m <= 0 || n <= 0 || k <= 0 || alpha == 0.0 || ldc < m || N < 2 || N > kCrtMaxModuli)
    return GB300_ERR_ARG;
  OzakiGemmArgs a;
  int b = 0;
  const int rc = crt_block_args(m, n, k, 0, m, 0, n, alpha, beta, C, ldc, N, ws, ws_bytes, a, b);
  if (rc != GB300_OK) return rc;
  return crt_reconstruct_launch(a, b, st);
}

int crt_dgemm(char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
              const double *B, int ldb, double beta, double *C, int ldc, int moduli, void *ws,
              size_t ws_bytes, cudaStream_t st, unsigned *err) {
  const int ck = check_args(ta, tb, m, n, k, lda, ldb, ldc);
  if (ck != GB300_OK) return ck < 0 ? GB300_OK : ck;
  const int N = resolve_moduli(moduli, m, n, k);
  if (N < 2 || N > kCrtMaxModuli) return GB300_ERR_ARG;
  if (alpha == 0.0 || k == 0)
    return plain_dgemm('N', 'N', m, n, 0, alpha, nullptr, m > 1 ? m : 1, nullptr, 1, beta, C, ldc,
                       st, err);
  int rc = crt_prepare(ta, tb, m, n, k, A, lda, B, ldb, N, ws, ws_bytes, st);
  if (rc != GB300_OK) return rc;
  return crt_run(m, n, k, alpha, beta, C, ldc, N, ws, ws_bytes, st, err);
}

}  // namespace gb300
