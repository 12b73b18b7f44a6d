// split_tiles.cuh -- device helpers shared by the split-form prepare kernels
// (tc_gemm.cu, crt.cu): the coalesced 32 x 64 tile read of op(X), the per-row
// scale exponent and exact power-of-two scaling (FP64 and FP32).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace gb300 {

// Read op(X) (an R x K view of a column-major matrix) in 32 x 64 tiles through
// shared memory so that both the read and the K-major write are coalesced
// whatever the transpose.  256 threads.
template <typename T>
__device__ __forceinline__ void load_tile_32x64(const T *__restrict__ X, int ld, int R, int K,
                                                bool kcontig, int r0, int k0, T (*tile)[65]) {
  const int tid = threadIdx.x;  // 256 threads
  if (kcontig) {  // element (r, k) at X[k + r*ld]: read along k
#pragma unroll
    for (int p = 0; p < 8; ++p) {
      const int r = p * 4 + (tid >> 6), k = tid & 63;
      const int gr = r0 + r, gk = k0 + k;
      tile[r][k] = (gr < R && gk < K) ? X[(int64_t)gr * ld + gk] : T(0);
    }
  } else {  // element (r, k) at X[r + k*ld]: read along r
#pragma unroll
    for (int p = 0; p < 8; ++p) {
      const int r = tid & 31, k = p * 8 + (tid >> 5);
      const int gr = r0 + r, gk = k0 + k;
      tile[r][k] = (gr < R && gk < K) ? X[gr + (int64_t)gk * ld] : T(0);
    }
  }
}

// The two FP64 operands of a slice / residue pass, launched together:
// blockIdx.z = 0 is op(A) (R = m rows), 1 is op(B) read as its n x k transpose.
struct OperandPair {
  const double *X0, *X1;
  int ld0, ld1, R0, R1, kc0, kc1, Rp0, Rp1;
  const int *ex0, *ex1;  // row exponents
  void *out0, *out1;     // 16-bit blocks of Rp rows x Kp
  int K, Kp;
  // a launch over one operand part (CRT residues): blockIdx.z + zbase is the
  // operand, and the blocks of the whole operand are plane elements apart
  // (0: Rp x Kp)
  int zbase = 0;
  int64_t plane0 = 0, plane1 = 0;
};

// Scale exponent of a row: 2^-E * max|x| < 1.  Non-finite rows return a marker.
constexpr int kNonFiniteExp = 0x40000000;
__device__ __forceinline__ int row_exponent(unsigned long long amax_bits) {
  const double m = __longlong_as_double((long long)amax_bits);
  if (!(m <= 1.7976931348623157e308)) return kNonFiniteExp;  // Inf or NaN
  if (m == 0.0) return 0;
  int e;
  frexp(m, &e);  // m = f * 2^e, f in [0.5, 1)
  return e;
}

// The same for an FP32 row (max |x| in [2^(E-1), 2^E)).
__device__ __forceinline__ int row_exponent_f32(unsigned amax_bits) {
  const float m = __uint_as_float(amax_bits);
  if (!(m <= 3.40282347e38f)) return kNonFiniteExp;  // Inf or NaN
  if (m == 0.0f) return 0;
  int e;
  frexpf(m, &e);
  return e;
}

// 2^e for e in [-126, 127], from the exponent bits.
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((e + 127) << 23); }

// 2^e as a double when it is a normal number, built from the exponent bits
// (one multiply then scales exactly); ldexp outside that range.
__device__ __forceinline__ double scale_pow2(double v, int e) {
  if (e >= -1022 && e <= 1023) return v * __longlong_as_double((long long)(e + 1023) << 52);
  return ldexp(v, e);
}

// v * 2^e rounded once to FP32: one multiply when 2^e is a normal float;
// otherwise exactly in FP64 (|e| < 400 here) and one conversion.
__device__ __forceinline__ float scale_pow2f(float v, int e) {
  if (e >= -126 && e <= 127) return v * pow2f(e);
  return __double2float_rn(scale_pow2((double)v, e));
}

}  // namespace gb300
