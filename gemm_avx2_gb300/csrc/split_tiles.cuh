// split_tiles.cuh -- device helpers shared by the split-form prepare kernels
// (tc_gemm.cu, crt.cu): the coalesced 32 x 64 tile read of op(X), the per-row
// scale exponent and exact power-of-two scaling.
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

// 2^e as a double when it is a normal number, built from the exponent bits
// (one multiply then scales exactly); ldexp outside that range.
__device__ __forceinline__ double scale_pow2(double v, int e) {
  if (e >= -1022 && e <= 1023) return v * __longlong_as_double((long long)(e + 1023) << 52);
  return ldexp(v, e);
}

}  // namespace gb300
