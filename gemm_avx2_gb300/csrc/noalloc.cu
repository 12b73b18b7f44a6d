// noalloc.cu -- a split-precision SGEMM entry point that allocates nothing.
//
// Some callers cannot call cudaMalloc: code that runs under a framework owning
// all device memory (a pool allocator or a fixed memory budget that must not be
// bypassed), and code on a latency-critical path where an allocation, a free or
// the implicit synchronisation they can cause is not acceptable.  For them,
// gb300_sgemm_bf16x_noalloc runs the BF16xP split SGEMM with its scratch in a
// fixed array that is part of this library's device image, instead of a
// workspace allocated by the library or passed in by the caller.
//
// The array is a file-scope __device__ object of kNoAllocScratchBytes: every
// GPU that loads the library holds it until the process exits.  Host code must
// not use the symbol itself as a device address (on the host it names a
// host-side stand-in); it asks the runtime for the device address once per
// device and passes that pointer to the kernels.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "plain_gemm.h"
#include "split_gemm.h"

namespace gb300 {

// 32 MiB: enough for the 3xBF16 and scaled FP16 forms up to about
// m = n = k = 1980 and the 6xBF16 form up to about 1600 (see
// gb300_split_workspace_bytes).
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
static __device__ unsigned g_noalloc_error_word;

namespace {
constexpr int kMaxDev = 64;
struct NoAllocSlot {
  void *scratch = nullptr;
  unsigned *err = nullptr;
  bool ready = false;
};
NoAllocSlot g_slots[kMaxDev];
std::mutex g_mu;

// Device addresses of the scratch array and error word for the current device,
// looked up once per device (the first call on a device does this set-up).
int noalloc_setup(NoAllocSlot **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return GB300_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_mu);
  NoAllocSlot &s = g_slots[dev];
  if (!s.ready) {
    void *p = nullptr, *e = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) return GB300_ERR_CUDA;
    if (cudaGetSymbolAddress(&e, g_noalloc_error_word) != cudaSuccess) return GB300_ERR_CUDA;
    s.scratch = p;
    s.err = static_cast<unsigned *>(e);
    s.ready = true;
  }
  *out = &s;
  return GB300_OK;
}
}  // namespace

// The error word of the no-allocation entry point on the current device: 0
// if no call has set up this device yet.  Reads it (and, with `clear`, zeroes
// it) through the symbol, so nothing is allocated.
int noalloc_error_read(int clear, unsigned *out) {
  *out = 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return GB300_ERR_CUDA;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_slots[dev].ready) return GB300_OK;
  }
  unsigned w = 0;
  if (cudaMemcpyFromSymbol(&w, g_noalloc_error_word, sizeof w) != cudaSuccess)
    return GB300_ERR_CUDA;
  if (clear && w) {
    const unsigned zero = 0;
    if (cudaMemcpyToSymbol(g_noalloc_error_word, &zero, sizeof zero) != cudaSuccess)
      return GB300_ERR_CUDA;
  }
  *out = w;
  return GB300_OK;
}

}  // namespace gb300

using namespace gb300;

extern "C" __attribute__((visibility("default"))) int gb300_sgemm_bf16x_noalloc(
    char ta, char tb, int m, int n, int k, float alpha, const float *A, int lda, const float *B,
    int ldb, float beta, float *C, int ldc, int products, void *stream) {
  if (!split_products_ok(products)) return GB300_ERR_ARG;
  const int ck = check_args(ta, tb, m, n, k, lda, ldb, ldc);
  if (ck != GB300_OK) return ck < 0 ? GB300_OK : ck;
  const size_t need = split_workspace_bytes(0, m, n, k, products);
  if (need > kNoAllocScratchBytes) return GB300_ERR_NOALLOC_LIMIT;
  NoAllocSlot *slot = nullptr;
  const int rc = noalloc_setup(&slot);
  if (rc != GB300_OK) return rc;
  // Nothing in the scratch has to start at zero: the split kernels write every
  // byte of the operand area that the GEMM kernel reads (padding included).
  return split_sgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, products,
                     slot->scratch, kNoAllocScratchBytes, static_cast<cudaStream_t>(stream),
                     slot->err);
}

