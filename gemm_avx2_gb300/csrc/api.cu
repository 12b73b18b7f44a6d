// api.cu -- the C ABI of libgemm_gb300.so: device-pointer entry points,
// host-pointer (drop-in) staging, tensor-map encoding, device error words and
// the cached split-form workspace.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <unordered_map>
#include <utility>
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <thread>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "plain_gemm.h"
#include "split_gemm.h"

#define GB300_API extern "C" __attribute__((visibility("default")))

namespace gb300 {

// ---------------------------------------------------------------- tensor maps
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn get_encode() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

bool encode_2d(CUtensorMap *map, const void *base, size_t elem_bytes, int64_t rows, int64_t cols,
               int64_t ld, int box_rows, int box_cols, bool swizzle128) {
  EncodeTiledFn fn = get_encode();
  if (!fn || rows <= 0 || cols <= 0) return false;
  CUtensorMapDataType dt = elem_bytes == 8   ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64
                           : elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                             : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
  cuuint64_t dims[2] = {(cuuint64_t)rows, (cuuint64_t)cols};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * (int64_t)elem_bytes)};
  cuuint32_t box[2] = {(cuuint32_t)box_rows, (cuuint32_t)box_cols};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, dt, 2, const_cast<void *>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE,
                  swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

bool encode_3d(CUtensorMap *map, const void *base, size_t elem_bytes, int64_t d0, int64_t d1,
               int64_t d2, int64_t ld1, int64_t ld2, int box0, int box1, int box2) {
  EncodeTiledFn fn = get_encode();
  if (!fn || d0 <= 0 || d1 <= 0 || d2 <= 0) return false;
  CUtensorMapDataType dt = elem_bytes == 8   ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64
                           : elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                             : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
  cuuint64_t dims[3] = {(cuuint64_t)d0, (cuuint64_t)d1, (cuuint64_t)d2};
  cuuint64_t strides[2] = {(cuuint64_t)(ld1 * (int64_t)elem_bytes),
                           (cuuint64_t)(ld2 * (int64_t)elem_bytes)};
  cuuint32_t box[3] = {(cuuint32_t)box0, (cuuint32_t)box1, (cuuint32_t)box2};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(map, dt, 3, const_cast<void *>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// ---------------------------------------------------------------- per-device state
struct DeviceState {
  unsigned *err = nullptr;  // device error word
  // cached workspaces of the split forms, one per stream (grow-only): calls on
  // one stream are ordered, calls on different streams never share scratch
  std::unordered_map<cudaStream_t, std::pair<void *, size_t>> ws;
  // staging buffers of the host-pointer (drop-in) path
  void *stage[3] = {nullptr, nullptr, nullptr};
  size_t stage_bytes[3] = {0, 0, 0};
  cudaStream_t stage_stream = nullptr;
  cudaStream_t side_stream = nullptr;          // C staging beside the split forms' prepare
  cudaEvent_t ev_start = nullptr, ev_c = nullptr;
  cudaStream_t copy_stream = nullptr;          // operand parts of the pipelined host path
  cudaStream_t out_stream = nullptr;           // its finished C blocks
  cudaStream_t prep_stream = nullptr;          // its operand splits
  cudaStream_t block_stream = nullptr;         // its second stream of C blocks
  std::vector<cudaEvent_t> part_ev;            // one per operand part
  std::mutex mu;  // guards ws and staging (one host-pointer call at a time per device)
};
static constexpr int kMaxDevices = 64;
static DeviceState g_dev[kMaxDevices];
static std::mutex g_init_mu;

static DeviceState *dev_state() {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= kMaxDevices) return nullptr;
  DeviceState &s = g_dev[d];
  if (!s.err) {
    std::lock_guard<std::mutex> lk(g_init_mu);
    if (!s.err) {
      unsigned *p = nullptr;
      if (cudaMalloc(&p, sizeof(unsigned)) != cudaSuccess) return nullptr;
      if (cudaMemset(p, 0, sizeof(unsigned)) != cudaSuccess) return nullptr;
      s.err = p;
    }
  }
  return &s;
}

unsigned *device_error_word() {
  DeviceState *s = dev_state();
  return s ? s->err : nullptr;
}

static bool grow(void **p, size_t *have, size_t need) {
  if (*have >= need) return true;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *have = 0;
  size_t sz = need + need / 8 + 256;
  if (cudaMalloc(p, sz) != cudaSuccess) {
    *p = nullptr;
    return false;
  }
  *have = sz;
  return true;
}

// Library-owned workspace for the split forms on `st` (caller holds s->mu).
void *cached_workspace(DeviceState *s, cudaStream_t st, size_t need) {
  auto &e = s->ws[st];
  if (e.second < need) {
    // the stream may still be using the old buffer
    if (e.first && cudaStreamSynchronize(st) != cudaSuccess) return nullptr;
  }
  if (!grow(&e.first, &e.second, need)) return nullptr;
  return e.first;
}

// ---------------------------------------------------------------- host-pointer staging
// True when every non-null pointer is page-locked (or registered) host memory.
static bool host_pinned(const void *a, const void *b, const void *c) {
  for (const void *p : {a, b, c}) {
    if (!p) continue;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    if (at.type != cudaMemoryTypeHost) return false;
  }
  return true;
}

// True when kernels may dereference these host pointers directly: the device
// reads pageable memory through the host's page tables (coherent CPU-GPU
// systems such as Grace + GB300), or every pointer is page-locked / registered.
static bool host_direct_ok(const void *a, const void *b, const void *c) {
  int dev = 0, pageable = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) ==
          cudaSuccess &&
      pageable == 1)
    return true;
  return host_pinned(a, b, c);
}

// A small persistent pool of host threads for scans of host buffers (started
// on first use; the pipelined host path's C scan).  start(n, f) has the
// workers call f(0) .. f(n - 1) and returns at once; wait() joins in and
// returns when all are done (one job at a time: start blocks while another
// caller's job runs).
class HostPool {
 public:
  static HostPool &get() {
    static HostPool p;
    return p;
  }
  int size() const { return (int)workers_.size() + 1; }
  void start(int n, std::function<void(int)> f) {
    run_mu_.lock();  // one job at a time (calls from several devices); wait() unlocks
    std::lock_guard<std::mutex> lk(mu_);
    fn_ = std::move(f);
    job_ = &fn_;
    njobs_ = n;
    next_ = 0;
    done_ = 0;
    ++gen_;
    cv_.notify_all();
  }
  void wait() {
    work();
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return done_ == njobs_; });
    job_ = nullptr;
    lk.unlock();
    run_mu_.unlock();
  }

 private:
  HostPool() {
    // at most 12 threads with the caller, and 4 cores left to the caller's
    // other threads: the caller waits for the slowest chunk, so a scan thread
    // preempted by another runnable thread would hold up the whole call
    const int hw = (int)std::thread::hardware_concurrency();
    const int nt = hw >= 16 ? 11 : hw > 5 ? hw - 5 : 0;
    for (int i = 0; i < nt; ++i) workers_.emplace_back([this] { loop(); });
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
      ++gen_;
    }
    cv_.notify_all();
    for (auto &t : workers_) t.join();
  }
  void work() {
    for (;;) {
      int i;
      {
        std::lock_guard<std::mutex> lk(mu_);
        if (!job_ || next_ >= njobs_) return;
        i = next_++;
      }
      (*job_)(i);
      std::lock_guard<std::mutex> lk(mu_);
      if (++done_ == njobs_) done_cv_.notify_all();
    }
  }
  void loop() {
    unsigned long seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
        if (stop_) return;
        seen = gen_;
      }
      work();
    }
  }
  std::vector<std::thread> workers_;
  std::mutex run_mu_, mu_;
  std::condition_variable cv_, done_cv_;
  std::function<void(int)> fn_;
  const std::function<void(int)> *job_ = nullptr;
  int njobs_ = 0, next_ = 0, done_ = 0;
  unsigned long gen_ = 0;
  bool stop_ = false;
};

// True when every entry of the m x n window of C is finite with its sign bit
// clear: then beta = 0 makes 0 * C = +0 everywhere, exactly what a zero-filled
// copy gives, so C need not cross the CPU-GPU link.  The bit patterns are
// compared as unsigned integers: negative values (sign bit) and Inf / NaN lie
// at or above the +Inf pattern.
// The scan starts on the pool and runs while the caller queues other work;
// *bad is final after HostPool::get().wait().
template <typename T>
static void host_c_scan_start(const T *c, int m, int n, int ldc, std::atomic<bool> *bad) {
  using U = typename std::conditional<sizeof(T) == 8, uint64_t, uint32_t>::type;
  const U lim = sizeof(T) == 8 ? (U)0x7ff0000000000000ull : (U)0x7f800000u;
  bad->store(false);
  HostPool &pool = HostPool::get();
  const int chunks = pool.size() * 4 < n ? pool.size() * 4 : n;
  pool.start(chunks, [=](int t) {
    const int j0 = (int)((int64_t)n * t / chunks), j1 = (int)((int64_t)n * (t + 1) / chunks);
    for (int j = j0; j < j1 && !bad->load(std::memory_order_relaxed); ++j) {
      const U *col = reinterpret_cast<const U *>(c + (int64_t)j * ldc);
      U mx = 0;
      for (int i = 0; i < m; ++i) mx = col[i] > mx ? col[i] : mx;
      if (mx >= lim) bad->store(true, std::memory_order_relaxed);
    }
  });
}

// Operand parts of the pipelined host path (GB300_TUNE_HOST_PARTS): 0 =
// by shape, 1 = no pipeline, P = P row parts of op(A) and P column parts of
// op(B).
static int g_host_parts = 0;
static int host_parts_for(int R, int k, bool pinned, bool fp64) {
  if (g_host_parts) return g_host_parts;
  // four parts of at least 1024 rows / columns once the operands are large
  // enough for the link to matter: measured best of 1-6 parts at SGEMM TN
  // 8192^3 (5.04 ms a call against 5.47 unpipelined) and 16384^3 (23.5 ms
  // against 30.4); for the FP64 CRT form two from 2048 (DGEMM NN 2048^3:
  // 0.787 ms against 1.088 unpipelined, 3 parts 0.788, 4 parts 0.827), not
  // for the FP32 splits, whose faster blocks leave less to hide (SGEMM TN
  // 2048^3 / 3072^3: 0.468 / 0.855 ms with two parts against 0.366 / 0.731).
  // Pageable memory is moved by SM copies, which compete with the GEMM for
  // SMs (slower pipelined): no pipeline by default.
  if (!pinned || k < 1024) return 1;
  return R >= 4096 ? 4 : (fp64 && R >= 2048) ? 2 : 1;
}

// Boundaries of `parts` parts of [0, R), each starting on a multiple of align.
static std::vector<int> part_bounds(int R, int parts, int align) {
  std::vector<int> b{0};
  const int64_t step = ((int64_t)(R + parts - 1) / parts + align - 1) / align * align;
  for (int64_t x = step; x < R; x += step) b.push_back((int)x);
  b.push_back(R);
  return b;
}

// Pipelined host-pointer call of the FP32 split forms and the FP64 CRT form
// (T = float / double; the same part and block structure).  op(A) goes in row
// parts and op(B) in column parts; a copy stream moves them to HBM in the
// order A0 B0 A1 B1 ... (with B part j, the columns of C it covers), and the
// compute stream prepares each part once it has arrived and
// runs every C block (i, j) into HBM as soon as both of its parts are
// prepared; an output stream copies each finished block back.  So the link
// transfers (about 210 GB/s one way, 320 GB/s both ways together: the bound
// of this path) overlap the GEMMs of other blocks.  With beta = 0 a C part
// is copied only when one of its entries is negative, Inf or NaN (a scan of
// the part on host threads while its shard's A and B copy): otherwise 0 * C
// is +0 there and the device copy of that part is zero-filled instead, with
// the same result bits and a third fewer bytes over the link (A, B and C of
// equal size).  The splits run on a
// stream of their own and the blocks alternate between two streams, so one
// block's partial last wave of tiles overlaps the next block.  The epilogues stay in
// HBM: writing C over the link from the epilogue slowed the blocks 1.5-3x
// while the operand copies ran.  The results equal the whole-problem call's
// bit for bit: the exponents are per row / column over all of K, and every C
// element's K order is the same.  Caller holds s->mu; st is s->stage_stream.
template <typename T>
static int host_split_pipelined(DeviceState *s, cudaStream_t st, char ta, char tb, int m, int n,
                                int k, T alpha, const T *a, int lda, const T *b, int ldb, T beta,
                                T *c, int ldc, int prm, bool ce) {
  const bool an = notrans(ta), bn = notrans(tb);
  const int arows = an ? m : k, acols = an ? k : m;
  const int brows = bn ? k : n, bcols = bn ? n : k;
  const std::vector<int> rb = part_bounds(m, host_parts_for(m, k, ce, sizeof(T) == 8), kSplitBM);
  const std::vector<int> cb = part_bounds(n, host_parts_for(n, k, ce, sizeof(T) == 8), kBf16xBN);
  const int P = (int)rb.size() - 1, Q = (int)cb.size() - 1;
  constexpr int epl = 16 / (int)sizeof(T);  // 16-byte aligned columns in HBM
  auto up = [](int r) { return ((r > 1 ? r : 1) + epl - 1) / epl * epl; };
  const int ulda = up(arows), uldb = up(brows), uldc = up(m);
  if (!grow(&s->stage[0], &s->stage_bytes[0], (size_t)ulda * acols * sizeof(T) + 16) ||
      !grow(&s->stage[1], &s->stage_bytes[1], (size_t)uldb * bcols * sizeof(T) + 16) ||
      !grow(&s->stage[2], &s->stage_bytes[2], (size_t)uldc * n * sizeof(T) + 16))
    return GB300_ERR_NOMEM;
  T *dA = static_cast<T *>(s->stage[0]), *dB = static_cast<T *>(s->stage[1]);
  T *dC = static_cast<T *>(s->stage[2]);
  for (cudaStream_t *q : {&s->copy_stream, &s->out_stream, &s->prep_stream, &s->block_stream})
    if (!*q && cudaStreamCreateWithFlags(q, cudaStreamNonBlocking) != cudaSuccess)
      return GB300_ERR_CUDA;
  while ((int)s->part_ev.size() < 1 + 2 * (P + Q) + P * Q + Q) {
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return GB300_ERR_CUDA;
    s->part_ev.push_back(e);
  }
  // FP32: the BF16xP / scaled FP16 split; FP64: the CRT form
  const size_t wneed = sizeof(T) == 4 ? split_workspace_bytes(0, m, n, k, prm)
                                      : crt_workspace_bytes(m, n, k, prm);
  auto prepare_part = [&](int z, char t, const T *X, int ldx, int r0, int rows, void *w,
                          cudaStream_t q) {
    if constexpr (sizeof(T) == 4)
      return split_sgemm_prepare_part(z, t, m, n, k, X, ldx, r0, rows, prm, w, wneed, q);
    else
      return crt_prepare_part(z, t, m, n, k, X, ldx, r0, rows, prm, w, wneed, q);
  };
  auto run_block = [&](int i0, int h, int j0, int w, void *wsp, cudaStream_t q) {
    if constexpr (sizeof(T) == 4)
      return split_sgemm_run_block(m, n, k, i0, h, j0, w, alpha, beta, dC, uldc, prm, wsp, wneed,
                                   q, s->err);
    else
      return crt_run_block(m, n, k, i0, h, j0, w, alpha, beta, dC, uldc, prm, wsp, wneed, q,
                           s->err);
  };
  void *ws = wneed ? cached_workspace(s, st, wneed) : nullptr;
  if (!ws) return GB300_ERR_NOMEM;
  cudaStream_t cs = s->copy_stream, os = s->out_stream, ps = s->prep_stream;
  const cudaStream_t bs[2] = {st, s->block_stream};
  // copy engines for page-locked memory, else SM copies (the device reads the
  // host memory); one 2-D copy per part or block (w elements x cols)
  auto copy = [&](T *dst, int dp, const T *src, int sp, int w, int cols,
                  cudaMemcpyKind kind, cudaStream_t q) {
    if (ce)
      return cudaMemcpy2DAsync(dst, (size_t)dp * sizeof(T), src, (size_t)sp * sizeof(T),
                               (size_t)w * sizeof(T), cols, kind, q) == cudaSuccess;
    return copy_2d(dst, (size_t)dp * sizeof(T), src, (size_t)sp * sizeof(T),
                   (size_t)w * sizeof(T), cols, q) == GB300_OK;
  };
  const cudaMemcpyKind h2d = cudaMemcpyHostToDevice, d2h = cudaMemcpyDeviceToHost;
  // arrival of the parts in HBM, their splits done, the blocks done
  cudaEvent_t *evA = s->part_ev.data() + 1, *evB = evA + P, *evPA = evB + Q, *evPB = evPA + P;
  cudaEvent_t *evC = evPB + Q, *evCin = evC + P * Q;  // blocks done, C parts in HBM
  // the side streams start after the work already queued on st (buffer reuse)
  bool ok = cudaEventRecord(s->part_ev[0], st) == cudaSuccess;
  for (cudaStream_t q : {cs, os, ps, bs[1]})
    ok = ok && cudaStreamWaitEvent(q, s->part_ev[0], 0) == cudaSuccess;
  // One pass over the shards, so the GPU never waits for this thread: each
  // shard's A and B parts go on the copy stream; with beta = 0 the scan of
  // its C part (host threads, started first) decides whether that part is
  // copied or zero-filled, and runs while the shard's A and B copy; then the
  // shard's splits, and every block whose parts are now all queued.
  const bool b0 = beta == T(0);
  std::atomic<bool> c_bad{false};
  bool scanning = false;
  auto c_part = [&](int j, bool need) {  // C columns of part j, then evCin[j]
    const int c0 = cb[j], w = cb[j + 1] - c0;
    return (need ? copy(dC + (int64_t)c0 * uldc, uldc, c + (int64_t)c0 * ldc, ldc, m, w, h2d, cs)
                 : cudaMemset2DAsync(dC + (int64_t)c0 * uldc, (size_t)uldc * sizeof(T), 0,
                                     (size_t)m * sizeof(T), w, cs) == cudaSuccess) &&
           cudaEventRecord(evCin[j], cs) == cudaSuccess;
  };
  int nblk = 0;
  auto block = [&](int i, int j) {
    const int i0 = rb[i], h = rb[i + 1] - i0, j0 = cb[j], w = cb[j + 1] - j0;
    const cudaStream_t q = bs[nblk & 1];
    if (cudaStreamWaitEvent(q, evPA[i], 0) != cudaSuccess ||
        cudaStreamWaitEvent(q, evPB[j], 0) != cudaSuccess ||
        cudaStreamWaitEvent(q, evCin[j], 0) != cudaSuccess)
      return (int)GB300_ERR_CUDA;
    int r = run_block(i0, h, j0, w, ws, q);
    // the finished block goes back while the next ones compute
    cudaEvent_t e = evC[nblk++];
    if (r == GB300_OK &&
        (cudaEventRecord(e, q) != cudaSuccess || cudaStreamWaitEvent(os, e, 0) != cudaSuccess ||
         !copy(c + i0 + (int64_t)j0 * ldc, ldc, dC + i0 + (int64_t)j0 * uldc, uldc, h, w, d2h,
               os)))
      r = GB300_ERR_CUDA;
    return r;
  };
  const int nsh = P > Q ? P : Q;
  int rc = ok ? GB300_OK : GB300_ERR_CUDA;
  for (int sh = 0; rc == GB300_OK && sh < nsh; ++sh) {
    if (b0 && sh < Q) {
      host_c_scan_start(c + (int64_t)cb[sh] * ldc, m, cb[sh + 1] - cb[sh], ldc, &c_bad);
      scanning = true;
    }
    if (sh < P) {  // op(A) rows [r0, r1): rows of A, or columns of A when transposed
      const int r0 = rb[sh], h = rb[sh + 1] - r0;
      ok = (an ? copy(dA + r0, ulda, a + r0, lda, h, k, h2d, cs)
               : copy(dA + (int64_t)r0 * ulda, ulda, a + (int64_t)r0 * lda, lda, k, h, h2d, cs)) &&
           cudaEventRecord(evA[sh], cs) == cudaSuccess;
    }
    if (ok && sh < Q) {  // op(B) columns [c0, c1), and those columns of C (read when beta != 0,
                         // and with beta = 0 when one is negative, Inf or NaN: C * 0 keeps
                         // the NaN / Inf and the negative zeros, as C_MULT_BETA does)
      const int c0 = cb[sh], w = cb[sh + 1] - c0;
      ok = (bn ? copy(dB + (int64_t)c0 * uldb, uldb, b + (int64_t)c0 * ldb, ldb, k, w, h2d, cs)
               : copy(dB + c0, uldb, b + c0, ldb, w, k, h2d, cs)) &&
           cudaEventRecord(evB[sh], cs) == cudaSuccess;
      if (ok && !b0) ok = c_part(sh, true);
    }
    if (scanning) {
      HostPool::get().wait();
      scanning = false;
      if (ok) ok = c_part(sh, c_bad.load());
    }
    rc = ok ? GB300_OK : GB300_ERR_CUDA;
    // the shard's splits, once its parts have arrived
    if (rc == GB300_OK && sh < P) {
      rc = cudaStreamWaitEvent(ps, evA[sh], 0) == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
      if (rc == GB300_OK)
        rc = prepare_part(0, ta, dA, ulda, rb[sh], rb[sh + 1] - rb[sh], ws, ps);
      if (rc == GB300_OK && cudaEventRecord(evPA[sh], ps) != cudaSuccess) rc = GB300_ERR_CUDA;
    }
    if (rc == GB300_OK && sh < Q) {
      rc = cudaStreamWaitEvent(ps, evB[sh], 0) == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
      if (rc == GB300_OK)
        rc = prepare_part(1, tb, dB, uldb, cb[sh], cb[sh + 1] - cb[sh], ws, ps);
      if (rc == GB300_OK && cudaEventRecord(evPB[sh], ps) != cudaSuccess) rc = GB300_ERR_CUDA;
    }
    // the blocks whose second part is this shard's
    if (sh < P)
      for (int j = 0; rc == GB300_OK && j < Q && j <= sh; ++j) rc = block(sh, j);
    if (sh < Q)
      for (int i = 0; rc == GB300_OK && i < P && i < sh; ++i) rc = block(i, sh);
  }
  if (scanning) HostPool::get().wait();  // its threads use this frame's flag
  cudaError_t e = cudaSuccess;
  for (cudaStream_t q : {cs, ps, bs[0], bs[1], os}) {
    const cudaError_t eq = cudaStreamSynchronize(q);
    if (e == cudaSuccess) e = eq;
  }
  if (rc != GB300_OK) return rc;
  if (e != cudaSuccess) return GB300_ERR_CUDA;
  unsigned word = 0;
  cudaMemcpy(&word, s->err, sizeof(unsigned), cudaMemcpyDeviceToHost);
  return word ? GB300_ERR_TIMEOUT : GB300_OK;
}

// form: 0 = plain kernel; 1 = BF16xP split (FP32, param = products);
//       2 = Ozaki slices (FP64, param = slices); 3 = CRT (FP64, param = moduli).
template <typename T>
static int host_gemm(char ta, char tb, int m, int n, int k, T alpha, const T *a, int lda,
                     const T *b, int ldb, T beta, T *c, int ldc, int form = 0, int param = 0) {
  const bool an = notrans(ta), bn = notrans(tb);
  const int arows = an ? m : k, acols = an ? k : m;
  const int brows = bn ? k : n, bcols = bn ? n : k;
  const int ck = check_args(ta, tb, m, n, k, lda, ldb, ldc);
  if (ck != GB300_OK) return ck < 0 ? GB300_OK : ck;
  if (alpha == T(0) && beta == T(1)) return GB300_OK;
  DeviceState *s = dev_state();
  if (!s) return GB300_ERR_CUDA;
  std::lock_guard<std::mutex> lk(s->mu);
  if (!s->stage_stream &&
      cudaStreamCreateWithFlags(&s->stage_stream, cudaStreamNonBlocking) != cudaSuccess)
    return GB300_ERR_CUDA;
  cudaStream_t st = s->stage_stream;
  const bool need_ab = alpha != T(0) && k > 0;
  const bool direct = host_direct_ok(a, b, c);
  if (form != 0 && direct) {
    // Split forms on host memory the device can read.  The BF16-term split
    // reads A and B once: it reads them in place over the coherent CPU-GPU
    // link.  The forms with a max |.| pass before the split (Ozaki, CRT,
    // scaled FP16) read them twice, so A and B are first copied to HBM.  The
    // GEMM epilogues of the FP32 and Ozaki forms read and write C in place,
    // overlapped with other tiles' MMAs.  The CRT form updates C in a
    // separate, latency-bound reconstruction after its GEMMs: for large C, C
    // is copied to HBM on a side stream while A and B are prepared and copied
    // back at the end (measured: DGEMM 16384^3 54.6 -> 69.0 TFLOP/s end to
    // end; a rank-256 update with 8.6 GB of C 2.2 -> 3.9).  All copies are SM
    // loads/stores: about 200 GB/s host to device, the copy engines' rate on
    // pinned memory, and the same on pageable memory the device reads.
    int prm = param;
    if (form == 1 && prm == 0) {
      int ch = 0;
      bf16x_resolve(m, n, k, &prm, &ch);
    }
    {
      // the FP32 split forms and the FP64 CRT form
      const bool pinned = host_pinned(a, b, c);
      if ((form == 1 || form == 3) && need_ab &&
          (host_parts_for(m, k, pinned, sizeof(T) == 8) > 1 ||
           host_parts_for(n, k, pinned, sizeof(T) == 8) > 1))
        return host_split_pipelined<T>(s, st, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c,
                                       ldc, param, pinned);
    }
    const bool two_pass = form >= 2 || prm == kFp16x3;
    const int epl = 16 / (int)sizeof(T);
    auto up = [&](int r) { return ((r > 1 ? r : 1) + epl - 1) / epl * epl; };
    const T *ua = a, *ub = b;
    T *uc = c;
    int ulda = lda, uldb = ldb, uldc = ldc;
    if (two_pass && need_ab) {
      ulda = up(arows);
      uldb = up(brows);
      const size_t bA = (size_t)ulda * acols * sizeof(T), bB = (size_t)uldb * bcols * sizeof(T);
      if (!grow(&s->stage[0], &s->stage_bytes[0], bA + 16) ||
          !grow(&s->stage[1], &s->stage_bytes[1], bB + 16))
        return GB300_ERR_NOMEM;
      T *dA = static_cast<T *>(s->stage[0]), *dB = static_cast<T *>(s->stage[1]);
      if (copy_2d(dA, ulda * sizeof(T), a, (size_t)lda * sizeof(T), arows * sizeof(T), acols,
                  st) != GB300_OK ||
          copy_2d(dB, uldb * sizeof(T), b, (size_t)ldb * sizeof(T), brows * sizeof(T), bcols,
                  st) != GB300_OK)
        return GB300_ERR_CUDA;
      ua = dA;
      ub = dB;
    }
    const bool stage_c = need_ab && form == 3 && (size_t)m * n * sizeof(T) >= ((size_t)16 << 20);
    if (stage_c) {
      uldc = up(m);
      if (!grow(&s->stage[2], &s->stage_bytes[2], (size_t)uldc * n * sizeof(T) + 16))
        return GB300_ERR_NOMEM;
      if (!s->side_stream &&
          cudaStreamCreateWithFlags(&s->side_stream, cudaStreamNonBlocking) != cudaSuccess)
        return GB300_ERR_CUDA;
      if ((!s->ev_start && cudaEventCreateWithFlags(&s->ev_start, cudaEventDisableTiming) !=
                               cudaSuccess) ||
          (!s->ev_c && cudaEventCreateWithFlags(&s->ev_c, cudaEventDisableTiming) != cudaSuccess))
        return GB300_ERR_CUDA;
      uc = static_cast<T *>(s->stage[2]);
      if (cudaEventRecord(s->ev_start, st) != cudaSuccess ||
          cudaStreamWaitEvent(s->side_stream, s->ev_start, 0) != cudaSuccess ||
          copy_2d(uc, uldc * sizeof(T), c, (size_t)ldc * sizeof(T), m * sizeof(T), n,
                  s->side_stream) != GB300_OK ||
          cudaEventRecord(s->ev_c, s->side_stream) != cudaSuccess)
        return GB300_ERR_CUDA;
    }
    const size_t wneed = need_ab ? split_workspace_bytes(form - 1, m, n, k, prm) : 0;
    void *ws = wneed ? cached_workspace(s, st, wneed) : nullptr;
    if (wneed && !ws) return GB300_ERR_NOMEM;
    int rc;
    if (!need_ab) {  // alpha == 0 or k == 0: the beta update only
      if constexpr (sizeof(T) == 8)
        rc = plain_dgemm(ta, tb, m, n, 0, alpha, nullptr, m > 1 ? m : 1, nullptr, 1, beta, c, ldc,
                         st, s->err);
      else
        rc = plain_sgemm(ta, tb, m, n, 0, alpha, nullptr, m > 1 ? m : 1, nullptr, 1, beta, c, ldc,
                         st, s->err);
    } else {
      // prepare (exponents, split / slices / residues of A and B), then the GEMM on C
      if constexpr (sizeof(T) == 8)
        rc = form == 3 ? crt_prepare(ta, tb, m, n, k, ua, ulda, ub, uldb, prm, ws, wneed, st)
                       : ozaki_prepare(ta, tb, m, n, k, ua, ulda, ub, uldb, prm, ws, wneed, st);
      else
        rc = split_sgemm_prepare(ta, tb, m, n, k, ua, ulda, ub, uldb, param, ws, wneed, st);
      if (rc == GB300_OK && stage_c && cudaStreamWaitEvent(st, s->ev_c, 0) != cudaSuccess)
        rc = GB300_ERR_CUDA;
      if (rc == GB300_OK) {
        if constexpr (sizeof(T) == 8)
          rc = form == 3 ? crt_run(m, n, k, alpha, beta, uc, uldc, prm, ws, wneed, st, s->err)
                         : ozaki_run(m, n, k, alpha, beta, uc, uldc, prm, ws, wneed, st, s->err);
        else  // param 0: products and chunk from the tune cache
          rc = split_sgemm_run(m, n, k, alpha, beta, uc, uldc, param, ws, wneed, st, s->err);
      }
      if (rc == GB300_OK && stage_c)
        rc = copy_2d(c, (size_t)ldc * sizeof(T), uc, uldc * sizeof(T), m * sizeof(T), n, st);
    }
    // the side stream's copy has finished too (also when a launch above failed)
    if (stage_c && cudaStreamSynchronize(s->side_stream) != cudaSuccess && rc == GB300_OK)
      rc = GB300_ERR_CUDA;
    const cudaError_t e = cudaStreamSynchronize(st);
    if (rc != GB300_OK) return rc;
    if (e != cudaSuccess) return GB300_ERR_CUDA;
    unsigned word = 0;
    cudaMemcpy(&word, s->err, sizeof(unsigned), cudaMemcpyDeviceToHost);
    return word ? GB300_ERR_TIMEOUT : GB300_OK;
  }
  // Device copies use leading dimensions rounded up to 16 bytes so that the
  // TMA path applies whatever the host ld was.
  const int epl = 16 / (int)sizeof(T);
  auto up = [&](int r) { return ((r > 1 ? r : 1) + epl - 1) / epl * epl; };
  const int dla = up(arows), dlb = up(brows), dlc = up(m);
  const size_t bytesA = need_ab ? (size_t)dla * acols * sizeof(T) : 0;
  const size_t bytesB = need_ab ? (size_t)dlb * bcols * sizeof(T) : 0;
  const size_t bytesC = (size_t)dlc * n * sizeof(T);
  if (!grow(&s->stage[0], &s->stage_bytes[0], bytesA + 16) ||
      !grow(&s->stage[1], &s->stage_bytes[1], bytesB + 16) ||
      !grow(&s->stage[2], &s->stage_bytes[2], bytesC + 16))
    return GB300_ERR_NOMEM;
  T *dA = static_cast<T *>(s->stage[0]), *dB = static_cast<T *>(s->stage[1]);
  T *dC = static_cast<T *>(s->stage[2]);
  // SM loads/stores where the device can read the host memory (the copy
  // engines' rate on pinned memory, and no driver staging for pageable
  // memory), else the copy engines
  auto copy = [&](void *dst, size_t dp, const void *src, size_t sp, size_t w, int cols,
                  cudaMemcpyKind kind) -> cudaError_t {
    if (direct) return copy_2d(dst, dp, src, sp, w, cols, st) == GB300_OK ? cudaSuccess
                                                                        : cudaErrorUnknown;
    return cudaMemcpy2DAsync(dst, dp, src, sp, w, cols, kind, st);
  };
  cudaError_t e = cudaSuccess;
  if (need_ab) {
    e = copy(dA, dla * sizeof(T), a, (size_t)lda * sizeof(T), arows * sizeof(T), acols,
             cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = copy(dB, dlb * sizeof(T), b, (size_t)ldb * sizeof(T), brows * sizeof(T), bcols,
               cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess)
    e = copy(dC, dlc * sizeof(T), c, (size_t)ldc * sizeof(T), m * sizeof(T), n,
             cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return GB300_ERR_CUDA;
  int rc;
  const int dlda = need_ab ? dla : up(arows), dldb = need_ab ? dlb : up(brows);
  if (form != 0 && need_ab) {
    const size_t wneed = split_workspace_bytes(form - 1, m, n, k, param);
    void *ws = wneed ? cached_workspace(s, st, wneed) : nullptr;
    if (!ws) return GB300_ERR_NOMEM;
    if constexpr (sizeof(T) == 8)
      rc = form == 3 ? crt_dgemm(ta, tb, m, n, k, alpha, dA, dlda, dB, dldb, beta, dC, dlc, param,
                                 ws, wneed, st, s->err)
                     : ozaki_dgemm(ta, tb, m, n, k, alpha, dA, dlda, dB, dldb, beta, dC, dlc, param, ws,
                       wneed, st, s->err);
    else
      rc = split_sgemm(ta, tb, m, n, k, alpha, dA, dlda, dB, dldb, beta, dC, dlc, param, ws,
                       wneed, st, s->err);
  } else {
    // the plain kernels, split along K where the shape asks for it
    const size_t pneed = need_ab ? plain_workspace_bytes(sizeof(T) == 8, m, n, k) : 0;
    void *pw = pneed ? cached_workspace(s, st, pneed) : nullptr;
    const size_t pwb = pw ? pneed : 0;
    if constexpr (sizeof(T) == 8)
      rc = plain_dgemm(ta, tb, m, n, k, alpha, need_ab ? dA : nullptr, dlda,
                       need_ab ? dB : nullptr, dldb, beta, dC, dlc, st, s->err, pw, pwb);
    else
      rc = plain_sgemm(ta, tb, m, n, k, alpha, need_ab ? dA : nullptr, dlda,
                       need_ab ? dB : nullptr, dldb, beta, dC, dlc, st, s->err, pw, pwb);
  }
  if (rc != GB300_OK) {
    cudaStreamSynchronize(st);
    return rc;
  }
  e = copy(c, (size_t)ldc * sizeof(T), dC, dlc * sizeof(T), m * sizeof(T), n,
           cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return GB300_ERR_CUDA;
  unsigned word = 0;
  cudaMemcpy(&word, s->err, sizeof(unsigned), cudaMemcpyDeviceToHost);
  return word ? GB300_ERR_TIMEOUT : GB300_OK;
}

// Complex host-pointer path (the pattern of host_gemm above).  Complex
// elements are 2 * sizeof(T) bytes; leading dimensions are in complex elements.
template <typename T>
static int host_complex(char ta, char tb, int m, int n, int k, const T *alpha, const T *a, int lda,
                        const T *b, int ldb, const T *beta, T *c, int ldc, int method,
                        int param) {
  const int ck = complex_check(ta, tb, m, n, k, lda, ldb, ldc, method);
  if (ck != GB300_OK) return ck < 0 ? GB300_OK : ck;
  const bool alpha_zero = alpha[0] == T(0) && alpha[1] == T(0);
  if (alpha_zero && beta[0] == T(1) && beta[1] == T(0)) return GB300_OK;
  auto trans = [](char t) { return !(t == 'N' || t == 'n' || t == 'R' || t == 'r'); };
  const int arows = trans(ta) ? k : m, acols = trans(ta) ? m : k;
  const int brows = trans(tb) ? n : k, bcols = trans(tb) ? k : n;
  DeviceState *s = dev_state();
  if (!s) return GB300_ERR_CUDA;
  std::lock_guard<std::mutex> lk(s->mu);
  if (!s->stage_stream &&
      cudaStreamCreateWithFlags(&s->stage_stream, cudaStreamNonBlocking) != cudaSuccess)
    return GB300_ERR_CUDA;
  cudaStream_t st = s->stage_stream;
  const bool need_ab = !alpha_zero && k > 0;
  const size_t wneed =
      need_ab ? complex_workspace_bytes(sizeof(T) == 8, method, tb, m, n, k, param) : 0;
  if (need_ab && !wneed) return GB300_ERR_ARG;
  auto run = [&](const T *A, int la, const T *B, int lb, T *C, int lc) -> int {
    void *ws = wneed ? cached_workspace(s, st, wneed) : nullptr;
    if (wneed && !ws) return GB300_ERR_NOMEM;
    if constexpr (sizeof(T) == 8)
      return complex_gemm_d(ta, tb, m, n, k, alpha, A, la, B, lb, beta, C, lc, method, param, ws,
                            wneed, st, s->err);
    else
      return complex_gemm_s(ta, tb, m, n, k, alpha, A, la, B, lb, beta, C, lc, method, param, ws,
                            wneed, st, s->err);
  };
  auto finish = [&](int rc) -> int {
    const cudaError_t e = cudaStreamSynchronize(st);
    if (rc != GB300_OK) return rc;
    if (e != cudaSuccess) return GB300_ERR_CUDA;
    unsigned word = 0;
    cudaMemcpy(&word, s->err, sizeof(unsigned), cudaMemcpyDeviceToHost);
    return word ? GB300_ERR_TIMEOUT : GB300_OK;
  };
  const bool direct = host_direct_ok(a, b, c);
  if (method == GB300_CPLX_SPLIT && sizeof(T) == 4 && direct) {
    // the FP32 split method reads A and B once (pack and split kernels) and C
    // once (GEMM epilogue, overlapped with the MMAs): it runs on the caller's
    // memory over the coherent link.  The FP64 split forms read B twice and
    // end in a latency-bound C update, so they take the staged path below.
    return finish(run(a, lda, b, ldb, c, ldc));
  }
  // host <-> HBM copies: SM loads/stores where the device can read the host
  // memory (the copy engines' rate on pinned memory, and no driver staging
  // for pageable memory)
  auto copy = [&](void *dst, size_t dp, const void *src, size_t sp, size_t w, int cols,
                  cudaMemcpyKind kind) -> cudaError_t {
    if (direct) return copy_2d(dst, dp, src, sp, w, cols, st) == GB300_OK ? cudaSuccess
                                                                        : cudaErrorUnknown;
    return cudaMemcpy2DAsync(dst, dp, src, sp, w, cols, kind, st);
  };
  const size_t E = 2 * sizeof(T);
  const int epl = 16 / (int)E > 0 ? 16 / (int)E : 1;
  auto up = [&](int r) { return ((r > 1 ? r : 1) + epl - 1) / epl * epl; };
  const int dla = up(arows), dlb = up(brows), dlc = up(m);
  const size_t bytesA = need_ab ? (size_t)dla * acols * E : 0;
  const size_t bytesB = need_ab ? (size_t)dlb * bcols * E : 0;
  const size_t bytesC = (size_t)dlc * n * E;
  if (!grow(&s->stage[0], &s->stage_bytes[0], bytesA + 16) ||
      !grow(&s->stage[1], &s->stage_bytes[1], bytesB + 16) ||
      !grow(&s->stage[2], &s->stage_bytes[2], bytesC + 16))
    return GB300_ERR_NOMEM;
  T *dA = static_cast<T *>(s->stage[0]), *dB = static_cast<T *>(s->stage[1]);
  T *dC = static_cast<T *>(s->stage[2]);
  cudaError_t e = cudaSuccess;
  if (need_ab) {
    e = copy(dA, dla * E, a, (size_t)lda * E, arows * E, acols, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = copy(dB, dlb * E, b, (size_t)ldb * E, brows * E, bcols, cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess)
    e = copy(dC, dlc * E, c, (size_t)ldc * E, m * E, n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return GB300_ERR_CUDA;
  const int rc = run(need_ab ? dA : nullptr, dla, need_ab ? dB : nullptr, dlb, dC, dlc);
  if (rc != GB300_OK) {
    cudaStreamSynchronize(st);
    return rc;
  }
  e = copy(c, (size_t)ldc * E, dC, dlc * E, m * E, n, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    cudaStreamSynchronize(st);
    return GB300_ERR_CUDA;
  }
  return finish(GB300_OK);
}

// Failure-detection self-test: one CTA waits on an mbarrier that nothing ever
// arrives on, with a short poll limit; the wait gives up, records
// kErrTimeoutFull in the error word and the kernel returns normally.
__global__ void wait_timeout_selftest_kernel(unsigned limit, unsigned *err, int *reached_end) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  const bool ok = mbar_wait_limit(&bar, 0, limit, err, kErrTimeoutFull);
  __syncthreads();
  if (threadIdx.x == 0) *reached_end = ok ? 2 : 1;
}

}  // namespace gb300

using namespace gb300;

// ---------------------------------------------------------------- exported C ABI
GB300_API int gb300_host_dgemm(char ta, char tb, int m, int n, int k, double alpha,
                               const double *a, int lda, const double *b, int ldb, double beta,
                               double *c, int ldc) {
  return host_gemm<double>(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}
GB300_API int gb300_host_sgemm(char ta, char tb, int m, int n, int k, float alpha,
                               const float *a, int lda, const float *b, int ldb, float beta,
                               float *c, int ldc) {
  return host_gemm<float>(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}

GB300_API int gb300_host_sgemm_bf16x(char ta, char tb, int m, int n, int k, float alpha,
                                     const float *a, int lda, const float *b, int ldb, float beta,
                                     float *c, int ldc, int products) {
  if (products != 0 && !split_products_ok(products)) return GB300_ERR_ARG;
  return host_gemm<float>(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, 1, products);
}
GB300_API int gb300_host_dgemm_ozaki(char ta, char tb, int m, int n, int k, double alpha,
                                     const double *a, int lda, const double *b, int ldb,
                                     double beta, double *c, int ldc, int slices) {
  if (slices != 0 && (slices < 2 || slices > kOzakiMaxSlices)) return GB300_ERR_ARG;
  return host_gemm<double>(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, 2,
                           slices > 0 ? slices : ozaki_default_slices(m, n, k));
}

GB300_API int gb300_host_dgemm_ozaki2(char ta, char tb, int m, int n, int k, double alpha,
                                      const double *a, int lda, const double *b, int ldb,
                                      double beta, double *c, int ldc, int moduli) {
  if (moduli != 0 && (moduli < 2 || moduli > kCrtMaxModuli)) return GB300_ERR_ARG;
  return host_gemm<double>(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, 3, moduli);
}

GB300_API int gb300_dgemm_ozaki2(char ta, char tb, int m, int n, int k, double alpha,
                                 const double *A, int lda, const double *B, int ldb, double beta,
                                 double *C, int ldc, int moduli, void *ws, size_t ws_bytes,
                                 void *stream) {
  if (moduli != 0 && (moduli < 2 || moduli > kCrtMaxModuli)) return GB300_ERR_ARG;
  const int ck = check_args(ta, tb, m, n, k, lda, ldb, ldc);
  if (ck != GB300_OK) return ck < 0 ? GB300_OK : ck;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (ws) {
    unsigned *err = device_error_word();
    if (!err) return GB300_ERR_CUDA;
    return crt_dgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, moduli, ws, ws_bytes,
                     st, err);
  }
  DeviceState *s = dev_state();
  if (!s) return GB300_ERR_CUDA;
  const size_t need = (alpha != 0.0 && k > 0) ? crt_workspace_bytes(m, n, k, moduli) : 0;
  std::lock_guard<std::mutex> lk(s->mu);
  void *w = need ? cached_workspace(s, st, need) : nullptr;
  if (need && !w) return GB300_ERR_NOMEM;
  return crt_dgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, moduli, w, need, st,
                   s->err);
}

// The plain kernels on device pointers.  A split-K call gets room for its
// slices from the stream's cached workspace; if that cannot grow, it runs
// unsplit.
template <typename T>
static int plain_api(char ta, char tb, int m, int n, int k, T alpha, const T *A, int lda,
                     const T *B, int ldb, T beta, T *C, int ldc, void *stream) {
  const int ck = check_args(ta, tb, m, n, k, lda, ldb, ldc);
  if (ck != GB300_OK) return ck < 0 ? GB300_OK : ck;
  DeviceState *s = dev_state();
  if (!s) return GB300_ERR_CUDA;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t need = alpha != T(0) ? plain_workspace_bytes(sizeof(T) == 8, m, n, k) : 0;
  if (!need) {
    if constexpr (sizeof(T) == 8)
      return plain_dgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, st, s->err);
    else
      return plain_sgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, st, s->err);
  }
  std::lock_guard<std::mutex> lk(s->mu);
  void *w = cached_workspace(s, st, need);
  const size_t wb = w ? need : 0;
  if constexpr (sizeof(T) == 8)
    return plain_dgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, st, s->err, w, wb);
  else
    return plain_sgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, st, s->err, w, wb);
}

GB300_API int gb300_dgemm(char ta, char tb, int m, int n, int k, double alpha, const double *A,
                          int lda, const double *B, int ldb, double beta, double *C, int ldc,
                          void *stream) {
  return plain_api<double>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, stream);
}
GB300_API int gb300_sgemm(char ta, char tb, int m, int n, int k, float alpha, const float *A,
                          int lda, const float *B, int ldb, float beta, float *C, int ldc,
                          void *stream) {
  return plain_api<float>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, stream);
}

// ---------------------------------------------------------------- complex
static bool complex_param_ok(bool dbl, int method, int param) {
  if (method == GB300_CPLX_CRT) return dbl && (param == 0 || (param >= 2 && param <= kCrtMaxModuli));
  if (method != GB300_CPLX_SPLIT) return true;
  return dbl ? (param == 0 || (param >= 2 && param <= kOzakiMaxSlices))
             : (param == 0 || split_products_ok(param));
}

GB300_API size_t gb300_complex_workspace_bytes(int is_double, int method, char tb, int m, int n,
                                               int k, int param) {
  if (!complex_param_ok(is_double != 0, method, param)) return 0;
  return complex_workspace_bytes(is_double, method, tb, m, n, k, param);
}

template <typename T>
static int device_complex(char ta, char tb, int m, int n, int k, const T *alpha, const T *A,
                          int lda, const T *B, int ldb, const T *beta, T *C, int ldc, int method,
                          int param, void *ws, size_t ws_bytes, void *stream) {
  const bool dbl = sizeof(T) == 8;
  if (!alpha || !beta || !complex_param_ok(dbl, method, param)) return GB300_ERR_ARG;
  const int ck = complex_check(ta, tb, m, n, k, lda, ldb, ldc, method);
  if (ck != GB300_OK) return ck < 0 ? GB300_OK : ck;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  auto call = [&](void *w, size_t wb, unsigned *err) -> int {
    if constexpr (sizeof(T) == 8)
      return complex_gemm_d(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, method, param,
                            w, wb, st, err);
    else
      return complex_gemm_s(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, method, param,
                            w, wb, st, err);
  };
  if (ws) {
    unsigned *err = device_error_word();
    if (!err) return GB300_ERR_CUDA;
    return call(ws, ws_bytes, err);
  }
  DeviceState *s = dev_state();
  if (!s) return GB300_ERR_CUDA;
  const bool reads_ab = !(alpha[0] == T(0) && alpha[1] == T(0)) && k > 0;
  const size_t need = reads_ab ? complex_workspace_bytes(dbl, method, tb, m, n, k, param) : 0;
  if (reads_ab && !need) return GB300_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  void *w = need ? cached_workspace(s, st, need) : nullptr;
  if (need && !w) return GB300_ERR_NOMEM;
  return call(w, need, s->err);
}

GB300_API int gb300_cgemm(char ta, char tb, int m, int n, int k, const float *alpha,
                          const float *A, int lda, const float *B, int ldb, const float *beta,
                          float *C, int ldc, int method, int param, void *ws, size_t ws_bytes,
                          void *stream) {
  return device_complex<float>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, method,
                               param, ws, ws_bytes, stream);
}
GB300_API int gb300_zgemm(char ta, char tb, int m, int n, int k, const double *alpha,
                          const double *A, int lda, const double *B, int ldb, const double *beta,
                          double *C, int ldc, int method, int param, void *ws, size_t ws_bytes,
                          void *stream) {
  return device_complex<double>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, method,
                                param, ws, ws_bytes, stream);
}
GB300_API int gb300_host_cgemm(char ta, char tb, int m, int n, int k, const float *alpha,
                               const float *a, int lda, const float *b, int ldb,
                               const float *beta, float *c, int ldc, int method, int param) {
  if (!alpha || !beta || !complex_param_ok(false, method, param)) return GB300_ERR_ARG;
  return host_complex<float>(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, method, param);
}
GB300_API int gb300_host_zgemm(char ta, char tb, int m, int n, int k, const double *alpha,
                               const double *a, int lda, const double *b, int ldb,
                               const double *beta, double *c, int ldc, int method, int param) {
  if (!alpha || !beta || !complex_param_ok(true, method, param)) return GB300_ERR_ARG;
  return host_complex<double>(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, method,
                              param);
}

GB300_API size_t gb300_split_workspace_bytes(int kind, int m, int n, int k, int param) {
  return split_workspace_bytes(kind, m, n, k, param);
}

GB300_API int gb300_sgemm_bf16x_ws(char ta, char tb, int m, int n, int k, float alpha,
                                   const float *A, int lda, const float *B, int ldb, float beta,
                                   float *C, int ldc, int products, void *ws, size_t ws_bytes,
                                   void *stream) {
  if (products != 0 && !split_products_ok(products)) return GB300_ERR_ARG;
  const int ck = check_args(ta, tb, m, n, k, lda, ldb, ldc);
  if (ck != GB300_OK) return ck < 0 ? GB300_OK : ck;
  unsigned *err = device_error_word();
  if (!err) return GB300_ERR_CUDA;
  return split_sgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, products, ws, ws_bytes,
                     static_cast<cudaStream_t>(stream), err);
}
GB300_API int gb300_sgemm_bf16x(char ta, char tb, int m, int n, int k, float alpha,
                                const float *A, int lda, const float *B, int ldb, float beta,
                                float *C, int ldc, int products, void *stream) {
  if (products != 0 && !split_products_ok(products)) return GB300_ERR_ARG;
  const int ck = check_args(ta, tb, m, n, k, lda, ldb, ldc);
  if (ck != GB300_OK) return ck < 0 ? GB300_OK : ck;
  DeviceState *s = dev_state();
  if (!s) return GB300_ERR_CUDA;
  const size_t need = split_workspace_bytes(0, m, n, k, products);
  std::lock_guard<std::mutex> lk(s->mu);
  void *ws = need ? cached_workspace(s, static_cast<cudaStream_t>(stream), need) : nullptr;
  if (need && !ws) return GB300_ERR_NOMEM;
  return split_sgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, products, ws, need,
                     static_cast<cudaStream_t>(stream), s->err);
}

GB300_API int gb300_dgemm_ozaki_ws(char ta, char tb, int m, int n, int k, double alpha,
                                   const double *A, int lda, const double *B, int ldb,
                                   double beta, double *C, int ldc, int slices, void *ws,
                                   size_t ws_bytes, void *stream) {
  if (slices != 0 && (slices < 2 || slices > kOzakiMaxSlices)) return GB300_ERR_ARG;
  const int ck = check_args(ta, tb, m, n, k, lda, ldb, ldc);
  if (ck != GB300_OK) return ck < 0 ? GB300_OK : ck;
  unsigned *err = device_error_word();
  if (!err) return GB300_ERR_CUDA;
  return ozaki_dgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, slices, ws, ws_bytes,
                     static_cast<cudaStream_t>(stream), err);
}
GB300_API int gb300_dgemm_ozaki(char ta, char tb, int m, int n, int k, double alpha,
                                const double *A, int lda, const double *B, int ldb, double beta,
                                double *C, int ldc, int slices, void *stream) {
  if (slices != 0 && (slices < 2 || slices > kOzakiMaxSlices)) return GB300_ERR_ARG;
  const int ck = check_args(ta, tb, m, n, k, lda, ldb, ldc);
  if (ck != GB300_OK) return ck < 0 ? GB300_OK : ck;
  DeviceState *s = dev_state();
  if (!s) return GB300_ERR_CUDA;
  const size_t need = split_workspace_bytes(1, m, n, k, slices);
  std::lock_guard<std::mutex> lk(s->mu);
  void *ws = need ? cached_workspace(s, static_cast<cudaStream_t>(stream), need) : nullptr;
  if (need && !ws) return GB300_ERR_NOMEM;
  return ozaki_dgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, slices, ws, need,
                     static_cast<cudaStream_t>(stream), s->err);
}

GB300_API int gb300_sgemm_bf16x_prepare(char ta, char tb, int m, int n, int k, const float *A,
                                        int lda, const float *B, int ldb, int products, void *ws,
                                        size_t ws_bytes, void *stream) {
  return split_sgemm_prepare(ta, tb, m, n, k, A, lda, B, ldb, products, ws, ws_bytes,
                             static_cast<cudaStream_t>(stream));
}
GB300_API int gb300_sgemm_bf16x_run(int m, int n, int k, float alpha, float beta, float *C,
                                    int ldc, int products, const void *ws, size_t ws_bytes,
                                    void *stream) {
  if (m < 0 || n < 0 || k < 0 || ldc < (m > 1 ? m : 1) ||
      (products != 0 && !split_products_ok(products)))
    return GB300_ERR_ARG;
  if (m == 0 || n == 0) return GB300_OK;
  unsigned *err = device_error_word();
  if (!err) return GB300_ERR_CUDA;
  return split_sgemm_run(m, n, k, alpha, beta, C, ldc, products, ws, ws_bytes,
                         static_cast<cudaStream_t>(stream), err);
}
GB300_API int gb300_dgemm_ozaki2_prepare(char ta, char tb, int m, int n, int k,
                                         const double *A, int lda, const double *B, int ldb,
                                         int moduli, void *ws, size_t ws_bytes, void *stream) {
  return crt_prepare(ta, tb, m, n, k, A, lda, B, ldb, moduli, ws, ws_bytes,
                     static_cast<cudaStream_t>(stream));
}
GB300_API int gb300_dgemm_ozaki2_run(int m, int n, int k, double alpha, double beta, double *C,
                                     int ldc, int moduli, const void *ws, size_t ws_bytes,
                                     void *stream) {
  if (m < 0 || n < 0 || k < 0 || ldc < (m > 1 ? m : 1) ||
      (moduli != 0 && (moduli < 2 || moduli > kCrtMaxModuli)))
    return GB300_ERR_ARG;
  if (m == 0 || n == 0) return GB300_OK;
  unsigned *err = device_error_word();
  if (!err) return GB300_ERR_CUDA;
  return crt_run(m, n, k, alpha, beta, C, ldc, moduli, ws, ws_bytes,
                 static_cast<cudaStream_t>(stream), err);
}
GB300_API int gb300_dgemm_ozaki_prepare(char ta, char tb, int m, int n, int k, const double *A,
                                        int lda, const double *B, int ldb, int slices, void *ws,
                                        size_t ws_bytes, void *stream) {
  return ozaki_prepare(ta, tb, m, n, k, A, lda, B, ldb, slices, ws, ws_bytes,
                       static_cast<cudaStream_t>(stream));
}
GB300_API int gb300_dgemm_ozaki_run(int m, int n, int k, double alpha, double beta, double *C,
                                    int ldc, int slices, const void *ws, size_t ws_bytes,
                                    void *stream) {
  if (m < 0 || n < 0 || k < 0 || ldc < (m > 1 ? m : 1) ||
      (slices != 0 && (slices < 2 || slices > kOzakiMaxSlices)))
    return GB300_ERR_ARG;
  if (m == 0 || n == 0) return GB300_OK;
  unsigned *err = device_error_word();
  if (!err) return GB300_ERR_CUDA;
  return ozaki_run(m, n, k, alpha, beta, C, ldc, slices, ws, ws_bytes,
                   static_cast<cudaStream_t>(stream), err);
}

// ---------------------------------------------------------------- grouped
GB300_API size_t gb300_grouped_workspace_bytes(int count) { return grouped_workspace_bytes(count); }

GB300_API int gb300_gemm_grouped_ws(const gb300_gemm_problem *problems, int count, void *ws,
                                    size_t ws_bytes, void *stream) {
  for (int i = 0; i < count; ++i) {
    const gb300_gemm_problem &q = problems[i];
    if ((q.precision != 'd' && q.precision != 's') ||
        check_args(q.transa, q.transb, q.m, q.n, q.k, q.lda, q.ldb, q.ldc) == GB300_ERR_ARG)
      return GB300_ERR_ARG;
  }
  if (count <= 0) return count < 0 ? GB300_ERR_ARG : GB300_OK;
  unsigned *err = device_error_word();
  if (!err) return GB300_ERR_CUDA;
  return grouped_plain(problems, count, ws, ws_bytes, static_cast<cudaStream_t>(stream), err);
}

GB300_API int gb300_gemm_grouped(const gb300_gemm_problem *problems, int count, void *stream) {
  for (int i = 0; i < count; ++i) {
    const gb300_gemm_problem &q = problems[i];
    if ((q.precision != 'd' && q.precision != 's') ||
        check_args(q.transa, q.transb, q.m, q.n, q.k, q.lda, q.ldb, q.ldc) == GB300_ERR_ARG)
      return GB300_ERR_ARG;
  }
  if (count <= 0) return count < 0 ? GB300_ERR_ARG : GB300_OK;
  DeviceState *s = dev_state();
  if (!s) return GB300_ERR_CUDA;
  const size_t need = grouped_workspace_bytes(count);
  std::lock_guard<std::mutex> lk(s->mu);
  // the grouped metadata gets its own cache slot (key: stream pointer + 1)
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  void *ws = cached_workspace(s, reinterpret_cast<cudaStream_t>(reinterpret_cast<uintptr_t>(st) + 1),
                              need);
  if (!ws) return GB300_ERR_NOMEM;
  return grouped_plain(problems, count, ws, need, st, s->err);
}

// Split-form batches (form 1) are captured in three phases: the problems'
// operand preparation in parallel branches (forked from and joined into the
// capture stream, problems assigned longest-work-first to the least-loaded
// branch), one grouped persistent launch of the CRT residue GEMMs of all FP64
// problems and one of the 6xBF16 GEMMs of all FP32 problems, then the FP64
// problems' reconstructions in branches.  Each branch prepares its FP32
// problems first: their GEMM launch (on a forked stream) then overlaps the
// FP64 problems' preparation.  Every problem has its own workspace (one
// allocation).  Problems with alpha = 0 or k = 0 run their per-problem call
// in a branch.  GB300_TUNE_GRAPH_BRANCHES (read when a graph is created) sets
// the branch count.  (Grouped launches of the preparation and
// reconstruction kernels too, one per kernel over all problems, measured
// slower on the 1024-problem batch: 12.3 against 10.5 ms, as the phases no
// longer overlap.)
constexpr int kGraphBranches = 64;  // upper bound
constexpr int kDefaultGraphBranches = 32;
static int g_graph_branches = kDefaultGraphBranches;

struct gb300_grouped_graph_s {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  void *meta = nullptr;  // form 0: grouped metadata blob; form 1: the grouped GEMM tables
  void *ws = nullptr;    // form 1: the problems' workspaces
  int device = 0;
  int kernel_nodes = 0, gemm_launches = 0;
};

GB300_API int gb300_grouped_graph_destroy(gb300_grouped_graph g) {
  if (!g) return GB300_ERR_ARG;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  if (g->meta) cudaFree(g->meta);
  if (g->ws) cudaFree(g->ws);
  delete g;
  return GB300_OK;
}

GB300_API int gb300_grouped_graph_stats(gb300_grouped_graph g, int *kernel_nodes,
                                        int *gemm_launches) {
  if (!g || !g->exec) return GB300_ERR_ARG;
  if (kernel_nodes) *kernel_nodes = g->kernel_nodes;
  if (gemm_launches) *gemm_launches = g->gemm_launches;
  return GB300_OK;
}

namespace {
// One problem of a split-form graph: its class, workspace and branch.
struct GraphItem {
  int cls = 0;        // 0: nothing to do, 1: per-problem call, 2: FP64 CRT, 3: FP32 6xBF16
  size_t ws_off = 0, ws_bytes = 0;
  int branch = 0;
  double work = 0;    // LPT weight
  int cost = 0;       // tensor work per tile unit (order inside the grouped launch)
};
constexpr int kGroupProducts = 6;
}  // namespace

GB300_API int gb300_grouped_graph_create(const gb300_gemm_problem *problems, int count, int form,
                                         gb300_grouped_graph *out) {
  if (!out || count < 0 || (count > 0 && !problems) || (form != 0 && form != 1))
    return GB300_ERR_ARG;
  *out = nullptr;
  for (int i = 0; i < count; ++i) {
    const gb300_gemm_problem &q = problems[i];
    if ((q.precision != 'd' && q.precision != 's') ||
        check_args(q.transa, q.transb, q.m, q.n, q.k, q.lda, q.ldb, q.ldc) == GB300_ERR_ARG)
      return GB300_ERR_ARG;
  }
  DeviceState *s = dev_state();
  if (!s) return GB300_ERR_CUDA;
  gb300_grouped_graph g = new (std::nothrow) gb300_grouped_graph_s();
  if (!g) return GB300_ERR_NOMEM;
  cudaGetDevice(&g->device);
  cudaStream_t cs = nullptr, fs = nullptr;  // capture stream, the FP32 GEMM's stream
  int rc = GB300_OK;
  std::vector<uint8_t> blob;
  int used = 0, tiles = 0;
  const int nbr = g_graph_branches;
  cudaStream_t bs[kGraphBranches] = {nullptr};
  cudaEvent_t fork = nullptr, fdone = nullptr, join[kGraphBranches] = {nullptr};
  std::vector<GraphItem> items(count > 0 ? count : 1);
  // form 1: the grouped GEMM tables (FP64 entries, then FP32), in device order
  std::vector<int> ord_d, ord_s;
  std::vector<uint8_t> table;
  int units_d = 0, units_s = 0;
  const size_t eb_d = ozaki_group_entry_bytes(), eb_s = bf16x_group_entry_bytes();
  if (form == 0) {
    rc = grouped_build(problems, count, nullptr, blob, used, tiles);
    if (rc == GB300_OK && used > 0) {
      if (cudaMalloc(&g->meta, blob.size()) != cudaSuccess) rc = GB300_ERR_NOMEM;
      else if (cudaMemcpy(g->meta, blob.data(), blob.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        rc = GB300_ERR_CUDA;
    }
  } else {
    size_t total_ws = 0;
    for (int i = 0; i < count; ++i) {
      const gb300_gemm_problem &q = problems[i];
      GraphItem &it = items[i];
      if (check_args(q.transa, q.transb, q.m, q.n, q.k, q.lda, q.ldb, q.ldc) < 0) continue;
      const int64_t kb = (q.k + 63) / 64;
      if (q.alpha == 0.0 || q.k == 0) {
        it.cls = 1;
        it.work = (double)q.m * q.n + 1e6;
      } else if (q.precision == 'd') {
        it.cls = 2;
        const int N = crt_default_moduli(q.m, q.n, q.k);
        it.ws_bytes = crt_workspace_bytes(q.m, q.n, q.k, N);
        it.cost = (int)(N * kb);
        it.work = (double)(q.m + q.n) * q.k * N + 1e6;
      } else {
        it.cls = 3;
        it.ws_bytes = split_workspace_bytes(0, q.m, q.n, q.k, kGroupProducts);
        it.cost = (int)(6 * kb);
        it.work = (double)(q.m + q.n) * q.k * 3 + 1e6;
      }
      if (it.ws_bytes) {
        it.ws_off = total_ws;
        total_ws += (it.ws_bytes + 1023) / 1024 * 1024;
      }
      if (it.cls == 2) ord_d.push_back(i);
      if (it.cls == 3) ord_s.push_back(i);
    }
    // longest work first onto the least-loaded branch
    std::vector<int> order;
    for (int i = 0; i < count; ++i)
      if (items[i].cls) order.push_back(i);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return items[a].work > items[b].work; });
    double load[kGraphBranches] = {0};
    for (int i : order) {
      int b = 0;
      for (int j = 1; j < nbr; ++j)
        if (load[j] < load[b]) b = j;
      load[b] += items[i].work;
      items[i].branch = b;
    }
    // inside a grouped launch the CTAs take units round-robin: the problems
    // with the costliest tiles go first
    auto by_cost = [&](int a, int b) { return items[a].cost > items[b].cost; };
    std::stable_sort(ord_d.begin(), ord_d.end(), by_cost);
    std::stable_sort(ord_s.begin(), ord_s.end(), by_cost);
    if (total_ws && cudaMalloc(&g->ws, total_ws) != cudaSuccess) rc = GB300_ERR_NOMEM;
    table.resize(ord_d.size() * eb_d + ord_s.size() * eb_s);
    for (size_t j = 0; j < ord_d.size() && rc == GB300_OK; ++j) {
      const gb300_gemm_problem &q = problems[ord_d[j]];
      const GraphItem &it = items[ord_d[j]];
      int u = 0;
      rc = crt_group_entry(q.m, q.n, q.k, q.alpha, q.beta, static_cast<double *>(q.C), q.ldc, 0,
                           static_cast<uint8_t *>(g->ws) + it.ws_off, it.ws_bytes, s->err,
                           units_d, table.data() + j * eb_d, &u);
      units_d += u;
    }
    for (size_t j = 0; j < ord_s.size() && rc == GB300_OK; ++j) {
      const gb300_gemm_problem &q = problems[ord_s[j]];
      const GraphItem &it = items[ord_s[j]];
      int u = 0;
      rc = bf16x_group_entry(q.m, q.n, q.k, (float)q.alpha, (float)q.beta,
                             static_cast<float *>(q.C), q.ldc, kGroupProducts,
                             static_cast<uint8_t *>(g->ws) + it.ws_off, it.ws_bytes, s->err,
                             units_s, table.data() + ord_d.size() * eb_d + j * eb_s, &u);
      units_s += u;
    }
    if (rc == GB300_OK && !table.empty()) {
      if (cudaMalloc(&g->meta, table.size()) != cudaSuccess) rc = GB300_ERR_NOMEM;
      else if (cudaMemcpy(g->meta, table.data(), table.size(), cudaMemcpyHostToDevice) !=
               cudaSuccess)
        rc = GB300_ERR_CUDA;
    }
  }
  if (rc == GB300_OK && cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess)
    rc = GB300_ERR_CUDA;
  if (rc == GB300_OK && form == 1) {
    bool ok = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&fdone, cudaEventDisableTiming) == cudaSuccess &&
              cudaStreamCreateWithFlags(&fs, cudaStreamNonBlocking) == cudaSuccess;
    for (int b = 0; b < nbr && ok; ++b)
      ok = cudaStreamCreateWithFlags(&bs[b], cudaStreamNonBlocking) == cudaSuccess &&
           cudaEventCreateWithFlags(&join[b], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) rc = GB300_ERR_CUDA;
  }
  if (rc == GB300_OK && cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    rc = GB300_ERR_CUDA;
  if (rc == GB300_OK) {
    int rc2 = GB300_OK;
    // fork the branches off the capture stream / join them back into it
    auto fork_all = [&]() {
      if (cudaEventRecord(fork, cs) != cudaSuccess) return false;
      for (int b = 0; b < nbr; ++b)
        if (cudaStreamWaitEvent(bs[b], fork, 0) != cudaSuccess) return false;
      return true;
    };
    auto join_all = [&]() {
      bool ok = true;
      for (int b = 0; b < nbr; ++b)
        ok = cudaEventRecord(join[b], bs[b]) == cudaSuccess &&
             cudaStreamWaitEvent(cs, join[b], 0) == cudaSuccess && ok;
      return ok;
    };
    if (form == 0) {
      if (used > 0) {
        if (cudaMemsetAsync(g->meta, 0, sizeof(int), cs) != cudaSuccess) rc2 = GB300_ERR_CUDA;
        else rc2 = grouped_launch_blob(g->meta, used, tiles, cs, s->err);
      }
    } else {
      // 1. preparation (and the per-problem calls): each branch prepares its
      // FP32 problems first, so that their grouped GEMM (on the forked stream
      // fs) runs while the branches prepare the FP64 problems
      if (!fork_all()) rc2 = GB300_ERR_CUDA;
      for (int pass = 0; pass < 2 && rc2 == GB300_OK; ++pass) {
      if (pass == 1 && !ord_s.empty()) {
        for (int b = 0; b < nbr && rc2 == GB300_OK; ++b)
          if (cudaEventRecord(join[b], bs[b]) != cudaSuccess ||
              cudaStreamWaitEvent(fs, join[b], 0) != cudaSuccess)
            rc2 = GB300_ERR_CUDA;
        if (rc2 == GB300_OK) {
          rc2 = bf16x_group_launch(static_cast<uint8_t *>(g->meta) + ord_d.size() * eb_d,
                                   (int)ord_s.size(), units_s, fs, s->err);
          ++g->gemm_launches;
        }
        if (rc2 == GB300_OK && cudaEventRecord(fdone, fs) != cudaSuccess) rc2 = GB300_ERR_CUDA;
      }
      for (int i = 0; i < count && rc2 == GB300_OK; ++i) {
        const gb300_gemm_problem &q = problems[i];
        const GraphItem &it = items[i];
        if ((it.cls == 2) != (pass == 1)) continue;
        cudaStream_t st = bs[it.branch];
        void *ws = static_cast<uint8_t *>(g->ws) + it.ws_off;
        if (it.cls == 1) {  // C = beta C, as the split calls do it
          const int ld1 = q.m > 1 ? q.m : 1;
          rc2 = q.precision == 'd'
                    ? plain_dgemm('N', 'N', q.m, q.n, 0, q.alpha, nullptr, ld1, nullptr, 1, q.beta,
                                  static_cast<double *>(q.C), q.ldc, st, s->err)
                    : plain_sgemm('N', 'N', q.m, q.n, 0, (float)q.alpha, nullptr, ld1, nullptr, 1,
                                  (float)q.beta, static_cast<float *>(q.C), q.ldc, st, s->err);
        } else if (it.cls == 2) {
          rc2 = crt_prepare(q.transa, q.transb, q.m, q.n, q.k, static_cast<const double *>(q.A),
                            q.lda, static_cast<const double *>(q.B), q.ldb, 0, ws, it.ws_bytes,
                            st);
        } else if (it.cls == 3) {
          rc2 = split_sgemm_prepare(q.transa, q.transb, q.m, q.n, q.k,
                                    static_cast<const float *>(q.A), q.lda,
                                    static_cast<const float *>(q.B), q.ldb, kGroupProducts, ws,
                                    it.ws_bytes, st);
        }
      }
      }
      if (rc2 == GB300_OK && !join_all()) rc2 = GB300_ERR_CUDA;
      // 2. the FP64 problems' grouped GEMM
      if (rc2 == GB300_OK && !ord_d.empty()) {
        rc2 = ozaki_group_launch(g->meta, (int)ord_d.size(), units_d, cs, s->err);
        ++g->gemm_launches;
      }
      // 3. the FP64 problems' reconstruction
      if (rc2 == GB300_OK && !ord_d.empty()) {
        if (!fork_all()) rc2 = GB300_ERR_CUDA;
        for (size_t j = 0; j < ord_d.size() && rc2 == GB300_OK; ++j) {
          const gb300_gemm_problem &q = problems[ord_d[j]];
          const GraphItem &it = items[ord_d[j]];
          rc2 = crt_group_reconstruct(q.m, q.n, q.k, q.alpha, q.beta, static_cast<double *>(q.C),
                                      q.ldc, 0, static_cast<uint8_t *>(g->ws) + it.ws_off,
                                      it.ws_bytes, bs[it.branch]);
        }
        if (rc2 == GB300_OK && !join_all()) rc2 = GB300_ERR_CUDA;
      }
      if (rc2 == GB300_OK && !ord_s.empty() && cudaStreamWaitEvent(cs, fdone, 0) != cudaSuccess)
        rc2 = GB300_ERR_CUDA;
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(cs, &graph);
    g->graph = graph;
    if (rc2 != GB300_OK) rc = rc2;
    else if (e != cudaSuccess || !graph) rc = GB300_ERR_CUDA;
    else if (cudaGraphInstantiate(&g->exec, graph, 0) != cudaSuccess) rc = GB300_ERR_CUDA;
    if (rc == GB300_OK) {
      size_t nn = 0;
      if (cudaGraphGetNodes(graph, nullptr, &nn) == cudaSuccess && nn) {
        std::vector<cudaGraphNode_t> nodes(nn);
        if (cudaGraphGetNodes(graph, nodes.data(), &nn) == cudaSuccess)
          for (size_t j = 0; j < nn; ++j) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nodes[j], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel)
              ++g->kernel_nodes;
          }
      }
      if (form == 0 && used > 0) g->gemm_launches = 1;
    }
  }
  if (cs) cudaStreamDestroy(cs);
  for (int b = 0; b < kGraphBranches; ++b) {
    if (bs[b]) cudaStreamDestroy(bs[b]);
    if (join[b]) cudaEventDestroy(join[b]);
  }
  if (fork) cudaEventDestroy(fork);
  if (fdone) cudaEventDestroy(fdone);
  if (fs) cudaStreamDestroy(fs);
  if (rc != GB300_OK) {
    gb300_grouped_graph_destroy(g);
    return rc;
  }
  *out = g;
  return GB300_OK;
}

GB300_API int gb300_grouped_graph_launch(gb300_grouped_graph g, void *stream) {
  if (!g || !g->exec) return GB300_ERR_ARG;
  return cudaGraphLaunch(g->exec, static_cast<cudaStream_t>(stream)) == cudaSuccess ? GB300_OK
                                                                                    : GB300_ERR_CUDA;
}

// ---------------------------------------------------------------- TRSM / TRMM
template <typename T>
static int tr_api(int solve, char side, char uplo, char ta, char diag, int m, int n, T alpha,
                  const T *A, int lda, T *B, int ldb, int form, void *stream) {
  const int ck = tr_check(side, uplo, ta, diag, m, n, lda, ldb);
  if (ck != GB300_OK) return ck < 0 ? GB300_OK : ck;
  if (form < 0 || form > 2) return GB300_ERR_ARG;
  DeviceState *s = dev_state();
  if (!s) return GB300_ERR_CUDA;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t need = tr_workspace_bytes(sizeof(T) == 8, form, m, n);
  std::lock_guard<std::mutex> lk(s->mu);
  void *ws = need ? cached_workspace(s, st, need) : nullptr;
  if (need && !ws) return GB300_ERR_NOMEM;
  if constexpr (sizeof(T) == 8)
    return trsm_d(solve, side, uplo, ta, diag, m, n, alpha, A, lda, B, ldb, form, ws, need, st,
                  s->err);
  else
    return trsm_s(solve, side, uplo, ta, diag, m, n, alpha, A, lda, B, ldb, form, ws, need, st,
                  s->err);
}

GB300_API int gb300_dtrsm(char side, char uplo, char transa, char diag, int m, int n,
                          double alpha, const double *A, int lda, double *B, int ldb, int form,
                          void *stream) {
  return tr_api<double>(1, side, uplo, transa, diag, m, n, alpha, A, lda, B, ldb, form, stream);
}
GB300_API int gb300_strsm(char side, char uplo, char transa, char diag, int m, int n, float alpha,
                          const float *A, int lda, float *B, int ldb, int form, void *stream) {
  return tr_api<float>(1, side, uplo, transa, diag, m, n, alpha, A, lda, B, ldb, form, stream);
}
GB300_API int gb300_dtrmm(char side, char uplo, char transa, char diag, int m, int n,
                          double alpha, const double *A, int lda, double *B, int ldb, int form,
                          void *stream) {
  return tr_api<double>(0, side, uplo, transa, diag, m, n, alpha, A, lda, B, ldb, form, stream);
}
GB300_API int gb300_strmm(char side, char uplo, char transa, char diag, int m, int n, float alpha,
                          const float *A, int lda, float *B, int ldb, int form, void *stream) {
  return tr_api<float>(0, side, uplo, transa, diag, m, n, alpha, A, lda, B, ldb, form, stream);
}

// Reads the per-device word and the no-allocation entry point's word without
// allocating either: a device on which no kernel has run yet has no error.
GB300_API unsigned gb300_device_error(int clear) {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= kMaxDevices) return 0xFFFFFFFFu;
  unsigned *err = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_init_mu);
    err = g_dev[d].err;
  }
  unsigned w = 0;
  if (err) {
    if (cudaMemcpy(&w, err, sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess)
      return 0xFFFFFFFFu;
    if (clear && w && cudaMemset(err, 0, sizeof(unsigned)) != cudaSuccess) return 0xFFFFFFFFu;
  }
  unsigned wn = 0;
  if (noalloc_error_read(clear, &wn) != GB300_OK) return 0xFFFFFFFFu;
  return w ? w : wn;
}

GB300_API int gb300_selftest_wait_timeout(unsigned poll_limit) {
  DeviceState *s = dev_state();
  if (!s) return GB300_ERR_CUDA;
  int *flag = nullptr;
  if (cudaMalloc(&flag, sizeof(int)) != cudaSuccess) return GB300_ERR_CUDA;
  cudaMemset(flag, 0, sizeof(int));
  wait_timeout_selftest_kernel<<<1, 32>>>(poll_limit, s->err, flag);
  int reached = 0;
  cudaError_t e = cudaMemcpy(&reached, flag, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(flag);
  if (e != cudaSuccess) return GB300_ERR_CUDA;
  unsigned w = 0;
  cudaMemcpy(&w, s->err, sizeof(unsigned), cudaMemcpyDeviceToHost);
  if (reached == 1 && w == kErrTimeoutFull) return GB300_ERR_TIMEOUT;
  return reached == 2 ? GB300_OK : GB300_ERR_CUDA;
}

GB300_API int gb300_autotune(int kind, char ta, char tb, int m, int n, int k, const void *A,
                             int lda, const void *B, int ldb, void *stream, int *chosen) {
  if (kind < 0 || kind > 4) return GB300_ERR_ARG;
  if (check_args(ta, tb, m, n, k, lda, ldb, m > 1 ? m : 1) != GB300_OK || k == 0)
    return GB300_ERR_ARG;
  unsigned *err = device_error_word();
  if (!err) return GB300_ERR_CUDA;
  return autotune(kind, ta, tb, m, n, k, A, lda, B, ldb, static_cast<cudaStream_t>(stream), err,
                  chosen);
}
GB300_API int gb300_tune_lookup(int kind, int m, int n, int k, int *param, int *chunk) {
  if (kind < 0 || kind > 4) return GB300_ERR_ARG;
  int p = 0, c = 0;
  if (kind == 0) bf16x_resolve(m, n, k, &p, &c);
  else if (kind == 1) p = ozaki_default_slices(m, n, k);
  else if (kind == 2) p = crt_default_moduli(m, n, k);
  else p = plain_split_k(kind == 3, m, n, k);
  if (param) *param = p;
  if (chunk) *chunk = c;
  return tune_lookup(kind, m, n, k, nullptr, nullptr) ? GB300_OK : GB300_ERR_UNSUPPORTED;
}
GB300_API int gb300_tune_layout(int kind, int m, int n, int k, int *tile_n, int *pair_mma) {
  if (kind < 0 || kind > 2) return GB300_ERR_ARG;
  if (tile_n) *tile_n = split_tile_n(kind, m, n, k);
  if (pair_mma) {
    const int o = pair_mma_override();
    const int v = o ? o : tune_pair_mma(kind, m, n, k);
    *pair_mma = v ? v : 1;
  }
  return tune_lookup(kind, m, n, k, nullptr, nullptr) ? GB300_OK : GB300_ERR_UNSUPPORTED;
}
GB300_API int gb300_plain_layout(int is_double, int m, int n, int k, int *split_k, int *stages) {
  if (m < 0 || n < 0 || k < 0) return GB300_ERR_ARG;
  const int kind = is_double ? 3 : 4;
  if (split_k) *split_k = plain_split_k(is_double != 0, m, n, k);
  if (stages) {
    const int o = plain_stages_override();
    const int v = o ? o : tune_plain_stages(kind, m, n, k);
    *stages = v ? v : 4;
  }
  return tune_lookup(kind, m, n, k, nullptr, nullptr) ? GB300_OK : GB300_ERR_UNSUPPORTED;
}
GB300_API int gb300_tune_cache_save(const char *path) { return tune_cache_save(path); }
GB300_API int gb300_tune_cache_load(const char *path, int *loaded) {
  return tune_cache_load(path, loaded);
}
GB300_API void gb300_tune_cache_clear(void) { tune_cache_clear(); }

GB300_API int gb300_tune_param(int param, int value) {
  switch (param) {
    case GB300_TUNE_BF16X_CHUNK:
      set_bf16x_chunk_kblocks(value);
      return GB300_OK;
    case GB300_TUNE_TILE_N:
      if (value != 0 && value != 128 && value != 256) return GB300_ERR_ARG;
      set_split_tile_n(value);
      return GB300_OK;
    case GB300_TUNE_PAIR_MMA:
      if (value < 0 || value > 2) return GB300_ERR_ARG;
      set_pair_mma(value);
      return GB300_OK;
    case GB300_TUNE_GRAPH_BRANCHES:
      if (value < 0 || value > kGraphBranches) return GB300_ERR_ARG;
      g_graph_branches = value ? value : kDefaultGraphBranches;
      return GB300_OK;
    case GB300_TUNE_HOST_PARTS:
      if (value < 0 || value > 8) return GB300_ERR_ARG;
      g_host_parts = value;
      return GB300_OK;
    case GB300_TUNE_MODULUS_SPLIT:
      if (value < 0 || value > 2) return GB300_ERR_ARG;
      set_modulus_split(value);
      return GB300_OK;
    case GB300_TUNE_SPLIT_K:
      if (value < 0 || value > 65535) return GB300_ERR_ARG;
      set_plain_split_k(value);
      return GB300_OK;
    case GB300_TUNE_PLAIN_STAGES:
      if (value != 0 && value != 4 && value != 6) return GB300_ERR_ARG;
      set_plain_stages(value);
      return GB300_OK;
    default:
      return GB300_ERR_ARG;
  }
}

GB300_API const char *gb300_version(void) { return "gemm_gb300 0.1 (sm_103a)"; }
