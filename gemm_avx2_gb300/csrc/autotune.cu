// autotune.cu -- measured choice of the split forms' parameters, cached per
// shape class.  It replaces the reference's compile-time tune headers
// (wjc404/GEMM_AVX2 dgemm_tune.h, sgemm_tune.h, clamped and expanded in
// src/gemm_set_parameters.h:1-61), which fix block sizes once per build for one
// CPU model, by a run-time search on the GPU the library runs on:
//
//   split SGEMM : products P in {3, 6} (BF16 terms) or the scaled 3xFP16
//                 form, x hi*hi chunk length in {2, 4, 8};
//   all forms   : then the output tile width (128 / 256) of the chosen one,
//                 and its cluster mode (pair MMAs on 2-CTA clusters or one
//                 CTA per tile);
//   Ozaki DGEMM : slice count S in [4, 12];
//   plain D/SGEMM (kinds 3, 4): split-K factor in {1, 2, 3, 4, 6, 8, 12, 16, 24, 32}
//                 (at least 8 k-tiles a slice) x ring depth {4, 6}: the
//                 fastest, since every split sums the same products in K
//                 order within the same rounding bound (the reference's own
//                 K blocking, src/gemm_driver.c:156-190).
//
// A candidate qualifies when its max and Frobenius relative errors against a
// near-exact FP64 reference do not exceed those of the plain kernel on the
// same operands ("equal error"); the fastest qualifying candidate wins (for
// Ozaki: the smallest S, which is also the fastest).  The reference is the
// Ozaki form with S = 12 -- 84 bits per operand, whose truncation lies far
// below FP64 rounding -- run on FP64 copies of the operands for FP32 problems,
// where every product is then exact.
//
// Shape class: form and floor(log2) of m, n, k (the GEMM kernels read K-major
// workspace whatever the transposes, and the precision choice depends on the
// data, not the layout).  The cache is
// a JSON file (gb300_tune_cache_save / _load; path argument or the
// GB300_TUNE_CACHE environment variable); a missing or unreadable file leaves
// the built-in defaults (P = 6, chunk 4, S = 8).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "plain_gemm.h"
#include "split_gemm.h"

namespace gb300 {

struct TuneEntry {
  int param = 0;       // products (BF16xP), slices (Ozaki), moduli (CRT) or split-K (plain)
  int chunk = 0;       // BF16xP hi*hi chunk length (0 for Ozaki)
  int tile = 0;        // output tile width of the GEMM (128 / 256; 0 = by shape)
  int pair = 0;        // cluster mode (1 pair MMAs, 2 one CTA per tile; 0 = default)
  int stages = 0;      // plain kernels' ring depth (4 / 6; 0 = default)
  double ms = 0;       // measured time of the chosen candidate
  double err_max = 0, err_fro = 0;              // chosen candidate vs reference
  double plain_max = 0, plain_fro = 0;          // plain kernel vs reference
};

static std::map<std::string, TuneEntry> g_tune;
static std::mutex g_tune_mu;

static int ilog2(int x) {
  int l = 0;
  while (x > 1) { x >>= 1; ++l; }
  return l;
}

static const char *kind_name(int kind) {
  static const char *names[5] = {"bf16x", "ozaki", "crt", "plain_d", "plain_s"};
  return kind >= 0 && kind < 5 ? names[kind] : "?";
}

static std::string tune_key(int kind, int m, int n, int k) {
  char buf[96];
  snprintf(buf, sizeof buf, "%s:%d:%d:%d", kind_name(kind), ilog2(m), ilog2(n), ilog2(k));
  return buf;
}

bool tune_lookup(int kind, int m, int n, int k, int *param, int *chunk) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune.find(tune_key(kind, m, n, k));
  if (it == g_tune.end()) return false;
  if (param) *param = it->second.param;
  if (chunk) *chunk = it->second.chunk;
  return true;
}

int tune_tile_n(int kind, int m, int n, int k) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune.find(tune_key(kind, m, n, k));
  return it == g_tune.end() ? 0 : it->second.tile;
}

int tune_pair_mma(int kind, int m, int n, int k) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune.find(tune_key(kind, m, n, k));
  return it == g_tune.end() ? 0 : it->second.pair;
}

int tune_plain_split(int kind, int m, int n, int k) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune.find(tune_key(kind, m, n, k));
  return it == g_tune.end() ? 0 : it->second.param;
}

int tune_plain_stages(int kind, int m, int n, int k) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune.find(tune_key(kind, m, n, k));
  return it == g_tune.end() ? 0 : it->second.stages;
}

// ---------------------------------------------------------------- device helpers
// dst (FP64, column-major, ld = rows) = src (FP32, column-major, ld) over rows x cols
__global__ void widen_kernel(const float *__restrict__ src, int ld, int rows, int cols,
                             double *__restrict__ dst) {
  const int64_t total = (int64_t)rows * cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e / rows), r = (int)(e % rows);
    dst[e] = (double)src[(int64_t)c * ld + r];
  }
}

// stats[0] += sum (t - r)^2, stats[1] += sum r^2, stats[2] = max |t - r| / |r|
// (as the bit pattern of a non-negative double), over an m x n window.
template <typename T>
__global__ void err_stats_kernel(const T *__restrict__ t, int ldt, const double *__restrict__ r,
                                 int ldr, int m, int n, double *stats) {
  double s_d = 0, s_r = 0, mx = 0;
  const int64_t total = (int64_t)m * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e / m), i = (int)(e % m);
    const double tv = (double)t[(int64_t)c * ldt + i], rv = r[(int64_t)c * ldr + i];
    const double d = tv - rv;
    s_d += d * d;
    s_r += rv * rv;
    const double rel = rv != 0.0 ? fabs(d) / fabs(rv) : (d != 0.0 ? 1e300 : 0.0);
    mx = rel > mx ? rel : mx;
  }
  for (int o = 16; o > 0; o >>= 1) {
    s_d += __shfl_xor_sync(0xffffffffu, s_d, o);
    s_r += __shfl_xor_sync(0xffffffffu, s_r, o);
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&stats[0], s_d);
    atomicAdd(&stats[1], s_r);
    atomicMax(reinterpret_cast<unsigned long long *>(&stats[2]),
              (unsigned long long)__double_as_longlong(mx));
  }
}

// ---------------------------------------------------------------- tuning run
namespace {
struct DevBuf {
  void *p = nullptr;
  ~DevBuf() { if (p) cudaFree(p); }
  bool alloc(size_t n) { return cudaMalloc(&p, n > 0 ? n : 1) == cudaSuccess; }
};

struct Stats {
  double max_rel, fro;
};

int measure(const void *t, bool t_double, int m, int n, const double *ref, double *dstats,
            cudaStream_t st, Stats *out) {
  if (cudaMemsetAsync(dstats, 0, 3 * sizeof(double), st) != cudaSuccess) return GB300_ERR_CUDA;
  const int64_t total = (int64_t)m * n;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 2048) blocks = 2048;
  if (t_double)
    err_stats_kernel<double><<<blocks, 256, 0, st>>>(static_cast<const double *>(t), m, ref, m,
                                                      m, n, dstats);
  else
    err_stats_kernel<float><<<blocks, 256, 0, st>>>(static_cast<const float *>(t), m, ref, m, m,
                                                     n, dstats);
  double h[3];
  if (cudaMemcpyAsync(h, dstats, sizeof h, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return GB300_ERR_CUDA;
  out->fro = h[1] > 0 ? std::sqrt(h[0] / h[1]) : std::sqrt(h[0]);
  out->max_rel = h[2];
  return GB300_OK;
}
}  // namespace

int autotune(int kind, char ta, char tb, int m, int n, int k, const void *A, int lda,
             const void *B, int ldb, cudaStream_t st, unsigned *err, int *chosen) {
  if (kind < 0 || kind > 4) return GB300_ERR_ARG;
  const int ck = check_args(ta, tb, m, n, k, lda, ldb, m > 1 ? m : 1);
  if (ck != GB300_OK || k == 0) return ck == GB300_ERR_ARG ? ck : GB300_ERR_ARG;
  const bool f32 = kind == 0 || kind == 4;   // FP32 operands
  const bool plain_kind = kind >= 3;         // the plain kernels' split-K and ring depth
  const bool an = notrans(ta), bn = notrans(tb);
  const int ar = an ? m : k, ac = an ? k : m, br = bn ? k : n, bc = bn ? n : k;
  const size_t mn = (size_t)m * n;
  DevBuf cref, ctest, a64, b64, ws, dstats;
  const size_t ws_ref = split_workspace_bytes(1, m, n, k, 12);
  size_t ws_need = ws_ref;
  if (kind == 0) {
    const size_t w6 = split_workspace_bytes(0, m, n, k, 6);
    if (w6 > ws_need) ws_need = w6;
  } else if (kind == 2) {
    const size_t wc = crt_workspace_bytes(m, n, k, kCrtMaxModuli);
    if (wc > ws_need) ws_need = wc;
  } else if (plain_kind) {
    const size_t wp = 16 * mn * (f32 ? 4 : 8);  // the slices of the largest split
    if (wp > ws_need) ws_need = wp;
  }
  if (!cref.alloc(mn * 8) || !ctest.alloc(mn * (f32 ? 4 : 8)) || !ws.alloc(ws_need) ||
      !dstats.alloc(3 * sizeof(double)))
    return GB300_ERR_NOMEM;
  const double *Ad = static_cast<const double *>(A), *Bd = static_cast<const double *>(B);
  int Alda = lda, Bldb = ldb;
  if (f32) {  // exact FP64 copies of the FP32 operands for the reference
    if (!a64.alloc((size_t)ar * ac * 8) || !b64.alloc((size_t)br * bc * 8)) return GB300_ERR_NOMEM;
    widen_kernel<<<1024, 256, 0, st>>>(static_cast<const float *>(A), lda, ar, ac,
                                       static_cast<double *>(a64.p));
    widen_kernel<<<1024, 256, 0, st>>>(static_cast<const float *>(B), ldb, br, bc,
                                       static_cast<double *>(b64.p));
    Ad = static_cast<const double *>(a64.p);
    Bd = static_cast<const double *>(b64.p);
    Alda = ar;
    Bldb = br;
  }
  double *Cr = static_cast<double *>(cref.p);
  double *stats = static_cast<double *>(dstats.p);
  int rc = cudaMemsetAsync(Cr, 0, mn * 8, st) == cudaSuccess ? GB300_OK : GB300_ERR_CUDA;
  if (rc == GB300_OK)
    rc = ozaki_dgemm(ta, tb, m, n, k, 1.0, Ad, Alda, Bd, Bldb, 0.0, Cr, m, 12, ws.p, ws_ref, st,
                     err);
  if (rc != GB300_OK) return rc;

  // run one candidate into ctest (C = 0 first: beta = 0 still multiplies C)
  // (plain kinds: form 1 is the plain kernel with room for the split-K
  // slices, split and depth as set by the knobs)
  auto run = [&](int form, int param, int chunk) -> int {
    if (cudaMemsetAsync(ctest.p, 0, mn * (f32 ? 4 : 8), st) != cudaSuccess)
      return GB300_ERR_CUDA;
    void *pws = (plain_kind && form == 1) ? ws.p : nullptr;
    const size_t pwb = pws ? ws_need : 0;
    if (f32) {
      float *Ct = static_cast<float *>(ctest.p);
      if (form == 0 || plain_kind)
        return plain_sgemm(ta, tb, m, n, k, 1.0f, static_cast<const float *>(A), lda,
                           static_cast<const float *>(B), ldb, 0.0f, Ct, m, st, err, pws, pwb);
      return split_sgemm(ta, tb, m, n, k, 1.0f, static_cast<const float *>(A), lda,
                         static_cast<const float *>(B), ldb, 0.0f, Ct, m, param, ws.p, ws_need,
                         st, err, chunk);
    }
    double *Ct = static_cast<double *>(ctest.p);
    if (form == 0 || plain_kind)
      return plain_dgemm(ta, tb, m, n, k, 1.0, static_cast<const double *>(A), lda,
                         static_cast<const double *>(B), ldb, 0.0, Ct, m, st, err, pws, pwb);
    if (kind == 2)
      return crt_dgemm(ta, tb, m, n, k, 1.0, static_cast<const double *>(A), lda,
                       static_cast<const double *>(B), ldb, 0.0, Ct, m, param, ws.p, ws_need, st,
                       err);
    return ozaki_dgemm(ta, tb, m, n, k, 1.0, static_cast<const double *>(A), lda,
                       static_cast<const double *>(B), ldb, 0.0, Ct, m, param, ws.p, ws_need, st,
                       err);
  };
  auto timed = [&](int param, int chunk, double *ms) -> int {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int r = run(1, param, chunk);  // warm-up (and the result measured for accuracy)
    cudaEventRecord(e0, st);
    for (int i = 0; i < 2 && r == GB300_OK; ++i) r = run(1, param, chunk);
    cudaEventRecord(e1, st);
    float t = 0;
    if (r == GB300_OK && cudaEventSynchronize(e1) == cudaSuccess) cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = t / 2;
    return r;
  };

  // the bar: the plain kernel with one K slice (no workspace, so split-K
  // off), the full-K accumulation whose error the split forms must match
  Stats plain{};
  if ((rc = run(0, 0, 0)) != GB300_OK) return rc;
  if ((rc = measure(ctest.p, !f32, m, n, Cr, stats, st, &plain)) != GB300_OK) return rc;

  TuneEntry best;
  bool found = false;
  if (plain_kind) {
    // split-K x ring depth: the fastest (the caller's knobs are restored)
    const int user_split = plain_split_override(), user_stages = plain_stages_override();
    const int BK = f32 ? 32 : 16, ktiles = (k + BK - 1) / BK;
    const int splits[10] = {1, 2, 3, 4, 6, 8, 12, 16, 24, 32}, depths[2] = {4, 6};
    for (int S : splits) {
      if (S > 1 && ktiles / S < 8) break;
      for (int d : depths) {
        set_plain_split_k(S);
        set_plain_stages(d);
        double ms = 0;
        rc = timed(0, 0, &ms);
        Stats e{};
        if (rc == GB300_OK) rc = measure(ctest.p, !f32, m, n, Cr, stats, st, &e);
        if (rc != GB300_OK) break;
        if (!found || ms < best.ms) {
          found = true;
          best.param = S; best.stages = d; best.ms = ms;
          best.err_max = e.max_rel; best.err_fro = e.fro;
        }
      }
      if (rc != GB300_OK) break;
    }
    set_plain_split_k(user_split);
    set_plain_stages(user_stages);
    if (rc != GB300_OK) return rc;
    best.plain_max = plain.max_rel;
    best.plain_fro = plain.fro;
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      g_tune[tune_key(kind, m, n, k)] = best;
    }
    if (chosen) *chosen = best.param;
    return GB300_OK;
  }
  if (kind == 0) {
    const int Ps[3] = {3, 6, kFp16x3}, chunks[3] = {2, 4, 8};
    for (int P : Ps)
      for (int c : chunks) {
        double ms = 0;
        Stats e{};
        if ((rc = timed(P, c, &ms)) != GB300_OK) return rc;
        if ((rc = measure(ctest.p, false, m, n, Cr, stats, st, &e)) != GB300_OK) return rc;
        const bool ok = e.max_rel <= plain.max_rel && e.fro <= plain.fro;
        if (ok && (!found || ms < best.ms)) {
          found = true;
          best.param = P; best.chunk = c; best.ms = ms;
          best.err_max = e.max_rel; best.err_fro = e.fro;
        }
      }
    if (!found) { best.param = 6; best.chunk = 2; }  // most accurate candidate
  } else if (kind == 2) {
    // the smallest moduli count at equal error is also the fastest
    for (int N = 11; N <= kCrtMaxModuli; ++N) {
      if (crt_bits_for(N, k) < 1) continue;
      double ms = 0;
      Stats e{};
      if ((rc = timed(N, 0, &ms)) != GB300_OK) return rc;
      if ((rc = measure(ctest.p, true, m, n, Cr, stats, st, &e)) != GB300_OK) return rc;
      if (e.max_rel <= plain.max_rel && e.fro <= plain.fro) {
        found = true;
        best.param = N; best.ms = ms; best.err_max = e.max_rel; best.err_fro = e.fro;
        break;
      }
    }
    if (!found) best.param = kCrtMaxModuli;
  } else {
    for (int S = 4; S <= 12; ++S) {
      double ms = 0;
      Stats e{};
      if ((rc = timed(S, 0, &ms)) != GB300_OK) return rc;
      if ((rc = measure(ctest.p, true, m, n, Cr, stats, st, &e)) != GB300_OK) return rc;
      if (e.max_rel <= plain.max_rel && e.fro <= plain.fro) {
        found = true;
        best.param = S; best.ms = ms; best.err_max = e.max_rel; best.err_fro = e.fro;
        break;
      }
    }
    if (!found) best.param = 12;
  }
  // The output tile width, then the tensor-core GEMM's cluster mode at that
  // width: the results are the same bit for bit, so only the time decides.
  // The two candidates are timed alternately over kLayoutRounds rounds and
  // compared by their fastest round, so that a clock or power-cap transient
  // during one timing does not decide (the caller's own overrides are
  // restored afterwards).
  constexpr int kLayoutRounds = 3;
  auto faster_of = [&](auto set, int a, int b, int *pick, double *ms) -> int {
    double ta = 1e30, tb = 1e30;
    for (int r = 0; r < kLayoutRounds; ++r) {
      double t = 0;
      set(a);
      int e = timed(best.param, best.chunk, &t);
      if (e != GB300_OK) return e;
      ta = t < ta ? t : ta;
      set(b);
      e = timed(best.param, best.chunk, &t);
      if (e != GB300_OK) return e;
      tb = t < tb ? t : tb;
    }
    *pick = ta <= tb ? a : b;
    *ms = ta <= tb ? ta : tb;
    return GB300_OK;
  };
  {
    const int user_tile = split_tile_override(), user_pair = pair_mma_override();
    rc = faster_of([](int v) { set_split_tile_n(v); }, 256, 128, &best.tile, &best.ms);
    if (rc == GB300_OK) {
      set_split_tile_n(best.tile);
      rc = faster_of([](int v) { set_pair_mma(v); }, 1, 2, &best.pair, &best.ms);
    }
    set_pair_mma(user_pair);
    set_split_tile_n(user_tile);
    if (rc != GB300_OK) return rc;
  }
  best.plain_max = plain.max_rel;
  best.plain_fro = plain.fro;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[tune_key(kind, m, n, k)] = best;
  }
  if (chosen) *chosen = best.param;
  return GB300_OK;
}

// ---------------------------------------------------------------- cache file
static std::string cache_path(const char *path) {
  if (path && *path) return path;
  const char *env = getenv("GB300_TUNE_CACHE");
  if (env && *env) return env;
  const char *home = getenv("HOME");
  return std::string(home ? home : ".") + "/.gemm_gb300_tune.json";
}

int tune_cache_save(const char *path) {
  const std::string p = cache_path(path);
  FILE *f = fopen(p.c_str(), "w");
  if (!f) return GB300_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  fprintf(f, "{\"version\": 1, \"entries\": [\n");
  size_t i = 0;
  for (const auto &kv : g_tune) {
    const TuneEntry &e = kv.second;
    fprintf(f,
            "  {\"key\": \"%s\", \"param\": %d, \"chunk\": %d, \"ms\": %.6g, \"err_max\": %.6g, "
            "\"err_fro\": %.6g, \"plain_max\": %.6g, \"plain_fro\": %.6g, \"tile\": %d, "
            "\"pair\": %d, \"stages\": %d}%s\n",
            kv.first.c_str(), e.param, e.chunk, e.ms, e.err_max, e.err_fro, e.plain_max,
            e.plain_fro, e.tile, e.pair, e.stages, ++i < g_tune.size() ? "," : "");
  }
  fprintf(f, "]}\n");
  return fclose(f) == 0 ? GB300_OK : GB300_ERR_ARG;
}

// Reads entries written by tune_cache_save.  Lines that do not parse, keys of
// unknown forms and out-of-range values are skipped; an unreadable file
// returns GB300_ERR_ARG and leaves the cache as it was.
int tune_cache_load(const char *path, int *loaded) {
  const std::string p = cache_path(path);
  FILE *f = fopen(p.c_str(), "r");
  if (loaded) *loaded = 0;
  if (!f) return GB300_ERR_ARG;
  char line[512];
  std::map<std::string, TuneEntry> add;
  while (fgets(line, sizeof line, f)) {
    char key[96];
    TuneEntry e;
    if (sscanf(line,
               " {\"key\": \"%95[^\"]\", \"param\": %d, \"chunk\": %d, \"ms\": %lf, \"err_max\": "
               "%lf, \"err_fro\": %lf, \"plain_max\": %lf, \"plain_fro\": %lf",
               key, &e.param, &e.chunk, &e.ms, &e.err_max, &e.err_fro, &e.plain_max,
               &e.plain_fro) != 8)
      continue;
    // optional (files from before it was tuned have no tile width)
    const char *tp = strstr(line, "\"tile\":");
    if (tp && sscanf(tp, "\"tile\": %d", &e.tile) != 1) e.tile = 0;
    if (e.tile != 128 && e.tile != 256) e.tile = 0;
    const char *pp = strstr(line, "\"pair\":");
    if (pp && sscanf(pp, "\"pair\": %d", &e.pair) != 1) e.pair = 0;
    if (e.pair != 1 && e.pair != 2) e.pair = 0;
    const char *sp = strstr(line, "\"stages\":");
    if (sp && sscanf(sp, "\"stages\": %d", &e.stages) != 1) e.stages = 0;
    if (e.stages != 4 && e.stages != 6) e.stages = 0;
    const bool bx = strncmp(key, "bf16x:", 6) == 0, oz = strncmp(key, "ozaki:", 6) == 0;
    const bool cr = strncmp(key, "crt:", 4) == 0;
    const bool pl = strncmp(key, "plain_d:", 8) == 0 || strncmp(key, "plain_s:", 8) == 0;
    if (bx && split_products_ok(e.param) && e.chunk >= 0 && e.chunk <= 64)
      add[key] = e;
    else if (oz && e.param >= 2 && e.param <= kOzakiMaxSlices)
      add[key] = e;
    else if (cr && e.param >= 2 && e.param <= kCrtMaxModuli)
      add[key] = e;
    else if (pl && e.param >= 1 && e.param <= 32)
      add[key] = e;
  }
  fclose(f);
  std::lock_guard<std::mutex> lk(g_tune_mu);
  for (auto &kv : add) g_tune[kv.first] = kv.second;
  if (loaded) *loaded = (int)add.size();
  return GB300_OK;
}

void tune_cache_clear() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune.clear();
}

}  // namespace gb300
