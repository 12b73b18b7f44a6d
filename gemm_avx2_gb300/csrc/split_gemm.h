// split_gemm.h -- internal declarations of the tensor-core split forms.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace gb300 {

// Geometry shared by the split kernels and the workspace sizing.
constexpr int kSplitBK = 64;       // K elements per pipeline stage (128 B of BF16)
constexpr int kSplitBM = 128;      // tile rows (TMEM lanes)
constexpr int kBf16xBN = 256;      // tile columns of the BF16xP SGEMM
constexpr int kOzakiBN = 256;      // tile columns of the Ozaki DGEMM
constexpr int kOzakiMaxSlices = 12;
constexpr int kCrtMaxModuli = 24;  // moduli of the CRT (modular-integer) FP64 form

// `products` code of the scaled 3xFP16 SGEMM form (GB300_SPLIT_FP16X3): rows of
// op(A) / columns of op(B) scaled by powers of two into the FP16 range, FP16
// hi + lo terms, products hi*hi + (hi*lo + lo*hi) * 2^-11.
constexpr int kFp16x3 = 0x103;
inline bool split_products_ok(int p) { return p == 3 || p == 6 || p == kFp16x3; }
// Segments of the product stream (6xBF16: 6; 3xBF16 and the scaled FP16 form:
// 3) and distinct terms stored per operand (3 and 2).
inline int split_segments(int p) { return p == 6 ? 6 : 3; }
inline int split_terms(int p) { return p == 6 ? 3 : 2; }

size_t split_workspace_bytes(int kind, int m, int n, int k, int param);

// products: 3 / 6 (BF16 terms), kFp16x3, or 0 = the autotuned choice for the
// shape class (default 6); chunk0 = hi*hi chunk length in 64-wide K blocks
// (0 = tuned / knob / default).
int split_sgemm(char ta, char tb, int m, int n, int k, float alpha, const float *A, int lda,
                const float *B, int ldb, float beta, float *C, int ldc, int products, void *ws,
                size_t ws_bytes, cudaStream_t st, unsigned *err, int chunk0 = 0);

// The slice-product tcgen05 GEMM shared by the slice (mode 0) and CRT (mode 1)
// FP64 forms: operands are S blocks of Mp (Np) rows x Kp of BF16-held integers.
struct OzakiGemmArgs {
  int m, n, S, mode;
  int k;  // the problem's K (its shape class picks the tuned tile width)
  int64_t Mp, Np, Kp;
  const void *As, *Bs;
  double alpha, beta;
  double *C;
  int ldc;
  const int *expA, *expB;
  double *res;        // mode 0: Mp x Np FP64 scratch
  uint8_t *rres;      // mode 1: S x Mp x Np residues
  const int *mods;    // mode 1: the S moduli
  // mode 1, a sub-block of a larger problem: its first row of op(A) and
  // column of op(B) in the operand blocks (Mp, Np: the whole problem's; m, n:
  // the block's; rres, expA, expB point at the block's first entries)
  int row0 = 0, col0 = 0;
  // the whole problem's m and n: the operand blocks' rows that hold data (the
  // GEMM reads them through 3-D maps of k x m_all (n_all) x S, so rows past
  // them and K past k read as zeros whatever the workspace holds there)
  int m_all = 0, n_all = 0;
};
int ozaki_gemm_launch(const OzakiGemmArgs &a, cudaStream_t st, unsigned *err);
// Per-row max |.| of op(A) and per-column max of op(B) and their scale
// exponents: amax and ex hold Mp entries (rows of op(A)) then Np (columns of op(B)).
int row_scale_exponents(char ta, char tb, int m, int n, int k, const double *A, int lda,
                        const double *B, int ldb, unsigned long long *amax, int *ex, int64_t Mp,
                        int64_t Np, cudaStream_t st);
// The same over one operand part: rows [r0, r0 + R) of op(A) (z = 0) or
// columns of op(B) (z = 1), X at the part's first one (kc: k-contiguous);
// writes entries [r0, r0 + Rpart) of that operand's range.
int row_scale_exponents_part(int z, bool kc, int R, int Rpart, int r0, int k, const double *X,
                             int ldx, unsigned long long *amax, int *ex, int64_t Mp, int64_t Np,
                             cudaStream_t st);

// CRT form (crt.cu): C = alpha op(A) op(B) + beta C with the FP64 product
// computed exactly as residues modulo `moduli` (0 = tuned / 16) BF16 GEMMs.
size_t crt_workspace_bytes(int m, int n, int k, int moduli);
int crt_bits_for(int moduli, int k);
// Moduli count for a shape class (autotune cache, falls back to 16).
int crt_default_moduli(int m, int n, int k);
int crt_dgemm(char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
              const double *B, int ldb, double beta, double *C, int ldc, int moduli, void *ws,
              size_t ws_bytes, cudaStream_t st, unsigned *err);
// Two phases: prepare writes the exponents and residue operands, run does the
// per-modulus GEMMs, the reconstruction and the C update.
int crt_prepare(char ta, char tb, int m, int n, int k, const double *A, int lda, const double *B,
                int ldb, int moduli, void *ws, size_t ws_bytes, cudaStream_t st);
int crt_run(int m, int n, int k, double alpha, double beta, double *C, int ldc, int moduli,
            const void *ws, size_t ws_bytes, cudaStream_t st, unsigned *err);
// Parts of the two phases for a pipelined call, in the whole problem's
// workspace (as split_sgemm_prepare_part / split_sgemm_run_block: row parts
// start on multiples of 128, column parts on multiples of 256).
int crt_prepare_part(int z, char t, int m, int n, int k, const double *X, int ldx, int r0,
                     int rows, int moduli, void *ws, size_t ws_bytes, cudaStream_t st);
int crt_run_block(int m, int n, int k, int i0, int h, int j0, int w, double alpha, double beta,
                  double *C, int ldc, int moduli, const void *ws, size_t ws_bytes,
                  cudaStream_t st, unsigned *err);

int ozaki_dgemm(char ta, char tb, int m, int n, int k, double alpha, const double *A, int lda,
                const double *B, int ldb, double beta, double *C, int ldc, int slices, void *ws,
                size_t ws_bytes, cudaStream_t st, unsigned *err);

// Two-phase forms: prepare writes the split operands into the workspace,
// run computes C from a prepared workspace (same m, n, k, products/slices).
int split_sgemm_prepare(char ta, char tb, int m, int n, int k, const float *A, int lda,
                        const float *B, int ldb, int products, void *ws, size_t ws_bytes,
                        cudaStream_t st);
int split_sgemm_run(int m, int n, int k, float alpha, float beta, float *C, int ldc, int products,
                    const void *ws, size_t ws_bytes, cudaStream_t st, unsigned *err,
                    int chunk0 = 0);
// Parts of the same two phases for a pipelined call, in the whole m x n x k
// problem's workspace.  prepare_part: rows [r0, r0 + rows) of op(A) (z = 0,
// X = A, r0 a multiple of 128) or columns of op(B) (z = 1, X = B, r0 a
// multiple of 256).  run_block: C rows [i0, i0 + h) x columns [j0, j0 + w)
// (C = the whole C) from prepared parts covering them.  Same results bit for
// bit as the whole-problem calls.
int split_sgemm_prepare_part(int z, char t, int m, int n, int k, const float *X, int ldx, int r0,
                             int rows, int products, void *ws, size_t ws_bytes, cudaStream_t st);
int split_sgemm_run_block(int m, int n, int k, int i0, int h, int j0, int w, float alpha,
                          float beta, float *C, int ldc, int products, const void *ws,
                          size_t ws_bytes, cudaStream_t st, unsigned *err, int chunk0 = 0);
// Grouped launches of the tensor-core GEMMs: one persistent launch over the
// 128 x 128 tiles of many prepared problems, each problem described by one
// table entry (entry_bytes() bytes, 128-byte aligned) that *_group_entry
// fills on the host from the problem's prepared workspace, with its first
// work unit unit0 (the units of the entries before it; *units returns its
// own); the caller copies the table to device memory and launches.  alpha != 0
// and k > 0 (other problems need no GEMM).  The CRT
// problems' reconstruction runs after the launch (crt_group_reconstruct).
// Results are bit-identical to the per-problem calls.
size_t bf16x_group_entry_bytes();
size_t ozaki_group_entry_bytes();
int bf16x_group_entry(int m, int n, int k, float alpha, float beta, float *C, int ldc,
                      int products, const void *ws, size_t ws_bytes, unsigned *err, int unit0,
                      void *entry, int *units);
int ozaki_group_entry(const OzakiGemmArgs &a, unsigned *err, int unit0, void *entry, int *units);
int crt_group_entry(int m, int n, int k, double alpha, double beta, double *C, int ldc,
                    int moduli, const void *ws, size_t ws_bytes, unsigned *err, int unit0,
                    void *entry, int *units);
int crt_group_reconstruct(int m, int n, int k, double alpha, double beta, double *C, int ldc,
                          int moduli, const void *ws, size_t ws_bytes, cudaStream_t st);
int bf16x_group_launch(const void *table, int nprob, int total_units, cudaStream_t st,
                       unsigned *err);
int ozaki_group_launch(const void *table, int nprob, int total_units, cudaStream_t st,
                       unsigned *err);
int ozaki_prepare(char ta, char tb, int m, int n, int k, const double *A, int lda, const double *B,
                  int ldb, int slices, void *ws, size_t ws_bytes, cudaStream_t st);
int ozaki_run(int m, int n, int k, double alpha, double beta, double *C, int ldc, int slices,
              const void *ws, size_t ws_bytes, cudaStream_t st, unsigned *err);

// Tile width (128 or 256) of the split GEMMs (kind as for the autotuner:
// 0 BF16xP, 1 Ozaki, 2 CRT) for an m x n x k problem: the override, else the
// tuned width of the shape class, else by shape.  The override: 0 = none.
int split_tile_n(int kind, int m, int n, int k);
void set_split_tile_n(int v);
int split_tile_override();
// Cluster mode of the split GEMMs with two or more row tiles: 0 = default,
// 1 = pair MMAs (cta_group::2 on 2-CTA clusters), 2 = one CTA per tile.
void set_pair_mma(int v);
int pair_mma_override();
// Work units of the CRT GEMM: 0 = by shape, 1 = whole tiles, 2 = one modulus
// of one tile (the moduli are independent GEMMs).
void set_modulus_split(int v);
int modulus_split_override();
// Tuned tile width (0 = none) and cluster mode (0 = none, 1 = pair MMAs,
// 2 = one CTA per tile) of a shape class.
int tune_tile_n(int kind, int m, int n, int k);
int tune_pair_mma(int kind, int m, int n, int k);

// Accumulation chunk of the BF16xP GEMM in 64-wide K blocks (0 = default, 4).
int bf16x_chunk_kblocks();
void set_bf16x_chunk_kblocks(int c);

// Default slice count for a shape class (autotune cache, falls back to 8).
int ozaki_default_slices(int m, int n, int k);
// Products / chunk of the BF16xP form for a shape class (cache, else 6 / 0).
void bf16x_resolve(int m, int n, int k, int *products, int *chunk);

// Error word of gb300_sgemm_bf16x_noalloc on the current device (noalloc.cu),
// read (and with `clear` zeroed) without allocating; 0 before its first call.
int noalloc_error_read(int clear, unsigned *out);

// Autotuner (autotune.cu): kind 0 = BF16xP SGEMM, 1 = Ozaki DGEMM.
bool tune_lookup(int kind, int m, int n, int k, int *param, int *chunk);
int autotune(int kind, char ta, char tb, int m, int n, int k, const void *A, int lda,
             const void *B, int ldb, cudaStream_t st, unsigned *err, int *chosen);
int tune_cache_save(const char *path);
int tune_cache_load(const char *path, int *loaded);
void tune_cache_clear();

}  // namespace gb300
