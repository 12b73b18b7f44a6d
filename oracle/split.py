"""numpy restatements of the split-precision decompositions -- TEST INFRASTRUCTURE.

These have no counterpart in the reference (the split forms are tensor-core
forms of its sgemm_/dgemm_, src/gemm_driver.c:118); they restate the published
methods so that the GPU split kernels can be checked bit for bit:

* bf16_terms: x = t0 + t1 + t2 + r with t_i = RNE-to-BF16 of the running
  residual (Henry, Tang & Heinecke, "Leveraging the bfloat16 AI datatype for
  higher-precision computations", ARITH 2019).
* ozaki_slices: row scaling by 2^-E (E from frexp of the row max) and
  truncated 7-bit integer digits, x*2^-E = sum_s d_s 2^-7s + r, |d_s| <= 127
  (error-free splitting of Ozaki, Ogita, Oishi & Rump 2012, with the integer
  slices of Mukunoki, Ozaki, Ogita & Imamura, ISC 2020).
* ozaki_gemm_model: the exact-integer product/recombination model of the GPU
  kernel (slice products grouped by t = i + j, weight 2^-7t, FP64 folding from
  the largest t down).
* fp16x3_terms / fp16x3_model: the scaled 3xFP16 SGEMM form -- FP16 hi and
  2^11-scaled lo terms with the lo*lo product dropped (Ootomo & Yokota,
  "Recovering single precision accuracy from Tensor Cores while surpassing the
  FP32 theoretical peak performance", IJHPCA 2022), applied to rows / columns
  scaled by powers of two into the FP16 range (the row scaling of the Ozaki
  scheme above).
"""
from __future__ import annotations

import numpy as np


def bf16_round(x: np.ndarray) -> np.ndarray:
    """Round float32 to the nearest bfloat16 (ties to even), returned as float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    lsb = (b >> 16) & 1
    r = ((b + 0x7FFF + lsb) & 0xFFFF0000).astype(np.uint32)
    out = r.view(np.float32).copy()
    nan = np.isnan(x)
    out[nan] = x[nan]
    return out


def bf16_terms(x: np.ndarray, nterms: int):
    """[t0, t1, t2] (float32 arrays holding BF16 values); unused terms are 0."""
    r = np.asarray(x, dtype=np.float32)
    terms = []
    for i in range(3):
        if i < nterms:
            t = bf16_round(r)
            r = (r - t).astype(np.float32)
        else:
            t = np.zeros_like(r)
        terms.append(t)
    return terms


# The GEMM's product stream: segment s multiplies term SEGMENTS[P][0][s] of A'
# with term SEGMENTS[P][1][s] of B' (smallest products first).
SEGMENTS = {
    3: ([1, 0, 0], [0, 1, 0]),
    6: ([2, 1, 0, 1, 0, 0], [0, 1, 2, 0, 1, 0]),
}


def bf16x_operand(X: np.ndarray, products: int, is_a: bool) -> np.ndarray:
    """The K-major split operand of an R x K op(X) view (R x T*K, float32
    holding BF16): its T terms once each, [hi | lo] for P = 3 and
    [hi | mid | lo] for P = 6, the same for A and B (is_a: kept for the
    callers; the GEMM pairs the terms by SEGMENTS)."""
    nterms = 2 if products == 3 else 3
    terms = bf16_terms(np.asarray(X, np.float32), nterms)
    return np.concatenate(terms[:nterms], axis=1)


def row_exponents(X: np.ndarray) -> np.ndarray:
    """E_r with max_k |X[r,k]| * 2^-E_r < 1 (frexp exponent of the row max; 0 for zero rows)."""
    m = np.abs(np.asarray(X, np.float64)).max(axis=1) if X.shape[1] else np.zeros(X.shape[0])
    e = np.frexp(m)[1].astype(np.int64)
    e[m == 0] = 0
    return e


def ozaki_slices(X: np.ndarray, S: int):
    """(slices, E): slices[s] is an R x K float64 array of integers in [-127, 127]."""
    X = np.asarray(X, np.float64)
    E = row_exponents(X)
    x = np.ldexp(X, -E[:, None])
    out = []
    for _ in range(S):
        y = x * 128.0
        d = np.trunc(y)
        x = y - d
        out.append(d)
    return out, E


def ozaki_gemm_model(A_op: np.ndarray, B_op: np.ndarray, S: int) -> np.ndarray:
    """op(A) @ op(B) as computed by the Ozaki kernel: exact integer group sums,
    weight 2^-7t, FP64 folding from t = S+1 down to 2, then 2^(E_i + F_j)."""
    As, E = ozaki_slices(A_op, S)
    Bs, F = ozaki_slices(B_op.T, S)
    res = np.zeros((A_op.shape[0], B_op.shape[1]))
    for t in range(S + 1, 1, -1):
        P = np.zeros_like(res, dtype=object) if False else np.zeros(res.shape, dtype=np.int64)
        for sa in range(max(1, t - S), min(S, t - 1) + 1):
            sb = t - sa
            P += (As[sa - 1].astype(np.int64) @ Bs[sb - 1].astype(np.int64).T)
        res = P.astype(np.float64) * 2.0 ** (-7 * t) + res
    return np.ldexp(res, (E[:, None] + F[None, :]).astype(np.int64))


NONFINITE_EXP = 0x40000000  # scale exponent marker of a row holding Inf or NaN


def row_exponents_f32(X: np.ndarray) -> np.ndarray:
    """E_r of each FP32 row (frexp exponent of max |x|, 0 for zero rows,
    NONFINITE_EXP for rows holding Inf or NaN)."""
    X = np.asarray(X, np.float32)
    with np.errstate(invalid="ignore"):
        bad = ~np.isfinite(X).all(axis=1) if X.shape[1] else np.zeros(X.shape[0], bool)
        m = np.abs(np.where(np.isfinite(X), X, 0)).astype(np.float64).max(axis=1) \
            if X.shape[1] else np.zeros(X.shape[0])
    e = np.frexp(m)[1].astype(np.int64)
    e[m == 0] = 0
    e[bad] = NONFINITE_EXP
    return e


def fp16x3_terms(X: np.ndarray):
    """(hi, lo, E) of an R x K FP32 op(X) view: y = x 2^(15 - E_r) in
    (-2^15, 2^15) rounded once to FP32, hi = fp16(y), lo = fp16((y - hi) 2^11)
    (float32 arrays holding FP16 values); rows with E = NONFINITE_EXP are NaN."""
    X = np.asarray(X, np.float32)
    E = row_exponents_f32(X)
    ok = E != NONFINITE_EXP
    s = np.where(ok, 15 - E, 0)
    y = np.ldexp(X.astype(np.float64), s[:, None]).astype(np.float32)
    with np.errstate(over="ignore", invalid="ignore"):
        hi = y.astype(np.float16).astype(np.float32)
        lo = ((y - hi) * np.float32(2048)).astype(np.float16).astype(np.float32)
    hi[~ok] = np.nan
    lo[~ok] = np.nan
    return hi, lo, E


def fp16x3_operand(X: np.ndarray, is_a: bool) -> np.ndarray:
    """The K-major split operand (R x 2K, FP16 bit patterns as uint16):
    [hi | lo] for A and B alike (the GEMM's segments pair them as lo*hi,
    hi*lo, hi*hi by SEGMENTS[3])."""
    hi, lo, _ = fp16x3_terms(X)
    t = np.concatenate([hi, lo], axis=1)
    out = t.astype(np.float16).view(np.uint16).copy()
    out[np.isnan(t)] = 0x7E00
    return out


def fp16x3_model(A_op: np.ndarray, B_op: np.ndarray) -> np.ndarray:
    """op(A) @ op(B) in FP64 from the represented operands: 2^(E_i + F_j - 30)
    (hiA hiB + (hiA loB + loA hiB) 2^-11).  The GPU differs from it only by the
    FP32 accumulation."""
    ha, la, E = fp16x3_terms(A_op)
    hb, lb, F = fp16x3_terms(np.asarray(B_op).T)
    ha, la, hb, lb = (np.asarray(v, np.float64) for v in (ha, la, hb, lb))
    with np.errstate(invalid="ignore", over="ignore"):
        P = ha @ hb.T + (ha @ lb.T + la @ hb.T) / 2048.0
    e = np.minimum(E, 1024)[:, None] + np.minimum(F, 1024)[None, :] - 30
    with np.errstate(invalid="ignore", over="ignore"):
        return np.ldexp(P, e)
