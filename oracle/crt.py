"""Modular-integer (CRT) FP64 GEMM emulation restated in exact Python integers --
TEST INFRASTRUCTURE.

This restates the published Ozaki scheme II (Ozaki, Uchino & Imamura, "Ozaki
Scheme II: A GEMM-oriented emulation of floating-point matrix multiplication
using an integer modular technique", 2025) in the form the GPU kernels
implement, so that they can be checked bit for bit:

* every row i of op(A) and column j of op(B) is scaled by a power of two and
  truncated to an integer of at most b bits: A'_ik = trunc(a_ik 2^(b - E_i)),
  B'_kj = trunc(b_kj 2^(b - F_j)), with E_i, F_j the frexp exponents of the
  row / column maxima (the same as the slice form's);
* P = A' B' is computed exactly as its residues modulo N pairwise-coprime
  moduli p_1..p_N (odd, at most 255, so that every symmetric residue has
  |r| <= 127 and is exact in BF16): one integer GEMM per modulus;
* b is the largest integer with 2 k (2^b - 1)^2 < M = p_1 ... p_N, so that P
  lies in (-M/2, M/2) and the symmetric Chinese-remainder reconstruction
  recovers it exactly;
* the result is RN(P) scaled by 2^(E_i + F_j - 2b) (one rounding, a second
  only if the scaled value is subnormal), then C = alpha * that + beta * C.

Its only errors are the truncations of A and B to b bits relative to their
row / column maxima; the slice form also drops the products of slices beyond
its order.
"""
from __future__ import annotations

import math

import numpy as np

from .split import row_exponents

# pairwise coprime, odd, at most 255 (255 = 3*5*17, 253 = 11*23, 247 = 13*19,
# 217 = 7*31, the rest prime)
MODULI = (255, 253, 251, 247, 241, 239, 233, 229, 227, 223, 217, 211, 199, 197, 193, 191,
          181, 179, 173, 167, 163, 157, 151, 149)
MAX_MODULI = len(MODULI)


def modulus_product(N: int) -> int:
    M = 1
    for p in MODULI[:N]:
        M *= p
    return M


def crt_bits(N: int, k: int) -> int:
    """Largest b with 2 k (2^b - 1)^2 < M (0 if none)."""
    M = modulus_product(N)
    k = max(int(k), 1)
    b = 0
    while 2 * k * (2 ** (b + 1) - 1) ** 2 < M:
        b += 1
    return b


def crt_weights(N: int):
    """w_i = (M/p_i) * ((M/p_i)^-1 mod p_i) mod M: X = sum r_i w_i = P (mod M)."""
    M = modulus_product(N)
    out = []
    for p in MODULI[:N]:
        Mi = M // p
        out.append((Mi * pow(Mi % p, -1, p)) % M)
    return out


def scaled_integers(X: np.ndarray, b: int):
    """(A', E): A' as a Python-int object array, trunc(x * 2^(b - E_row)) per row."""
    X = np.asarray(X, np.float64)
    E = row_exponents(X)
    out = np.empty(X.shape, dtype=object)
    for r in range(X.shape[0]):
        for c in range(X.shape[1]):
            x = float(X[r, c])
            if x == 0.0 or not math.isfinite(x):
                out[r, c] = 0
                continue
            # exact: x = m * 2^e with integer m (53 bits); trunc toward zero
            mant, ex = math.frexp(abs(x))
            m = int(mant * 2 ** 53)
            t = b - int(E[r]) + ex - 53
            v = m << t if t >= 0 else m >> (-t)
            out[r, c] = -v if x < 0 else v
    return out, E


def symmetric(r: int, p: int) -> int:
    r %= p
    return r - p if r > p // 2 else r


def residues(Ap: np.ndarray, N: int):
    """Per modulus, the symmetric residues of the integer matrix Ap (float64
    arrays holding integers in [-127, 127])."""
    out = []
    for p in MODULI[:N]:
        out.append(np.vectorize(lambda v, p=p: symmetric(int(v), p), otypes=[np.float64])(Ap))
    return out


def crt_gemm_model(A_op: np.ndarray, B_op: np.ndarray, N: int, alpha: float = 1.0,
                   beta: float = 0.0, C: np.ndarray | None = None) -> np.ndarray:
    """The GPU CRT form's result, element for element (exact integer product,
    one correctly rounded conversion, then cb + alpha * v with cb = beta * c)."""
    A_op = np.asarray(A_op, np.float64)
    B_op = np.asarray(B_op, np.float64)
    m, k = A_op.shape
    n = B_op.shape[1]
    b = crt_bits(N, k)
    Ai, E = scaled_integers(A_op, b)
    Bi, F = scaled_integers(B_op.T, b)
    nonfin_a = ~np.isfinite(A_op).all(axis=1) if k else np.zeros(m, bool)
    nonfin_b = ~np.isfinite(B_op).all(axis=0) if k else np.zeros(n, bool)
    P = Ai.dot(Bi.T) if k else np.zeros((m, n), dtype=object)
    out = np.empty((m, n))
    for i in range(m):
        for j in range(n):
            if nonfin_a[i] or nonfin_b[j]:
                v = float("nan")
            else:
                v = math.ldexp(float(int(P[i, j])), int(E[i]) + int(F[j]) - 2 * b)
            c = 0.0 if C is None else float(C[i, j])
            cb = c if beta == 1.0 else c * beta
            out[i, j] = cb + alpha * v
    return out
