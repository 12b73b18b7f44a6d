"""numpy restatements of the BLAS TRSM / TRMM definitions -- TEST INFRASTRUCTURE.

The reference has TRSM/TRMM only as OpenBLAS-style packed-panel kernels outside
its built library (OpenBLAS-like_implementation/TRSM_KERNEL_*_simplified.c,
strsm_kernel_8x4_haswell_*.c, trmm_kernel_4x8_simplified.c).  These follow the
BLAS definitions directly, in FP64; they are pinned to those kernels, compiled
from their sources and driven on packed panels by oracle/ref_blas3.c
(tests/test_oracle_blas3.py: every side/uplo/trans/diag variant agrees to
rounding), and the fixtures in tests/golden/blas3.npz hold the kernels' own
outputs on inputs from ``generator_inputs``.

  trsm: side 'L': solve op(A) X = alpha B;  'R': X op(A) = alpha B
  trmm: side 'L': alpha op(A) B;            'R': alpha B op(A)
"""
from __future__ import annotations

import numpy as np


def op_triangle(A: np.ndarray, na: int, uplo: str, transa: str, diag: str) -> np.ndarray:
    """op(A) as a dense FP64 na x na matrix holding only the referenced triangle."""
    T = np.array(A[:na, :na], dtype=np.float64)
    T = np.tril(T) if uplo in "Ll" else np.triu(T)
    if diag in "Uu":
        np.fill_diagonal(T, 1.0)
    return T if transa in "Nn" else T.T


def trsm(side, uplo, transa, diag, m, n, alpha, A, B):
    na = m if side in "Ll" else n
    T = op_triangle(A, na, uplo, transa, diag)
    Bm = np.array(B[:m, :n], dtype=np.float64)
    if alpha == 0:
        return np.zeros((m, n))
    if side in "Ll":
        return np.linalg.solve(T, alpha * Bm)
    return np.linalg.solve(T.T, alpha * Bm.T).T


def trmm(side, uplo, transa, diag, m, n, alpha, A, B):
    na = m if side in "Ll" else n
    T = op_triangle(A, na, uplo, transa, diag)
    Bm = np.array(B[:m, :n], dtype=np.float64)
    if alpha == 0:
        return np.zeros((m, n))
    return alpha * (T @ Bm) if side in "Ll" else alpha * (Bm @ T)


def well_conditioned_triangle(rng, na, lda, dtype):
    """A na x na (ld = lda) matrix whose both triangles are well conditioned:
    diagonal in [1, 2), off-diagonal entries U[-1,1)/na."""
    A = (rng.uniform(-1, 1, (lda, na)) / max(na, 1)).astype(dtype)
    for i in range(na):
        A[i, i] = dtype(1.0 + rng.uniform())
    return np.asfortranarray(A)


def generator_inputs(na, lda, m, ldb, n, dtype, seed):
    """Inputs from the portable counter-based generator (bit-identical on x86-64
    and aarch64): a well-conditioned triangle source A (lda x na; diagonal in
    [1, 2), off-diagonal U[-1,1)/na) and B (ldb x n, U[-1,1))."""
    import oracle

    A = oracle.uniform((lda, na), np.float64, seed, 0) / max(na, 1)
    d = oracle.uniform((na,), np.float64, seed, 1)
    for i in range(na):
        A[i, i] = 1.5 + 0.5 * d[i]
    B = oracle.uniform((ldb, n), np.float64, seed, 2)
    return np.asfortranarray(A.astype(dtype)), np.asfortranarray(B.astype(dtype))

