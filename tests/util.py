"""Helpers shared by the tests: golden-case decoding and error bounds."""
from __future__ import annotations

import numpy as np

U64 = np.finfo(np.float64).eps / 2
U32 = np.finfo(np.float32).eps / 2


def golden_cases(golden):
    cases, data = golden["cases"], golden["data"]
    for c in cases:
        dt = np.float64 if c["precision"] == "d" else np.float32
        nbytes = int(c["count"]) * np.dtype(dt).itemsize
        raw = data[int(c["offset"]):int(c["offset"]) + nbytes]
        out = raw.view(dt).reshape((int(c["m"]), int(c["n"])), order="F") if nbytes else \
            np.zeros((int(c["m"]), int(c["n"])), dt, order="F")
        yield c, dt, out


def case_inputs(orc, c, dt):
    """Regenerate the inputs of a golden case (portable generator)."""
    ta, tb = str(c["transa"]), str(c["transb"])
    m, n, k = int(c["m"]), int(c["n"]), int(c["k"])
    ar, ac = (m, k) if ta in "Nn" else (k, m)
    br, bc = (k, n) if tb in "Nn" else (n, k)
    seed = int(c["seed"])
    A = orc.storage(ar, ac, int(c["lda"]), dt, seed, 0)
    B = orc.storage(br, bc, int(c["ldb"]), dt, seed, 1)
    C = orc.storage(m, n, int(c["ldc"]), dt, seed, 2)
    return A, B, C


def op(X, trans, rows, cols):
    """op(X) as a float64 (rows x cols) array from column-major storage."""
    if rows == 0 or cols == 0:
        return np.zeros((rows, cols))
    if trans in "Nn":
        return X[:rows, :cols].astype(np.float64)
    return X[:cols, :rows].astype(np.float64).T


def gemm_bound(A, B, C, ta, tb, m, n, k, alpha, beta, u, factor=2.0):
    """Elementwise bound on |computed - exact| for two GEMMs that differ only in
    summation order: factor*(k+2)*u*(|alpha| |op(A)||op(B)| + |beta||C|)."""
    a = np.abs(op(A, ta, m, k))
    b = np.abs(op(B, tb, k, n))
    c = np.abs(C[:m, :n].astype(np.float64))
    return factor * (k + 2) * u * (abs(alpha) * (a @ b) + abs(beta) * c) + 1e-300


def check_close(got, want, bound):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    both_nan = np.isnan(got) & np.isnan(want)
    same = (got == want) | both_nan
    diff = np.where(same, 0.0, np.abs(got - want))
    bad = diff > bound
    assert not bad.any(), "max excess %g at %s (got %r want %r bound %r)" % (
        float((diff - bound).max()), np.argwhere(bad)[0], got[bad][0], want[bad][0],
        bound[bad][0] if np.ndim(bound) else bound)


# ---------------------------------------------------------------- complex
def ctrans(t) -> bool:
    """Complex trans codes: 'N'/'R' keep the shape, anything else transposes."""
    return t not in "NnRr"


def cop(X, trans, rows, cols):
    """op(X) as a complex128 (rows x cols) array: 'N' X, 'R' conj(X), 'T' X^T,
    'C' conj(X)^T."""
    if rows == 0 or cols == 0:
        return np.zeros((rows, cols), np.complex128)
    Y = X[:cols, :rows].T if ctrans(trans) else X[:rows, :cols]
    Y = Y.astype(np.complex128)
    return np.conj(Y) if trans in "CcRr" else Y


def l1(z):
    """|re| + |im| elementwise (bounds both parts of a complex product sum)."""
    z = np.asarray(z)
    return np.abs(z.real) + np.abs(z.imag)


def cgemm_bound(Aop, Bop, C, alpha, beta, k, u, factor=1.0):
    """Elementwise bound on |got - exact| for alpha*Aop@Bop + beta*C computed in
    unit roundoff u: each part is a dot of 2k products plus the alpha/beta
    update, so (2k + 8) u (|alpha| |A||B| + |beta| |C|) with l1 moduli."""
    mag = l1(complex(alpha)) * (l1(Aop) @ l1(Bop))
    if C is not None:
        mag = mag + l1(complex(beta)) * l1(C)
    return factor * (2 * k + 8) * u * mag + np.finfo(np.float64).tiny


def check_close_c(got, want, bound):
    """Real and imaginary parts of got within `bound` of want, elementwise."""
    dr = np.abs(np.asarray(got, np.complex128).real - want.real)
    di = np.abs(np.asarray(got, np.complex128).imag - want.imag)
    bad = (dr > bound) | (di > bound)
    assert not bad.any(), (int(bad.sum()), float(np.max(dr - bound)), float(np.max(di - bound)))
