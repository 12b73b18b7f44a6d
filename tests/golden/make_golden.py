"""Generate the golden fixtures of the sgemm_/dgemm_ path from the reference itself.

Run in a checkout where the reference sources are available and compiled into
``oracle/_ref/`` (``oracle/build.sh <reference-dir>``; x86-64 only):

    python tests/golden/make_golden.py

Every case draws its inputs from the portable counter-based generator
(``oracle.uniform``; bit-identical on x86-64 and aarch64), runs the reference
library's own ``dgemm_``/``sgemm_`` with a fixed OpenMP team size, and stores
the raw output bits.  The inputs are not stored: the tests regenerate them from
(seed, stream, shape) and check the generator against pinned draws.

Output: tests/golden/golden.npz
  cases        structured array: precision, transa, transb, m, n, k, lda, ldb,
               ldc, alpha, beta, seed, threads, offset, count
  data         concatenated raw output bytes (column-major m x n, ld = m);
               case bytes [offset, offset + count*itemsize)
  cfg1_*       config-1 (DGEMM NN 2048^3, alpha 1, beta 0.5, seed 0) sampled
               entries of the reference output + sha256 of the full output
  draws        pinned generator draws (seed 0..2, stream 0..2, idx 0..7)
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402

THREADS = 2  # a team of 2 still exercises the rotated full-block path at n >= 2*(BDN+1)


def stored_shape(trans, rows_op, cols_op):
    return (rows_op, cols_op) if trans in "Nn" else (cols_op, rows_op)


def case_inputs(prec, ta, tb, m, n, k, lda, ldb, ldc, seed, phi=None):
    dt = np.float64 if prec == "d" else np.float32
    ar, ac = stored_shape(ta, m, k)
    br, bc = stored_shape(tb, k, n)
    A = oracle.storage(ar, ac, lda, dt, seed, 0)
    B = oracle.storage(br, bc, ldb, dt, seed, 1)
    C = oracle.storage(m, n, ldc, dt, seed, 2)
    return A, B, C


def case_list():
    cases = []
    # (17, 386, 700): each of the 2 threads owns > BDN columns and K spans a
    # K-edge block plus full K blocks, so the skewed full-block order is used.
    shapes = [(1, 1, 1), (3, 2, 1), (7, 5, 3), (17, 9, 33), (33, 97, 300), (0, 5, 5),
              (5, 0, 5), (5, 5, 0), (130, 7, 1), (31, 50, 64), (17, 386, 700)]
    ab = [(1.0, 0.5), (-1.5, 1.0), (0.0, 3.0), (2.0, 0.0), (0.75, -2.0)]
    i = 0
    for prec in "ds":
        for ta in "NT":
            for tb in "NT":
                for (m, n, k) in shapes:
                    alpha, beta = ab[i % len(ab)]
                    i += 1
                    ar = m if ta == "N" else k
                    br = k if tb == "N" else n
                    pad = (i % 3) + (1 if prec == "s" else 0)
                    lda, ldb, ldc = max(ar, 1) + pad, max(br, 1) + (i % 2), max(m, 1) + (i % 4)
                    cases.append((prec, ta, tb, m, n, k, lda, ldb, ldc, alpha, beta, 100 + i))
    # transpose characters other than N/T (any non-N char means transpose)
    cases.append(("d", "n", "c", 20, 30, 40, 20, 30, 21, 1.0, 1.0, 500))
    cases.append(("s", "t", "x", 20, 30, 40, 40, 30, 20, -1.0, 0.0, 501))
    return cases


def main():
    if not oracle.RefLib.available():
        raise SystemExit("reference library not built: oracle/build.sh <reference-dir>")
    ref = oracle.RefLib()
    oracle.set_threads(THREADS)
    recs, chunks, off = [], [], 0
    for (prec, ta, tb, m, n, k, lda, ldb, ldc, alpha, beta, seed) in case_list():
        A, B, C = case_inputs(prec, ta, tb, m, n, k, lda, ldb, ldc, seed)
        ref.gemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc)
        out = np.asfortranarray(C[:m, :n]) if m > 0 and n > 0 else np.zeros((0, 0), C.dtype)
        bits = out.ravel(order="F").view(np.uint64 if prec == "d" else np.uint32)
        chunks.append(bits.view(np.uint8))
        recs.append((prec, ta, tb, m, n, k, lda, ldb, ldc, alpha, beta, seed, THREADS, off,
                     bits.size))
        off += bits.size * bits.itemsize
    cases = np.array(recs, dtype=[("precision", "U1"), ("transa", "U1"), ("transb", "U1"),
                                  ("m", "i4"), ("n", "i4"), ("k", "i4"), ("lda", "i4"),
                                  ("ldb", "i4"), ("ldc", "i4"), ("alpha", "f8"), ("beta", "f8"),
                                  ("seed", "i8"), ("threads", "i4"), ("offset", "i8"),
                                  ("count", "i8")])
    data = np.concatenate(chunks) if chunks else np.zeros(0, np.uint8)

    # config 1: DGEMM NN 2048^3, alpha 1, beta 0.5, seed 0, reference team of 8
    oracle.set_threads(8)
    N = 2048
    A = oracle.uniform((N, N), np.float64, 0, 0)
    B = oracle.uniform((N, N), np.float64, 0, 1)
    C = oracle.uniform((N, N), np.float64, 0, 2)
    ref.gemm("N", "N", N, N, N, 1.0, A, N, B, N, 0.5, C, N)
    rng = np.random.default_rng(1234)
    rows = rng.integers(0, N, 4096)
    cols = rng.integers(0, N, 4096)
    cfg1_vals = C[rows, cols].copy()
    cfg1_sha = hashlib.sha256(np.asfortranarray(C).tobytes(order="F")).hexdigest()

    draws = np.array([[[oracle.lib().orc_draw(s, st, i) for i in range(8)] for st in range(3)]
                      for s in range(3)], dtype=np.uint64)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), cases=cases, data=data,
                        cfg1_rows=rows, cfg1_cols=cols, cfg1_vals=cfg1_vals,
                        cfg1_sha256=np.array(cfg1_sha), cfg1_threads=np.array(8), draws=draws)
    print("wrote %d cases, %d output bytes, cfg1 sha256 %s" % (len(cases), data.size, cfg1_sha))


if __name__ == "__main__":
    main()
