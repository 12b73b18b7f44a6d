"""Generate the TRSM / TRMM golden fixtures from the reference's own kernels.

Run where the reference sources are compiled into ``oracle/_ref/libblas3.so``
(``oracle/build.sh <reference-dir>``; x86-64 only):

    python tests/golden/make_golden_blas3.py

Each case draws A and B from the portable generator (``oracle.blas3.generator_inputs``),
runs the reference's TRSM kernels (TRSM_KERNEL_*_simplified.c over
dgemm_kernel_4x4_haswell.c in FP64, strsm_kernel_8x4_haswell_*.c in FP32) or its
TRMM kernel (trmm_kernel_4x8_simplified.c) through ``oracle/ref_blas3.c``, and
stores the m x n result.  The triangle's order na = 66 crosses one 64-wide
diagonal block of the GPU routines.

Output: tests/golden/blas3.npz
  cases   structured array: routine, precision, side, uplo, transa, diag, m, n,
          alpha, seed, offset, count
  data_d  concatenated FP64 results (column-major, ld = m)
  data_s  concatenated FP32 results
  inputs  sha256 of the generated (A, B) bytes of every case, in case order
"""
from __future__ import annotations

import hashlib
import itertools
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402
from oracle import blas3  # noqa: E402

CASE_DT = np.dtype([("routine", "U4"), ("precision", "U1"), ("side", "U1"), ("uplo", "U1"),
                    ("transa", "U1"), ("diag", "U1"), ("m", "i4"), ("n", "i4"), ("alpha", "f8"),
                    ("seed", "i4"), ("offset", "i8"), ("count", "i8")])


def case_list():
    out = []
    seed = 100
    for routine in ("trsm", "trmm"):
        for prec in ("d", "s"):
            for side, uplo, ta, diag in itertools.product("LR", "UL", "NT", "NU"):
                m, n = (66, 20) if side == "L" else (20, 66)
                alpha = -0.75 if routine == "trsm" else 1.25
                out.append((routine, prec, side, uplo, ta, diag, m, n, alpha, seed))
                seed += 1
    return out


def inputs(case):
    routine, prec, side, uplo, ta, diag, m, n, alpha, seed = case[:10]
    dt = np.float64 if prec == "d" else np.float32
    na = m if side == "L" else n
    return blas3.generator_inputs(na, na + 3, m, m + 2, n, dt, seed)


def main():
    R = oracle.RefBlas3()
    rows, data = [], {"d": [], "s": []}
    off = {"d": 0, "s": 0}
    digests = []
    for case in case_list():
        routine, prec, side, uplo, ta, diag, m, n, alpha, seed = case
        A, B = inputs(case)
        digests.append(hashlib.sha256(A.tobytes(order="F") + B.tobytes(order="F")).hexdigest())
        got = R.call(routine, side, uplo, ta, diag, m, n, alpha, A, B)[:m]
        flat = np.asfortranarray(got).ravel(order="F")
        rows.append(case + (off[prec], flat.size))
        data[prec].append(flat)
        off[prec] += flat.size
    np.savez(os.path.join(HERE, "blas3.npz"), cases=np.array(rows, dtype=CASE_DT),
             data_d=np.concatenate(data["d"]).astype(np.float64),
             data_s=np.concatenate(data["s"]).astype(np.float32),
             inputs=np.array(digests))
    print("wrote %d cases" % len(rows))


if __name__ == "__main__":
    main()
