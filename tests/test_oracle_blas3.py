"""The TRSM / TRMM checker (oracle/blas3.py) pinned to the reference's own
kernels: every side/uplo/trans/diag variant of both routines in both
precisions, through oracle/ref_blas3.c where the kernels are compiled here
(x86-64 with the reference sources), and through the committed fixtures
(tests/golden/blas3.npz, written by tests/golden/make_golden_blas3.py from the
same kernels) everywhere."""
import hashlib
import itertools
import os

import numpy as np
import pytest

import oracle
from oracle import blas3

HERE = os.path.dirname(os.path.abspath(__file__))
TOL = {"d": 1e-14, "s": 1e-6}  # relative Frobenius, rounding of the two orders
VARIANTS = list(itertools.product("LR", "UL", "NT", "NU"))


def rel(got, ref):
    return np.linalg.norm(got.astype(np.float64) - ref) / max(np.linalg.norm(ref), 1e-300)


def fixtures():
    z = np.load(os.path.join(HERE, "golden", "blas3.npz"))
    return z["cases"], {"d": z["data_d"], "s": z["data_s"]}, z["inputs"]


def case_inputs(c):
    dt = np.float64 if c["precision"] == "d" else np.float32
    m, n = int(c["m"]), int(c["n"])
    na = m if c["side"] == "L" else n
    return blas3.generator_inputs(na, na + 3, m, m + 2, n, dt, int(c["seed"]))


@pytest.mark.skipif(not oracle.RefBlas3.available(), reason="reference kernels not built here")
@pytest.mark.parametrize("prec", ["d", "s"])
@pytest.mark.parametrize("routine", ["trsm", "trmm"])
def test_reference_kernels_match_oracle(routine, prec):
    R = oracle.RefBlas3()
    dt = np.float64 if prec == "d" else np.float32
    for (side, uplo, ta, diag), (m, n) in itertools.product(
            VARIANTS, [(1, 1), (8, 4), (37, 23), (13, 70), (66, 20), (5, 131)]):
        rng = np.random.default_rng(m * 1000 + n)
        na = m if side == "L" else n
        A = blas3.well_conditioned_triangle(rng, na, na + 3, dt)
        B = np.asfortranarray(rng.uniform(-1, 1, (m + 2, n)).astype(dt))
        got = R.call(routine, side, uplo, ta, diag, m, n, -0.75, A, B)
        ref = getattr(blas3, routine)(side, uplo, ta, diag, m, n, -0.75, A, B)
        assert np.array_equal(got[m:], B[m:])
        d = rel(got[:m], ref)
        assert d < TOL[prec], (side, uplo, ta, diag, m, n, d)


def test_fixtures_cover_every_variant():
    cases, _, _ = fixtures()
    got = {(str(c["routine"]), str(c["precision"]), str(c["side"]), str(c["uplo"]),
            str(c["transa"]), str(c["diag"])) for c in cases}
    want = {(r, p) + v for r in ("trsm", "trmm") for p in "ds" for v in VARIANTS}
    assert got == want


def test_fixtures_match_oracle():
    cases, data, digests = fixtures()
    for c, dg in zip(cases, digests):
        A, B = case_inputs(c)
        assert hashlib.sha256(A.tobytes(order="F") + B.tobytes(order="F")).hexdigest() == dg
        m, n = int(c["m"]), int(c["n"])
        ref = getattr(blas3, str(c["routine"]))(str(c["side"]), str(c["uplo"]), str(c["transa"]),
                                                str(c["diag"]), m, n, float(c["alpha"]), A, B)
        fx = data[str(c["precision"])][c["offset"]:c["offset"] + c["count"]].reshape(
            (m, n), order="F")
        assert rel(fx, ref) < TOL[str(c["precision"])], tuple(c)


@pytest.mark.skipif(not oracle.RefBlas3.available(), reason="reference kernels not built here")
def test_fixtures_are_the_kernels_output():
    R = oracle.RefBlas3()
    cases, data, _ = fixtures()
    for c in cases:
        A, B = case_inputs(c)
        m, n = int(c["m"]), int(c["n"])
        got = R.call(str(c["routine"]), str(c["side"]), str(c["uplo"]), str(c["transa"]),
                     str(c["diag"]), m, n, float(c["alpha"]), A, B)[:m]
        fx = data[str(c["precision"])][c["offset"]:c["offset"] + c["count"]]
        assert np.array_equal(got.ravel(order="F"), fx), tuple(c)
