"""Blocked TRSM / TRMM on the GPU (BLAS semantics) against the FP64
restatement of the definitions (oracle/blas3.py), all 16 side/uplo/trans/diag
variants, both precisions, ragged sizes across the 64-wide blocks, padded ld,
plain and split-form GEMM updates; and against the reference kernels' own
outputs (tests/golden/blas3.npz)."""
import itertools
import os

import numpy as np
import pytest

import gemm_avx2_gb300 as g
from gpu_util import from_dev, sync, to_dev
from oracle import blas3

pytestmark = pytest.mark.gpu

VARIANTS = list(itertools.product("LR", "UL", "NT", "NU"))


def run(routine, prec, side, uplo, ta, diag, m, n, alpha, form, seed):
    dt = np.float64 if prec == "d" else np.float32
    rng = np.random.default_rng(seed)
    na = m if side == "L" else n
    A = blas3.well_conditioned_triangle(rng, na, na + 3, dt)
    B = np.asfortranarray(rng.uniform(-1, 1, (m + 2, n)).astype(dt))
    dA, dB = to_dev(A), to_dev(B)
    f = g.trsm if routine == "trsm" else g.trmm
    assert f(prec, side, uplo, ta, diag, m, n, alpha, dA.data_ptr(), na + 3, dB.data_ptr(), m + 2,
             form=form) == g.OK
    sync()
    got = from_dev(dB, m + 2)
    ref = getattr(blas3, routine)(side, uplo, ta, diag, m, n, alpha, A, B)
    d = np.linalg.norm(got[:m].astype(np.float64) - ref) / max(np.linalg.norm(ref), 1e-300)
    assert np.array_equal(got[m:], B[m:])          # ldb padding untouched
    return d


@pytest.mark.parametrize("side,uplo,ta,diag", VARIANTS)
@pytest.mark.parametrize("routine", ["trsm", "trmm"])
def test_all_variants_fp64(routine, side, uplo, ta, diag):
    d = run(routine, "d", side, uplo, ta, diag, 150, 131, -0.75, 0, 7)
    assert d < 1e-13, d


@pytest.mark.parametrize("side,uplo,ta,diag", VARIANTS[::3])
@pytest.mark.parametrize("routine", ["trsm", "trmm"])
def test_variants_fp32(routine, side, uplo, ta, diag):
    d = run(routine, "s", side, uplo, ta, diag, 140, 99, 1.5, 0, 8)
    assert d < 2e-6, d


@pytest.mark.parametrize("prec", ["d", "s"])
@pytest.mark.parametrize("routine", ["trsm", "trmm"])
def test_split_form_updates(routine, prec):
    d = run(routine, prec, "L", "L", "N", "N", 300, 200, 1.0, 1, 9)
    assert d < (1e-13 if prec == "d" else 2e-6), d
    d = run(routine, prec, "R", "U", "T", "U", 170, 260, 0.5, 1, 10)
    assert d < (1e-13 if prec == "d" else 2e-6), d


@pytest.mark.parametrize("side,uplo,ta,diag", [("L", "L", "N", "N"), ("R", "U", "T", "U"),
                                               ("L", "U", "T", "N"), ("R", "L", "N", "U")])
@pytest.mark.parametrize("routine", ["trsm", "trmm"])
def test_crt_form_updates_fp64(routine, side, uplo, ta, diag):
    """form 2: FP64 off-diagonal updates on the CRT form (exact products of the
    row / column scaled operands), ragged sizes over the 64-wide blocks and a
    padded ldb that stays untouched; FP32 takes 6xBF16 as form 1."""
    d = run(routine, "d", side, uplo, ta, diag, 300, 200, -0.75, 2, 11)
    assert d < 1e-13, d
    d = run(routine, "s", side, uplo, ta, diag, 170, 260, 0.5, 2, 12)
    assert d < 2e-6, d


def test_alpha_zero_and_args():
    B = np.full((8, 5), np.nan, order="F")
    A = np.eye(8, order="F")
    dA, dB = to_dev(A), to_dev(B)
    assert g.trsm("d", "L", "U", "N", "N", 8, 5, 0.0, dA.data_ptr(), 8, dB.data_ptr(), 8) == g.OK
    sync()
    assert np.all(from_dev(dB, 8) == 0.0)          # BLAS: alpha == 0 sets B to zero
    assert g.trsm("d", "X", "U", "N", "N", 8, 5, 1.0, dA.data_ptr(), 8, dB.data_ptr(), 8) == \
        g.ERR_ARG
    assert g.trsm("d", "L", "U", "N", "N", 8, 5, 1.0, dA.data_ptr(), 7, dB.data_ptr(), 8) == \
        g.ERR_ARG
    assert g.trsm("d", "L", "U", "N", "N", 8, 5, 1.0, dA.data_ptr(), 8, dB.data_ptr(), 8,
                  form=3) == g.ERR_ARG


def test_golden_fixtures_from_reference_kernels():
    """Every variant of both routines in both precisions against the outputs of
    the reference's TRSM / TRMM kernels on the same generated inputs (triangle
    order 66: one full 64-wide diagonal block and a ragged one)."""
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "blas3.npz"))
    data = {"d": z["data_d"], "s": z["data_s"]}
    for c in z["cases"]:
        prec, side = str(c["precision"]), str(c["side"])
        dt = np.float64 if prec == "d" else np.float32
        m, n = int(c["m"]), int(c["n"])
        na = m if side == "L" else n
        A, B = blas3.generator_inputs(na, na + 3, m, m + 2, n, dt, int(c["seed"]))
        dA, dB = to_dev(A), to_dev(B)
        f = g.trsm if str(c["routine"]) == "trsm" else g.trmm
        assert f(prec, side, str(c["uplo"]), str(c["transa"]), str(c["diag"]), m, n,
                 float(c["alpha"]), dA.data_ptr(), na + 3, dB.data_ptr(), m + 2) == g.OK
        sync()
        got = from_dev(dB, m + 2)
        assert np.array_equal(got[m:], B[m:])
        ref = data[prec][c["offset"]:c["offset"] + c["count"]].reshape((m, n), order="F")
        d = np.linalg.norm(got[:m].astype(np.float64) - ref) / np.linalg.norm(ref.astype(np.float64))
        assert d < (1e-13 if prec == "d" else 2e-6), (tuple(c), d)

