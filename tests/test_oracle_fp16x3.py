"""CPU tests of the scaled 3xFP16 restatement in oracle/split.py (the checker
of the FP16X3 split SGEMM): exact FP16 terms, the representation bound, the
model's error bound and the non-finite convention."""
import numpy as np
import pytest

from oracle import split as osp


def rng_rows(seed, r, k, spread):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, (r, k)) * np.exp2(rng.integers(-spread, spread + 1, (r, k)))
    return (x * np.exp2(rng.integers(-80, 80, (r, 1)))).astype(np.float32)


def test_terms_are_fp16_and_scaled_into_range():
    X = rng_rows(1, 40, 64, 10)
    hi, lo, E = osp.fp16x3_terms(X)
    for t in (hi, lo):
        assert np.array_equal(t.astype(np.float16).astype(np.float32), t)
    assert np.all(np.abs(hi) <= 2.0 ** 15)
    m = np.abs(X.astype(np.float64)).max(axis=1)
    assert np.all((m >= np.ldexp(0.5, E)) & (m < np.ldexp(1.0, E)))


@pytest.mark.parametrize("spread", [0, 8, 40])
def test_representation_bound(spread):
    """|x - 2^(E-15) (hi + lo 2^-11)| <= 2^-22 |x| + 2^-50 max|row| (the FP16
    subnormal quantum of lo, relative to the row's scale)."""
    X = rng_rows(2 + spread, 30, 200, spread)
    hi, lo, E = osp.fp16x3_terms(X)
    rep = np.ldexp(hi.astype(np.float64) + lo.astype(np.float64) / 2048.0, (E - 15)[:, None])
    x = X.astype(np.float64)
    rowmax = np.abs(x).max(axis=1, keepdims=True)
    assert np.all(np.abs(rep - x) <= 2.0 ** -22 * np.abs(x) + 2.0 ** -50 * rowmax)


def test_model_error_bound():
    rng = np.random.default_rng(5)
    A = rng.uniform(-1, 1, (50, 300)).astype(np.float32)
    B = rng.uniform(-1, 1, (300, 40)).astype(np.float32)
    exact = A.astype(np.float64) @ B.astype(np.float64)
    mag = np.abs(A.astype(np.float64)) @ np.abs(B.astype(np.float64))
    err = np.abs(osp.fp16x3_model(A, B) - exact)
    assert np.all(err <= 2.0 ** -20 * mag)
    # about 22 bits per operand: far below FP32 accumulation over k = 300
    assert np.linalg.norm(err) / np.linalg.norm(exact) < 2e-7


def test_operand_layout():
    X = rng_rows(7, 5, 8, 3)
    hi, lo, _ = osp.fp16x3_terms(X)
    a = osp.fp16x3_operand(X, True)
    b = osp.fp16x3_operand(X, False)
    h16, l16 = hi.astype(np.float16).view(np.uint16), lo.astype(np.float16).view(np.uint16)
    assert np.array_equal(a, np.concatenate([h16, l16], axis=1))
    assert np.array_equal(b, np.concatenate([h16, l16], axis=1))


def test_nonfinite_rows_give_nan():
    X = np.ones((3, 4), np.float32)
    X[1, 2] = np.inf
    X[2, 0] = np.nan
    E = osp.row_exponents_f32(X)
    assert E[0] == 1 and E[1] == osp.NONFINITE_EXP and E[2] == osp.NONFINITE_EXP
    a = osp.fp16x3_operand(X, True)
    assert np.all(a[1:] == 0x7E00) and not np.any(a[0] == 0x7E00)
    P = osp.fp16x3_model(X, np.ones((4, 2), np.float32))
    assert np.isnan(P[1:]).all() and np.array_equal(P[0], [4.0, 4.0])
