"""CPU tests of the CRT (modular-integer) FP64 GEMM model in oracle/crt.py:
the moduli and reconstruction constants, the bit count, and the model's
accuracy against the Dot2 ground truth."""
import math

import numpy as np
import pytest

import gemm_avx2_gb300 as g
import oracle
from oracle import crt
from oracle import split as osp


def test_moduli_pairwise_coprime_and_bounded():
    ps = crt.MODULI
    assert len(ps) == crt.MAX_MODULI == 24
    assert all(p % 2 == 1 and p <= 255 for p in ps)
    for i in range(len(ps)):
        for j in range(i + 1, len(ps)):
            assert math.gcd(ps[i], ps[j]) == 1


@pytest.mark.parametrize("N", [2, 8, 16, 24])
def test_weights_are_crt_idempotents(N):
    M = crt.modulus_product(N)
    for i, w in enumerate(crt.crt_weights(N)):
        assert 0 <= w < M
        for j, p in enumerate(crt.MODULI[:N]):
            assert w % p == (1 if i == j else 0)


@pytest.mark.parametrize("N,k", [(16, 4096), (16, 16384), (22, 16384), (8, 100), (2, 4096)])
def test_bits_bound_is_tight(N, k):
    M = crt.modulus_product(N)
    b = crt.crt_bits(N, k)
    assert 2 * k * (2 ** b - 1) ** 2 < M <= 2 * k * (2 ** (b + 1) - 1) ** 2
    if (N, k) == (16, 4096):
        assert b == 55


def test_model_exact_on_small_integers():
    rng = np.random.default_rng(1)
    A = rng.integers(-50, 50, (7, 30)).astype(np.float64)
    B = rng.integers(-50, 50, (30, 5)).astype(np.float64)
    assert np.array_equal(crt.crt_gemm_model(A, B, 6), A @ B)


@pytest.mark.parametrize("N", [10, 16, 20])
def test_model_error_within_truncation_bound(N):
    """Only the truncations to b bits err: |err_ij| <= k 2^(E_i + F_j - b + 1)."""
    m, n, k = 9, 7, 300
    A = oracle.spread((m, k), 41, 0, 1.5)
    B = oracle.spread((k, n), 41, 1, 1.5)
    got = crt.crt_gemm_model(A, B, N)
    truth = oracle.dot2gemm("N", "N", m, n, k, 1.0, A, m, B, k, 0.0,
                            np.zeros((m, n), order="F"), m)
    b = crt.crt_bits(N, k)
    E = osp.row_exponents(A)
    F = osp.row_exponents(B.T)
    bound = k * np.ldexp(1.0, (E[:, None] + F[None, :] - b + 1).astype(np.int64))
    assert (np.abs(got - truth) <= bound + 1e-300).all()


def test_model_beats_slice_form_at_equal_bits():
    """At about the same bits (16 moduli: 56-bit integers; 8 slices: 56 bits),
    the exact integer product is at least as accurate as the slice products."""
    m, n, k = 12, 10, 200
    A = oracle.uniform((m, k), np.float64, 43, 0)
    B = oracle.uniform((k, n), np.float64, 43, 1)
    truth = oracle.dot2gemm("N", "N", m, n, k, 1.0, A, m, B, k, 0.0,
                            np.zeros((m, n), order="F"), m)
    e_crt = np.abs(crt.crt_gemm_model(A, B, 16) - truth).max()
    e_oz = np.abs(osp.ozaki_gemm_model(A, B, 8) - truth).max()
    assert e_crt <= e_oz


def test_nonfinite_rows_give_nan():
    A = np.ones((3, 4))
    A[1, 2] = np.inf
    B = np.ones((4, 2))
    B[0, 1] = np.nan
    out = crt.crt_gemm_model(A, B, 8)
    assert np.isnan(out[1]).all() and np.isnan(out[:, 1]).all()
    assert out[0, 0] == 4.0 and out[2, 0] == 4.0


def test_argument_errors_need_no_gpu():
    f = g.dgemm_ozaki2
    assert f("N", "N", 8, 8, 8, 1.0, 0, 8, 0, 8, 0.0, 0, 8, moduli=1) == g.ERR_ARG
    assert f("N", "N", 8, 8, 8, 1.0, 0, 8, 0, 8, 0.0, 0, 8, moduli=25) == g.ERR_ARG
    assert f("N", "N", 8, 8, 8, 1.0, 0, 7, 0, 8, 0.0, 0, 8) == g.ERR_ARG
    assert f("N", "N", 0, 8, 8, 1.0, 0, 1, 0, 8, 0.0, 0, 1) == g.OK
    assert g.split_workspace_bytes(2, 1000, 1000, 1000, 16) >= 16 * 2048 * 1024 * 2
