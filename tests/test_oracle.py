"""CPU tests of the oracle: generator pins, bit-exact parity of the reference
restatement with the reference's own outputs (golden vectors), Dot2 accuracy."""
import numpy as np
import pytest

from util import case_inputs, golden_cases


def test_generator_pinned_draws(orc, golden):
    d = golden["draws"]
    for s in range(d.shape[0]):
        for st in range(d.shape[1]):
            got = [orc.lib().orc_draw(s, st, i) for i in range(d.shape[2])]
            assert got == [int(x) for x in d[s, st]]


def test_generator_ranges(orc):
    x = orc.uniform((1000, 3), np.float64, 5, 0)
    assert x.min() >= -1.0 and x.max() < 1.0
    y = orc.uniform((1000, 3), np.float32, 5, 0)
    assert y.min() >= -1.0 and y.max() < 1.0
    # FP32 values are on the 2^-23 grid, FP64 on 2^-52
    assert np.all((y.astype(np.float64) + 1.0) * 2**23 == np.round((y.astype(np.float64) + 1.0) * 2**23))
    z = orc.spread((500, 4), 2, 0, 4.0)
    assert np.isfinite(z).all() and orc.exponent_spread(z) > 20


def test_refgemm_bitexact_vs_reference_golden(orc, golden):
    """The restatement reproduces the reference library's outputs bit for bit."""
    n = 0
    for c, dt, want in golden_cases(golden):
        A, B, C = case_inputs(orc, c, dt)
        orc.refgemm(str(c["transa"]), str(c["transb"]), int(c["m"]), int(c["n"]), int(c["k"]),
                    float(c["alpha"]), A, int(c["lda"]), B, int(c["ldb"]), float(c["beta"]), C,
                    int(c["ldc"]), int(c["threads"]))
        got = np.asfortranarray(C[:int(c["m"]), :int(c["n"])])
        iv = np.uint64 if dt == np.float64 else np.uint32
        assert np.array_equal(got.view(iv), want.view(iv)), c
        n += 1
    assert n == len(golden["cases"])


def test_refgemm_cfg1_sampled_vs_reference(orc, golden):
    """Config 1 (DGEMM NN 2048^3, alpha 1, beta 0.5, seed 0): bitwise on 4096
    sampled entries of the reference's output."""
    N = 2048
    A = orc.uniform((N, N), np.float64, 0, 0)
    B = orc.uniform((N, N), np.float64, 0, 1)
    C = orc.uniform((N, N), np.float64, 0, 2)
    orc.refgemm("N", "N", N, N, N, 1.0, A, N, B, N, 0.5, C, N, int(golden["cfg1_threads"]))
    got = C[golden["cfg1_rows"], golden["cfg1_cols"]]
    assert np.array_equal(got.view(np.uint64), golden["cfg1_vals"].view(np.uint64))


@pytest.mark.skipif("not __import__('oracle').RefLib.available()")
def test_refgemm_vs_live_reference_randomized(orc):
    """Where the reference library was compiled here: random shapes, teams of 1-5."""
    ref = orc.RefLib()
    rng = np.random.default_rng(7)
    for it in range(24):
        prec = "d" if it % 2 == 0 else "s"
        dt = np.float64 if prec == "d" else np.float32
        ta, tb = "NT"[rng.integers(2)], "NT"[rng.integers(2)]
        m, n, k = (int(x) for x in rng.integers(0, 120, 3))
        n = n * 4
        k = k * 5
        T = int(rng.integers(1, 6))
        ar = m if ta == "N" else k
        br = k if tb == "N" else n
        lda, ldb, ldc = max(ar, 1) + 2, max(br, 1) + 1, max(m, 1) + 3
        A = orc.uniform((lda, k if ta == "N" else m), dt, it, 0)
        B = orc.uniform((ldb, n if tb == "N" else k), dt, it, 1)
        C = orc.uniform((ldc, n), dt, it, 2)
        alpha, beta = float(rng.choice([1.0, -0.5, 0.0])), float(rng.choice([1.0, 0.0, 2.5]))
        C1, C2 = C.copy(order="F"), C.copy(order="F")
        orc.set_threads(T)
        ref.gemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C1, ldc)
        orc.refgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C2, ldc, T)
        iv = np.uint64 if dt == np.float64 else np.uint32
        assert np.array_equal(C1.view(iv), C2.view(iv)), (prec, ta, tb, m, n, k, T)


def test_refgemm_nan_semantics(orc):
    """beta == 0 multiplies (NaN in C survives); alpha == 0 never reads A/B."""
    A = np.full((4, 4), np.nan, order="F")
    B = np.ones((4, 4), order="F")
    C = np.ones((4, 4), order="F")
    C[1, 2] = np.nan
    orc.refgemm("N", "N", 4, 4, 4, 0.0, A, 4, B, 4, 3.0, C, 4, 2)
    assert np.isnan(C[1, 2]) and np.all(C[~np.isnan(C)] == 3.0)
    A = np.ones((4, 4), order="F")
    C = np.ones((4, 4), order="F")
    C[0, 0] = np.nan
    orc.refgemm("N", "N", 4, 4, 4, 1.0, A, 4, B, 4, 0.0, C, 4, 2)
    assert np.isnan(C[0, 0]) and np.all(C[1:, :] == 4.0)


def test_dot2_exact_on_cancellation(orc):
    """Dot2 returns the exactly rounded result where plain summation fails."""
    a = np.array([[1e16, 1.0, -1e16, 1.0]], order="F")
    b = np.array([[1.0], [1.0], [1.0], [1.0]], order="F")
    c = np.zeros((1, 1), order="F")
    out = orc.dot2gemm("N", "N", 1, 1, 4, 1.0, a, 1, b, 4, 0.0, c, 1)
    assert out[0, 0] == 2.0
    s = orc.dot2gemm_sampled("N", "N", 1, 1, 4, 2.0, a, 1, b, 4, 1.0, np.full((1, 1), 3.0, order="F"), 1,
                             [0], [0])
    assert s[0] == 7.0


def test_dot2_matches_longdouble_small(orc):
    rng = np.random.default_rng(3)
    A = np.asfortranarray(rng.standard_normal((13, 11)))
    B = np.asfortranarray(rng.standard_normal((11, 9)))
    C = np.asfortranarray(rng.standard_normal((13, 9)))
    out = orc.dot2gemm("N", "N", 13, 9, 11, 1.5, A, 13, B, 11, -0.5, C, 13)
    from fractions import Fraction
    for i in range(13):
        for j in range(9):
            exact = Fraction(1.5) * sum(Fraction(A[i, p]) * Fraction(B[p, j]) for p in range(11)) \
                + Fraction(-0.5) * Fraction(C[i, j])
            assert abs(Fraction(out[i, j]) - exact) <= abs(exact) * Fraction(2.3e-16) + Fraction(1e-300)
