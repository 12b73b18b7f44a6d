"""GPU parity of the plain (drop-in) kernels through the C ABI.

Reference outputs come from the golden fixtures (the reference library's own
dgemm_/sgemm_) and from the bit-exact oracle restatement; tolerances are the
summation-order bound (k+2)*u*(|alpha||A||B| + |beta||C|), doubled, per
element, and for DGEMM additionally a 1e-13 relative Frobenius difference."""
import numpy as np
import pytest

import gemm_avx2_gb300 as g
from gpu_util import from_dev, sync, to_dev
from util import U32, U64, case_inputs, check_close, gemm_bound, golden_cases, op

pytestmark = pytest.mark.gpu


def run_device(prec, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, a_off=0, b_off=0):
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C)
    esz = 8 if prec == "d" else 4
    rc = g.gemm_device(prec, ta, tb, m, n, k, alpha, dA.data_ptr() + a_off * esz, lda,
                       dB.data_ptr() + b_off * esz, ldb, beta, dC.data_ptr(), ldc)
    assert rc == g.OK
    sync()
    return from_dev(dC, C.shape[0])


def frob_rel(x, y):
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    ok = np.isfinite(x) & np.isfinite(y)
    d = np.linalg.norm((x - y)[ok])
    ny = np.linalg.norm(y[ok])
    return d / ny if ny > 0 else d


def test_device_golden_cases(orc, golden):
    for c, dt, want in golden_cases(golden):
        A, B, C = case_inputs(orc, c, dt)
        prec, ta, tb = str(c["precision"]), str(c["transa"]), str(c["transb"])
        m, n, k = int(c["m"]), int(c["n"]), int(c["k"])
        alpha, beta = float(c["alpha"]), float(c["beta"])
        C0 = C.copy(order="F")
        got = run_device(prec, ta, tb, m, n, k, alpha, A, int(c["lda"]), B, int(c["ldb"]), beta,
                         C, int(c["ldc"]))
        u = U64 if prec == "d" else U32
        if m and n:
            check_close(got[:m, :n], want, gemm_bound(A, B, C0, ta, tb, m, n, k, alpha, beta, u))
            if prec == "d" and k:
                assert frob_rel(got[:m, :n], want) <= 1e-13
        # rows beyond m (padding of ldc) are never written
        assert np.array_equal(got[m:, :], C0[m:, :], equal_nan=True)
    assert g.device_error() == 0


@pytest.mark.parametrize("prec", ["d", "s"])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
@pytest.mark.parametrize("shape,ldpad", [((300, 257, 513), 0), ((129, 130, 17), 3),
                                         ((1, 700, 40), 1), ((257, 1, 129), 2),
                                         ((256, 384, 64), 4), ((97, 93, 1000), 5)])
def test_device_vs_oracle(orc, prec, ta, tb, shape, ldpad):
    """Multi-tile shapes; ldpad 0/4 keep TMA-aligned leading dimensions, odd pads
    force the cp.async fallback path."""
    dt = np.float64 if prec == "d" else np.float32
    m, n, k = shape
    ar, ac = (m, k) if ta == "N" else (k, m)
    br, bc = (k, n) if tb == "N" else (n, k)
    lda, ldb, ldc = ar + ldpad, br + ldpad, m + ldpad
    seed = 1000 + m + n + k
    A = orc.storage(ar, ac, lda, dt, seed, 0)
    B = orc.storage(br, bc, ldb, dt, seed, 1)
    C = orc.storage(m, n, ldc, dt, seed, 2)
    alpha, beta = 1.25, -0.5
    want = C.copy(order="F")
    orc.refgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, want, ldc, 4)
    got = run_device(prec, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc)
    u = U64 if prec == "d" else U32
    check_close(got[:m, :n], want[:m, :n], gemm_bound(A, B, C, ta, tb, m, n, k, alpha, beta, u))
    if prec == "d":
        assert frob_rel(got[:m, :n], want[:m, :n]) <= 1e-13
    assert np.array_equal(got[m:, :], C[m:, :])


@pytest.mark.parametrize("prec", ["d", "s"])
def test_misaligned_base_pointer(orc, prec):
    """Operands starting one element past a 16-byte boundary take the cp.async path."""
    dt = np.float64 if prec == "d" else np.float32
    m, n, k = 200, 150, 300
    Afull = orc.uniform((m * k + 1, 1), dt, 77, 0)
    Bfull = orc.uniform((k * n + 1, 1), dt, 77, 1)
    C = orc.uniform((m, n), dt, 77, 2)
    A = np.asfortranarray(Afull[1:, 0].reshape((m, k), order="F"))
    B = np.asfortranarray(Bfull[1:, 0].reshape((k, n), order="F"))
    want = C.copy(order="F")
    orc.refgemm("N", "N", m, n, k, 1.0, A, m, B, k, 1.0, want, m, 4)
    dA, dB, dC = to_dev(Afull), to_dev(Bfull), to_dev(C)
    esz = 8 if prec == "d" else 4
    assert g.gemm_device(prec, "N", "N", m, n, k, 1.0, dA.data_ptr() + esz, m,
                         dB.data_ptr() + esz, k, 1.0, dC.data_ptr(), m) == g.OK
    sync()
    got = from_dev(dC, m)
    u = U64 if prec == "d" else U32
    check_close(got, want, gemm_bound(A, B, C, "N", "N", m, n, k, 1.0, 1.0, u))


@pytest.mark.parametrize("prec", ["d", "s"])
def test_nan_and_alpha_beta_semantics(prec):
    dt = np.float64 if prec == "d" else np.float32
    m = n = k = 40
    A = np.full((m, k), np.nan, dt, order="F")
    B = np.ones((k, n), dt, order="F")
    C = np.ones((m, n), dt, order="F")
    C[3, 4] = np.nan
    # alpha == 0: A (all NaN) is never read; beta scales, NaN in C survives
    got = run_device(prec, "N", "N", m, n, k, 0.0, A, m, B, k, 3.0, C, m)
    assert np.isnan(got[3, 4]) and np.all(got[~np.isnan(got)] == 3.0)
    # beta == 0 still multiplies C: 0 * NaN = NaN, like the reference
    A = np.ones((m, k), dt, order="F")
    got = run_device(prec, "N", "N", m, n, k, 1.0, A, m, B, k, 0.0, C, m)
    assert np.isnan(got[3, 4]) and np.all(got[~np.isnan(got)] == float(k))
    # k == 0 with alpha != 0: beta*C only
    got = run_device(prec, "N", "N", m, n, 0, 1.0, A, m, B, 1, 2.0, C, m)
    assert np.isnan(got[3, 4]) and np.all(got[~np.isnan(got)] == 2.0)
    # alpha == 0, beta == 1: untouched
    got = run_device(prec, "N", "N", m, n, k, 0.0, A, m, B, k, 1.0, C, m)
    assert np.array_equal(np.isnan(got), np.isnan(C)) and np.all(got[~np.isnan(got)] == 1.0)


def test_dropin_host_path_golden(orc, golden):
    """DGEMM.so/SGEMM.so (the drop-in, host pointers) against the reference's outputs."""
    for c, dt, want in golden_cases(golden):
        A, B, C = case_inputs(orc, c, dt)
        prec, ta, tb = str(c["precision"]), str(c["transa"]), str(c["transb"])
        m, n, k = int(c["m"]), int(c["n"]), int(c["k"])
        alpha, beta = float(c["alpha"]), float(c["beta"])
        C0 = C.copy(order="F")
        f = g.dgemm if prec == "d" else g.sgemm
        f(ta, tb, m, n, k, alpha, A, int(c["lda"]), B, int(c["ldb"]), beta, C, int(c["ldc"]))
        u = U64 if prec == "d" else U32
        if m and n:
            check_close(C[:m, :n], want, gemm_bound(A, B, C0, ta, tb, m, n, k, alpha, beta, u))
        assert np.array_equal(C[m:, :], C0[m:, :], equal_nan=True)


def test_config1_dgemm_vs_reference(orc, golden):
    """Config 1: DGEMM NN 2048^3, alpha 1, beta 0.5, seed 0 through dgemm_ (host
    pointers) within 1e-13 relative Frobenius of the reference; error vs the
    Dot2 oracle on the sampled entries reported alongside."""
    N = 2048
    A = orc.uniform((N, N), np.float64, 0, 0)
    B = orc.uniform((N, N), np.float64, 0, 1)
    C = orc.uniform((N, N), np.float64, 0, 2)
    C0 = C.copy(order="F")
    g.dgemm("N", "N", N, N, N, 1.0, A, N, B, N, 0.5, C, N)
    rows, cols = golden["cfg1_rows"], golden["cfg1_cols"]
    ref_vals = golden["cfg1_vals"]
    got = C[rows, cols]
    assert frob_rel(got, ref_vals) <= 1e-13
    # full matrix against the bit-exact restatement of the reference
    want = C0.copy(order="F")
    orc.refgemm("N", "N", N, N, N, 1.0, A, N, B, N, 0.5, want, N, int(golden["cfg1_threads"]))
    assert frob_rel(C, want) <= 1e-13
    truth = orc.dot2gemm_sampled("N", "N", N, N, N, 1.0, A, N, B, N, 0.5, C0, N, rows, cols)
    e_gpu = frob_rel(got, truth)
    e_ref = frob_rel(ref_vals, truth)
    assert e_gpu < 4e-15 and e_ref < 4e-15
