"""The autotuner on the GPU: measured equal-error choice, cached per shape
class, then used by products = 0 / slices = 0."""
import numpy as np
import pytest

import gemm_avx2_gb300 as g
from gpu_util import from_dev, plain_unsplit, sync, to_dev

pytestmark = pytest.mark.gpu


def rel(x, t):
    d = np.abs(x - t)
    return float(np.max(d / np.maximum(np.abs(t), 1e-300))), float(np.linalg.norm(d) / np.linalg.norm(t))


def test_autotune_ozaki_and_use(orc):
    g.tune_cache_clear()
    m, n, k = 300, 260, 700
    A = orc.spread((m, k), 51, 0, 2.0)
    B = orc.spread((n, k), 51, 1, 2.0)          # transb = T
    dA, dB = to_dev(A), to_dev(B)
    rc, S = g.autotune(g.TUNE_OZAKI, "N", "T", m, n, k, dA.data_ptr(), m, dB.data_ptr(), n)
    assert rc == g.OK and 4 <= S <= 12
    assert g.tune_lookup(g.TUNE_OZAKI, m, n, k) == (g.OK, S, 0)
    C0 = np.zeros((m, n), order="F")
    truth = orc.dot2gemm("N", "T", m, n, k, 1.0, A, m, B, n, 0.0, C0, m)
    dC1, dC2 = to_dev(C0), to_dev(C0)
    assert g.dgemm_ozaki("N", "T", m, n, k, 1.0, dA.data_ptr(), m, dB.data_ptr(), n, 0.0,
                         dC1.data_ptr(), m, slices=0) == g.OK
    with plain_unsplit():
        assert g.gemm_device("d", "N", "T", m, n, k, 1.0, dA.data_ptr(), m, dB.data_ptr(), n,
                             0.0, dC2.data_ptr(), m) == g.OK
    sync()
    e_tuned, e_plain = rel(from_dev(dC1, m), truth), rel(from_dev(dC2, m), truth)
    # tuned against the S = 12 reference, checked here against Dot2: same order as plain
    assert e_tuned[0] <= 4 * e_plain[0] and e_tuned[1] <= 4 * e_plain[1], (S, e_tuned, e_plain)
    g.tune_cache_clear()


def test_autotune_crt_and_use(orc):
    g.tune_cache_clear()
    m, n, k = 300, 260, 700
    A = orc.spread((m, k), 52, 0, 2.0)
    B = orc.spread((n, k), 52, 1, 2.0)          # transb = T
    dA, dB = to_dev(A), to_dev(B)
    rc, N = g.autotune(g.TUNE_CRT, "N", "T", m, n, k, dA.data_ptr(), m, dB.data_ptr(), n)
    assert rc == g.OK and 11 <= N <= 24
    assert g.tune_lookup(g.TUNE_CRT, m, n, k) == (g.OK, N, 0)
    C0 = np.zeros((m, n), order="F")
    truth = orc.dot2gemm("N", "T", m, n, k, 1.0, A, m, B, n, 0.0, C0, m)
    dC1, dC2 = to_dev(C0), to_dev(C0)
    assert g.dgemm_ozaki2("N", "T", m, n, k, 1.0, dA.data_ptr(), m, dB.data_ptr(), n, 0.0,
                          dC1.data_ptr(), m, moduli=0) == g.OK
    with plain_unsplit():
        assert g.gemm_device("d", "N", "T", m, n, k, 1.0, dA.data_ptr(), m, dB.data_ptr(), n,
                             0.0, dC2.data_ptr(), m) == g.OK
    sync()
    e_tuned, e_plain = rel(from_dev(dC1, m), truth), rel(from_dev(dC2, m), truth)
    assert e_tuned[0] <= 4 * e_plain[0] and e_tuned[1] <= 4 * e_plain[1], (N, e_tuned, e_plain)
    g.tune_cache_clear()
    assert g.tune_lookup(g.TUNE_CRT, m, n, k) == (g.ERR_UNSUPPORTED, 16, 0)


def test_autotune_bf16x_and_use(orc):
    g.tune_cache_clear()
    m, n, k = 384, 300, 1000
    A = orc.uniform((k, m), np.float32, 52, 0)    # transa = T
    B = orc.uniform((k, n), np.float32, 52, 1)
    dA, dB = to_dev(A), to_dev(B)
    rc, P = g.autotune(g.TUNE_BF16X, "T", "N", m, n, k, dA.data_ptr(), k, dB.data_ptr(), k)
    assert rc == g.OK and P in (3, 6)
    st, P2, chunk = g.tune_lookup(g.TUNE_BF16X, m, n, k)
    assert st == g.OK and P2 == P and chunk in (2, 4, 8)
    C0 = np.zeros((m, n), np.float32, order="F")
    dC1, dC2 = to_dev(C0), to_dev(C0)
    assert g.sgemm_bf16x("T", "N", m, n, k, 1.0, dA.data_ptr(), k, dB.data_ptr(), k, 0.0,
                         dC1.data_ptr(), m, products=0) == g.OK
    g.tune_param(g.TUNE_BF16X_CHUNK, chunk)
    assert g.sgemm_bf16x("T", "N", m, n, k, 1.0, dA.data_ptr(), k, dB.data_ptr(), k, 0.0,
                         dC2.data_ptr(), m, products=P) == g.OK
    g.tune_param(g.TUNE_BF16X_CHUNK, 0)
    sync()
    # products = 0 runs exactly the tuned configuration
    assert np.array_equal(from_dev(dC1, m), from_dev(dC2, m))
    g.tune_cache_clear()
