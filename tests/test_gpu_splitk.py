"""Split-K of the plain kernels on the GPU (the role of the reference's K
blocking, src/gemm_driver.c:156-190: C *= beta first, then each K block's sum
is added to C).  Each slice of K goes to scratch and a second kernel adds the
slices to beta*C in K order, so a split call differs from the unsplit one only
in the grouping of the K sum.  Checked against the oracle's restatement of the
reference within the summation-order bound (DGEMM also 1e-13 relative
Frobenius), for forced splits, both ring depths, all transposes, ragged
shapes and padded leading dimensions; run twice for determinism."""
import numpy as np
import pytest

import gemm_avx2_gb300 as g
from gpu_util import from_dev, sync, to_dev
from util import U32, U64, check_close, gemm_bound

pytestmark = pytest.mark.gpu


@pytest.fixture
def knobs():
    yield
    g.tune_param(g.TUNE_SPLIT_K, 0)
    g.tune_param(g.TUNE_PLAIN_STAGES, 0)
    g.tune_cache_clear()


def frob_rel(x, y):
    return np.linalg.norm(np.asarray(x, np.float64) - y) / np.linalg.norm(y)


def inputs(orc, prec, ta, tb, m, n, k, pad, seed):
    dt = np.float64 if prec == "d" else np.float32
    ar, ac = (m, k) if ta == "N" else (k, m)
    br, bc = (k, n) if tb == "N" else (n, k)
    lda, ldb, ldc = ar + pad, br + pad, m + pad
    A = orc.storage(ar, ac, lda, dt, seed, 0)
    B = orc.storage(br, bc, ldb, dt, seed, 1)
    C = orc.storage(m, n, ldc, dt, seed, 2)
    return A, lda, B, ldb, C, ldc


def run(prec, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc):
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C)
    assert g.gemm_device(prec, ta, tb, m, n, k, alpha, dA.data_ptr(), lda, dB.data_ptr(), ldb,
                         beta, dC.data_ptr(), ldc) == g.OK
    sync()
    return from_dev(dC, C.shape[0])


@pytest.mark.parametrize("prec", ["d", "s"])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
@pytest.mark.parametrize("split,stages", [(2, 4), (5, 6), (16, 4)])
def test_forced_split_vs_oracle(orc, knobs, prec, ta, tb, split, stages):
    m, n, k = 200, 150, 3001   # 2 x 2 tiles, a ragged last k-tile
    A, lda, B, ldb, C, ldc = inputs(orc, prec, ta, tb, m, n, k, 0, 700 + split)
    want = C.copy(order="F")
    orc.refgemm(ta, tb, m, n, k, 0.75, A, lda, B, ldb, -1.5, want, ldc, 4)
    assert g.tune_param(g.TUNE_SPLIT_K, split) == g.OK
    assert g.tune_param(g.TUNE_PLAIN_STAGES, stages) == g.OK
    assert g.plain_layout(prec, m, n, k)[1:] == (split, stages)
    got = run(prec, ta, tb, m, n, k, 0.75, A, lda, B, ldb, -1.5, C, ldc)
    u = U64 if prec == "d" else U32
    check_close(got[:m], want[:m], gemm_bound(A, B, C, ta, tb, m, n, k, 0.75, -1.5, u))
    if prec == "d":
        assert frob_rel(got[:m], want[:m]) <= 1e-13
    again = run(prec, ta, tb, m, n, k, 0.75, A, lda, B, ldb, -1.5, C, ldc)
    assert np.array_equal(got, again)   # the slices are combined in a fixed order
    assert g.device_error() == 0


@pytest.mark.parametrize("prec", ["d", "s"])
def test_split_by_shape_ragged_padded(orc, knobs, prec):
    """The default choice splits a 3 x 2-tile output with long K; odd leading
    dimensions take the cp.async path; the ldc padding stays untouched."""
    m, n, k = 333, 190, 9000
    A, lda, B, ldb, C, ldc = inputs(orc, prec, "T", "N", m, n, k, 3, 77)
    assert g.plain_layout(prec, m, n, k)[1] > 1
    want = C.copy(order="F")
    orc.refgemm("T", "N", m, n, k, -1.0, A, lda, B, ldb, 1.0, want, ldc, 4)
    got = run(prec, "T", "N", m, n, k, -1.0, A, lda, B, ldb, 1.0, C, ldc)
    u = U64 if prec == "d" else U32
    check_close(got[:m], want[:m], gemm_bound(A, B, C, "T", "N", m, n, k, -1.0, 1.0, u))
    assert np.array_equal(got[m:], C[m:])
    assert g.device_error() == 0


def test_split_keeps_beta_semantics(orc, knobs):
    """beta = 0 still multiplies (NaN in C stays NaN, as C_MULT_BETA does);
    beta = 1 leaves C unscaled."""
    m, n, k = 130, 140, 2048
    A, lda, B, ldb, C, ldc = inputs(orc, "d", "N", "N", m, n, k, 0, 78)
    C[5, 7] = np.nan
    assert g.tune_param(g.TUNE_SPLIT_K, 4) == g.OK
    got = run("d", "N", "N", m, n, k, 1.0, A, lda, B, ldb, 0.0, C, ldc)
    finite = np.ones(got.shape, bool)
    finite[5, 7] = False
    assert np.isnan(got[5, 7]) and np.isfinite(got[finite]).all()
    C[5, 7] = 0.25
    want = C.copy(order="F")
    orc.refgemm("N", "N", m, n, k, 2.0, A, lda, B, ldb, 1.0, want, ldc, 4)
    got = run("d", "N", "N", m, n, k, 2.0, A, lda, B, ldb, 1.0, C, ldc)
    check_close(got, want, gemm_bound(A, B, C, "N", "N", m, n, k, 2.0, 1.0, U64))
    assert g.device_error() == 0


def test_host_dropin_splits(orc, knobs):
    """The drop-in dgemm_ (host pointers) takes the split too."""
    m, n, k = 256, 200, 12000
    A, lda, B, ldb, C, ldc = inputs(orc, "d", "N", "T", m, n, k, 0, 79)
    assert g.plain_layout("d", m, n, k)[1] > 1
    want = C.copy(order="F")
    orc.refgemm("N", "T", m, n, k, 1.0, A, lda, B, ldb, 0.5, want, ldc, 4)
    got = C.copy(order="F")
    g.dgemm("N", "T", m, n, k, 1.0, A, lda, B, ldb, 0.5, got, ldc)
    check_close(got, want, gemm_bound(A, B, C, "N", "T", m, n, k, 1.0, 0.5, U64))
    assert frob_rel(got, want) <= 1e-13


@pytest.mark.parametrize("prec", ["d", "s"])
def test_autotune_plain(orc, knobs, prec):
    """The autotuner times the split-K factors and ring depths of the plain
    kernel for a shape class and caches the fastest; calls of the class use it."""
    m, n, k = 256, 256, 16384
    A, lda, B, ldb, C, ldc = inputs(orc, prec, "N", "N", m, n, k, 0, 80)
    dA, dB = to_dev(A), to_dev(B)
    kind = g.TUNE_PLAIN_D if prec == "d" else g.TUNE_PLAIN_S
    rc, split = g.autotune(kind, "N", "N", m, n, k, dA.data_ptr(), lda, dB.data_ptr(), ldb)
    assert rc == g.OK and 1 <= split <= 32
    rc, sk, st = g.plain_layout(prec, m, n, k)
    assert rc == g.OK and sk == split and st in (4, 6)
    want = C.copy(order="F")
    orc.refgemm("N", "N", m, n, k, 1.0, A, lda, B, ldb, 1.0, want, ldc, 4)
    got = run(prec, "N", "N", m, n, k, 1.0, A, lda, B, ldb, 1.0, C, ldc)
    u = U64 if prec == "d" else U32
    check_close(got, want, gemm_bound(A, B, C, "N", "N", m, n, k, 1.0, 1.0, u))
    assert g.device_error() == 0
