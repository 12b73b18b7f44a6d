"""GPU tests of the CRT (modular-integer) FP64 form: the residue kernel and the
whole result bit for bit against the exact-integer model in oracle/crt.py, and
its accuracy against the Dot2 oracle and the plain FP64 kernel."""
import numpy as np
import pytest

import gemm_avx2_gb300 as g
import oracle
from gpu_util import from_dev, plain_unsplit, sync, to_dev, torch_cuda
from oracle import crt
from util import op

pytestmark = pytest.mark.gpu


def ru(x, a):
    return (x + a - 1) // a * a


def run_crt(ta, tb, m, n, k, A, lda, B, ldb, C, N, alpha=1.0, beta=0.0):
    """The CRT call on a workspace filled with 0xFF bytes (BF16 NaN): the
    padding rows and K columns of the residue blocks are never written, and
    the GEMM must never read them."""
    torch = torch_cuda()
    need = g.split_workspace_bytes(2, m, n, k, N)
    ws = torch.full((need,), 255, dtype=torch.uint8, device="cuda")
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C)
    rc = g.dgemm_ozaki2(ta, tb, m, n, k, alpha, dA.data_ptr(), lda, dB.data_ptr(), ldb, beta,
                        dC.data_ptr(), C.shape[0], moduli=N, workspace=ws.data_ptr(),
                        workspace_bytes=need)
    sync()
    return rc, from_dev(dC, C.shape[0]), ws


def residue_blocks(ws, N, Mp, Np, Kp):
    raw = ws.cpu().numpy()[(-ws.data_ptr()) % 1024:]
    bf = raw[:2 * N * (Mp + Np) * Kp].view(np.uint16).astype(np.uint32) << 16
    vals = bf.view(np.float32).astype(np.float64)
    return vals[:N * Mp * Kp].reshape(N, Mp, Kp), vals[N * Mp * Kp:].reshape(N, Np, Kp)


@pytest.mark.parametrize("N", [8, 16])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
def test_residues_and_result_bitexact(orc, N, ta, tb, tile_n):
    m, n, k = 150, 140, 200
    ar, ac = (m, k) if ta == "N" else (k, m)
    br, bc = (k, n) if tb == "N" else (n, k)
    A = orc.spread((ar + 2, ac), 51, 0, 1.0)
    B = orc.spread((br, bc), 51, 1, 1.0)
    C = orc.uniform((m, n), np.float64, 51, 2)
    rc, got, ws = run_crt(ta, tb, m, n, k, A, ar + 2, B, br, C, N, beta=0.5)
    assert rc == g.OK
    Aop, Bop = op(A, ta, m, k), op(B, tb, k, n)
    b = crt.crt_bits(N, k)
    As, Bs = residue_blocks(ws, N, ru(m, 128), ru(n, 256), ru(k, 64))
    ra = crt.residues(crt.scaled_integers(Aop, b)[0], N)
    rb = crt.residues(crt.scaled_integers(Bop.T, b)[0], N)
    for i in range(N):
        assert np.array_equal(As[i, :m, :k], ra[i]), i
        assert np.array_equal(Bs[i, :n, :k], rb[i]), i
    model = crt.crt_gemm_model(Aop, Bop, N, alpha=1.0, beta=0.5, C=C)
    assert np.array_equal(got, model), np.abs(got - model).max()
    assert g.device_error() == 0


@pytest.mark.parametrize("N", [16, 24])
def test_extreme_exponents_bitexact(orc, N):
    """Subnormal rows, rows spanning 600 decades, zero rows; 24 moduli make b
    large enough that most residues go through 2^t mod p."""
    m, n, k = 70, 40, 90
    rng = np.random.default_rng(7)
    Aop = rng.standard_normal((m, k)) * np.exp2(rng.integers(-40, 40, (m, k)))
    Aop[0] = rng.standard_normal(k) * 5e-324 * rng.integers(1, 2 ** 20, k)
    Aop[1, :] = 0.0
    Aop[2] = rng.standard_normal(k) * np.exp2(rng.integers(-1000, 1000, k))
    Aop[3, ::3] = 5e-324
    Aop[5, 0] = np.finfo(np.float64).max / 4
    A = np.asfortranarray(Aop)
    B = orc.uniform((k, n), np.float64, 52, 1)
    C = np.zeros((m, n), order="F")
    rc, got, ws = run_crt("N", "N", m, n, k, A, m, B, k, C, N)
    assert rc == g.OK
    b = crt.crt_bits(N, k)
    As, _ = residue_blocks(ws, N, ru(m, 128), ru(n, 256), ru(k, 64))
    ra = crt.residues(crt.scaled_integers(Aop, b)[0], N)
    for i in range(N):
        assert np.array_equal(As[i, :m, :k], ra[i]), i
    model = crt.crt_gemm_model(Aop, B, N)
    assert np.array_equal(got, model, equal_nan=True), np.nanmax(np.abs(got - model))


@pytest.mark.parametrize("m", [300, 129])
def test_odd_row_tiles_bitexact(orc, m, tile_n, cluster_mode):
    """3 and 2 row tiles, in each cluster mode (m = 300: the pair MMAs' 2-CTA
    clusters get a spare tile that must store no residues over a neighbour's;
    m = 129: a 1-row last tile)."""
    n, k = 290, 150
    A = orc.spread((m, k), 58, 0, 1.0)
    B = orc.spread((k, n), 58, 1, 1.0)
    C = orc.uniform((m + 3, n), np.float64, 58, 2)
    rc, got, _ = run_crt("N", "N", m, n, k, A, m, B, k, C, 16, beta=0.5)
    assert rc == g.OK
    assert np.array_equal(got[m:], C[m:])
    model = crt.crt_gemm_model(A, B, 16, alpha=1.0, beta=0.5, C=C[:m])
    assert np.array_equal(got[:m], model)
    assert g.device_error() == 0


@pytest.mark.parametrize("k", [1100, 2100])
def test_multi_chunk_bitexact(orc, k, cluster_mode):
    """K beyond one 1024-step TMEM chunk (2 and 3 chunks per modulus): the
    epilogue's integer path that reduces the chunk sums mod p and packs the
    residues of 4 columns per word; 2 row tiles, both cluster modes."""
    m, n = 140, 36
    A = orc.spread((m, k), 59, 0, 1.0)
    B = orc.spread((k, n), 59, 1, 1.0)
    C = orc.uniform((m + 1, n), np.float64, 59, 2)
    rc, got, _ = run_crt("N", "N", m, n, k, A, m, B, k, C, 15, alpha=-1.0, beta=1.0)
    assert rc == g.OK
    assert np.array_equal(got[m:], C[m:])
    model = crt.crt_gemm_model(A, B, 15, alpha=-1.0, beta=1.0, C=C[:m])
    assert np.array_equal(got[:m], model)
    assert g.device_error() == 0


def test_general_alpha_beta_bitexact(orc, cluster_mode):
    """alpha and beta that are not powers of two: the C update is
    beta c + alpha v with each product and the sum rounded once, as in the
    model (no fused multiply-add, whatever the kernel instantiation)."""
    m, n, k = 260, 150, 300
    A = orc.spread((m, k), 60, 0, 1.0)
    B = orc.spread((k, n), 60, 1, 1.0)
    C = orc.uniform((m, n), np.float64, 60, 2)
    rc, got, _ = run_crt("N", "N", m, n, k, A, m, B, k, C, 16, alpha=0.7318, beta=-1.3)
    assert rc == g.OK
    model = crt.crt_gemm_model(A, B, 16, alpha=0.7318, beta=-1.3, C=C)
    assert np.array_equal(got, model), np.abs(got - model).max()
    assert g.device_error() == 0


def test_nonfinite_rows_and_columns(orc):
    m, n, k = 40, 30, 50
    A = orc.uniform((m, k), np.float64, 53, 0)
    B = orc.uniform((k, n), np.float64, 53, 1)
    A[4, 7] = np.inf
    B[3, 9] = np.nan
    C = np.zeros((m, n), order="F")
    rc, got, _ = run_crt("N", "N", m, n, k, A, m, B, k, C, 16)
    assert rc == g.OK
    assert np.isnan(got[4]).all() and np.isnan(got[:, 9]).all()
    mask = np.ones((m, n), bool)
    mask[4] = False
    mask[:, 9] = False
    assert np.isfinite(got[mask]).all()


def test_accuracy_vs_plain(orc):
    """16 moduli: at least as accurate as the plain FP64 kernel (uniform data)."""
    m = n = 384
    k = 2048
    A = orc.uniform((m, k), np.float64, 54, 0)
    B = orc.uniform((n, k), np.float64, 54, 1)
    C = orc.uniform((m, n), np.float64, 54, 2)
    rc, got, _ = run_crt("N", "T", m, n, k, A, m, B, n, C, 16, beta=1.0)
    assert rc == g.OK
    dC = to_dev(C)
    dA, dB = to_dev(A), to_dev(B)
    with plain_unsplit():
        assert g.gemm_device("d", "N", "T", m, n, k, 1.0, dA.data_ptr(), m, dB.data_ptr(), n,
                             1.0, dC.data_ptr(), m) == g.OK
    sync()
    plain = from_dev(dC, m)
    truth = orc.dot2gemm("N", "T", m, n, k, 1.0, A, m, B, n, 1.0, C, m)
    e_crt = np.abs(got - truth).max() / np.abs(truth).max()
    e_plain = np.abs(plain - truth).max() / np.abs(truth).max()
    assert e_crt <= e_plain, (e_crt, e_plain)


def test_too_few_moduli_for_k(orc):
    # 2 moduli (M = 64515) leave no bit at k = 40000: 2k (2^1 - 1)^2 > M
    k = 40000
    A = orc.uniform((1, k), np.float64, 55, 0)
    B = orc.uniform((k, 1), np.float64, 55, 1)
    C = np.zeros((1, 1), order="F")
    torch = torch_cuda()
    need = g.split_workspace_bytes(2, 1, 1, k, 2)
    ws = torch.zeros(max(need, 1), dtype=torch.uint8, device="cuda")
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C)
    rc = g.dgemm_ozaki2("N", "N", 1, 1, k, 1.0, dA.data_ptr(), 1, dB.data_ptr(), k, 0.0,
                        dC.data_ptr(), 1, moduli=2, workspace=ws.data_ptr(), workspace_bytes=need)
    assert rc == g.ERR_ARG


def test_alpha0_and_k0(orc):
    m, n = 33, 17
    C = orc.uniform((m, n), np.float64, 56, 2)
    dC = to_dev(C)
    assert g.dgemm_ozaki2("N", "N", m, n, 5, 0.0, 0, m, 0, 5, 0.5, dC.data_ptr(), m) == g.OK
    assert g.dgemm_ozaki2("N", "N", m, n, 0, 1.0, 0, m, 0, 1, 2.0, dC.data_ptr(), m) == g.OK
    sync()
    assert np.array_equal(from_dev(dC, m), C)  # 0.5 then 2.0: exact


def test_host_path(orc):
    m, n, k = 90, 70, 130
    A = orc.uniform((k, m), np.float64, 57, 0)
    B = orc.uniform((k, n), np.float64, 57, 1)
    C = orc.uniform((m, n), np.float64, 57, 2)
    Cg = C.copy(order="F")
    assert g.host_split_gemm("crt", "T", "N", m, n, k, 1.0, A, k, B, k, 0.5, Cg, m, 16) == g.OK
    model = crt.crt_gemm_model(A.T, B, 16, alpha=1.0, beta=0.5, C=C)
    assert np.array_equal(Cg, model)


@pytest.mark.parametrize("shape", [(700, 600, 500), (2100, 1900, 300)])
def test_modulus_split_units_bitexact(orc, shape):
    """Whole-tile units and one-modulus units give the same result bit for bit
    (the moduli are independent GEMMs)."""
    m, n, k = shape
    A = orc.spread((m, k), 59, 0, 1.0)
    B = orc.spread((n, k), 59, 1, 1.0)
    C = orc.uniform((m, n), np.float64, 59, 2)
    got = {}
    try:
        for mode in (1, 2):
            assert g.tune_param(g.TUNE_MODULUS_SPLIT, mode) == g.OK
            rc, got[mode], _ = run_crt("N", "T", m, n, k, A, m, B, n, C, 15, beta=0.5)
            assert rc == g.OK
    finally:
        g.tune_param(g.TUNE_MODULUS_SPLIT, 0)
    assert np.array_equal(got[1], got[2])
    assert g.device_error() == 0
