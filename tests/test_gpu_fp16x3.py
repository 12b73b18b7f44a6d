"""GPU tests of the scaled 3xFP16 split SGEMM (products = FP16X3): the split
operands and scale exponents bit for bit against oracle/split.py, the result
against the FP64 model of the represented operands, and its accuracy against
the Dot2 oracle next to the plain FP32 kernel."""
import numpy as np
import pytest

import gemm_avx2_gb300 as g
from gpu_util import from_dev, plain_unsplit, sync, to_dev, torch_cuda
from oracle import split as osp
from util import op

pytestmark = pytest.mark.gpu


def ru(x, a):
    return (x + a - 1) // a * a


def rel_errs(x, truth):
    d = np.abs(np.asarray(x, np.float64) - truth)
    return np.max(d / np.maximum(np.abs(truth), 1e-300)), np.linalg.norm(d) / np.linalg.norm(truth)


def run(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc=None):
    torch = torch_cuda()
    need = g.split_workspace_bytes(0, m, n, k, g.FP16X3)
    ws = torch.full((need,), 255, dtype=torch.uint8, device="cuda")  # padding never read
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C)
    rc = g.sgemm_bf16x(ta, tb, m, n, k, alpha, dA.data_ptr(), lda, dB.data_ptr(), ldb, beta,
                       dC.data_ptr(), ldc or C.shape[0], products=g.FP16X3,
                       workspace=ws.data_ptr(), workspace_bytes=need)
    sync()
    return rc, from_dev(dC, C.shape[0]), ws


def workspace_parts(ws, m, n, k):
    """A' (Mp x 2Kp), B' (Np x 2Kp) as uint16 (terms hi, lo), then the
    exponents (Mp + Np)."""
    Kp, Mp, Np = ru(k, 64), ru(m, 128), ru(n, 256)
    raw = ws.cpu().numpy()
    base = ws.data_ptr()
    off = (-base) % 1024
    kld = 2 * Kp
    h = raw[off:off + 2 * (Mp + Np) * kld].view(np.uint16)
    Ap, Bp = h[:Mp * kld].reshape(Mp, kld), h[Mp * kld:].reshape(Np, kld)
    end = base + off + 2 * (Mp + Np) * kld
    a_off = (-end) % 256 + off + 2 * (Mp + Np) * kld
    ex_off = a_off + 4 * (Mp + Np) + 16  # past the max pass's completion counter
    ex = raw[ex_off:ex_off + 4 * (Mp + Np)].view(np.int32)
    return Ap, Bp, ex[:Mp], ex[Mp:], Mp, Np, Kp


def model_check(got, Aop, Bop, alpha, beta, C):
    """|got - (alpha model + beta C)| within FP32 accumulation error of |A||B|."""
    model = alpha * osp.fp16x3_model(Aop, Bop) + beta * C.astype(np.float64)
    mag = np.abs(Aop.astype(np.float64)) @ np.abs(Bop.astype(np.float64))
    bound = 2.0 ** -20 * (abs(alpha) * mag + abs(beta) * np.abs(C)) + 1e-300
    assert np.all(np.abs(got - model) <= bound), np.max(np.abs(got - model) / bound)


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
def test_split_bitexact_and_result(orc, ta, tb, tile_n):
    m, n, k = 200, 300, 100
    ar, ac = (m, k) if ta == "N" else (k, m)
    br, bc = (k, n) if tb == "N" else (n, k)
    A = orc.uniform((ar + 1, ac), np.float32, 71, 0)
    B = orc.uniform((br + 3, bc), np.float32, 71, 1)
    A[:, :] *= np.float32(2.0 ** 40)       # the row scaling brings it back into FP16 range
    C = orc.uniform((m, n), np.float32, 71, 2)
    rc, got, ws = run(ta, tb, m, n, k, 1.0, A, ar + 1, B, br + 3, 0.5, C)
    assert rc == g.OK
    Ap, Bp, eA, eB, Mp, Np, Kp = workspace_parts(ws, m, n, k)
    Aop = np.zeros((Mp, Kp), np.float32)
    Aop[:m, :k] = op(A, ta, m, k)
    Bop = np.zeros((Np, Kp), np.float32)
    Bop[:n, :k] = op(B, tb, k, n).T
    # the rows holding op(A) / op(B) (rows past them are left unwritten)
    assert np.array_equal(eA[:m], osp.row_exponents_f32(Aop)[:m])
    assert np.array_equal(eB[:n], osp.row_exponents_f32(Bop)[:n])
    assert np.array_equal(Ap[:m], osp.fp16x3_operand(Aop, True)[:m])
    assert np.array_equal(Bp[:n], osp.fp16x3_operand(Bop, False)[:n])
    model_check(got, op(A, ta, m, k), op(B, tb, k, n), 1.0, 0.5, C)
    assert g.device_error() == 0


def test_multi_tile_ragged_and_odd_row_tiles(orc, tile_n):
    m, n, k = 300, 520, 333
    A = orc.uniform((k, m), np.float32, 72, 0)
    B = orc.uniform((k, n), np.float32, 72, 1)
    C = orc.uniform((m + 5, n), np.float32, 72, 2)
    rc, got, _ = run("T", "N", m, n, k, -1.0, A, k, B, k, 1.0, C)
    assert rc == g.OK
    assert np.array_equal(got[m:], C[m:])  # padding rows and the cluster's spare tile
    model_check(got[:m], A.T, B, -1.0, 1.0, C[:m])


def test_extreme_exponents(orc):
    """Rows and columns at 2^+-100, FP32 subnormal rows, rows spanning 2^60,
    zero rows: the scale exponents and the result against the model."""
    m, n, k = 70, 60, 90
    rng = np.random.default_rng(9)
    Aop = rng.uniform(-1, 1, (m, k)).astype(np.float32)
    Aop[0] *= np.float32(2.0 ** 100)
    Aop[1] = (rng.uniform(-1, 1, k) * 2.0 ** -130).astype(np.float32)   # subnormal
    Aop[2] = 0
    Aop[3] = (rng.uniform(-1, 1, k) * np.exp2(rng.integers(-30, 30, k))).astype(np.float32)
    Aop[4, 5] = np.float32(3.0e38)
    Bop = rng.uniform(-1, 1, (k, n)).astype(np.float32)
    Bop[:, 0] *= np.float32(2.0 ** -100)
    Bop[:, 1] *= np.float32(2.0 ** 60)
    A, B = np.asfortranarray(Aop), np.asfortranarray(Bop)
    C = np.zeros((m, n), np.float32, order="F")
    rc, got, ws = run("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, C)
    assert rc == g.OK
    _, _, eA, eB, Mp, Np, Kp = workspace_parts(ws, m, n, k)
    assert np.array_equal(eA[:m], osp.row_exponents_f32(Aop))
    assert np.array_equal(eB[:n], osp.row_exponents_f32(Bop.T))
    with np.errstate(over="ignore", invalid="ignore"):
        model = osp.fp16x3_model(Aop, Bop)
    fin = np.isfinite(model) & (np.abs(model) < 3e38)
    assert np.all(np.isfinite(got[fin]))
    mag = np.abs(Aop.astype(np.float64)) @ np.abs(Bop.astype(np.float64))
    # + the FP32 underflow quantum: products near 2^-230 flush to zero
    assert np.all(np.abs(got[fin] - model[fin]) <= 2.0 ** -20 * mag[fin] + 2.0 ** -148)
    assert np.all(got[2] == 0)


def test_nonfinite_rows_and_columns(orc):
    m, n, k = 40, 30, 50
    A = orc.uniform((m, k), np.float32, 73, 0)
    B = orc.uniform((k, n), np.float32, 73, 1)
    A[4, 7] = np.inf
    B[3, 9] = np.nan
    C = np.zeros((m, n), np.float32, order="F")
    rc, got, _ = run("N", "N", m, n, k, 1.0, A, m, B, k, 0.0, C)
    assert rc == g.OK
    assert np.isnan(got[4]).all() and np.isnan(got[:, 9]).all()
    mask = np.ones((m, n), bool)
    mask[4] = False
    mask[:, 9] = False
    assert np.isfinite(got[mask]).all()


def test_accuracy_vs_plain_and_6xbf16(orc):
    """Uniform[-1,1) data (the SGEMM workload's distribution): max and
    Frobenius errors against the Dot2 oracle at or below the plain kernel's."""
    m = n = 384
    k = 4096
    A = orc.uniform((k, m), np.float32, 74, 0)
    B = orc.uniform((k, n), np.float32, 74, 1)
    C = np.zeros((m, n), np.float32, order="F")
    rc, got, _ = run("T", "N", m, n, k, 1.0, A, k, B, k, 0.0, C)
    assert rc == g.OK
    dA, dB, dP = to_dev(A), to_dev(B), to_dev(C)
    with plain_unsplit():
        assert g.gemm_device("s", "T", "N", m, n, k, 1.0, dA.data_ptr(), k, dB.data_ptr(), k,
                             0.0, dP.data_ptr(), m) == g.OK
    sync()
    truth = orc.dot2gemm("T", "N", m, n, k, 1.0, A, k, B, k, 0.0, C, m)
    mx, fro = rel_errs(got, truth)
    pmx, pfro = rel_errs(from_dev(dP, m), truth)
    assert mx <= pmx and fro <= pfro, (mx, fro, pmx, pfro)
    assert fro < 5e-7, fro


def test_host_and_noalloc_paths(orc):
    m, n, k = 130, 90, 70
    A = orc.uniform((m, k), np.float32, 75, 0)
    B = orc.uniform((n, k), np.float32, 75, 1)
    C = orc.uniform((m, n), np.float32, 75, 2)
    Ch = C.copy(order="F")
    assert g.host_split_gemm("bf16x", "N", "T", m, n, k, 2.0, A, m, B, n, 0.5, Ch, m,
                             g.FP16X3) == g.OK
    model_check(Ch, A, B.T, 2.0, 0.5, C)
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C)
    assert g.sgemm_bf16x_noalloc("N", "T", m, n, k, 2.0, dA.data_ptr(), m, dB.data_ptr(), n, 0.5,
                                 dC.data_ptr(), m, products=g.FP16X3) == g.OK
    sync()
    assert np.array_equal(from_dev(dC, m), Ch)


@pytest.mark.parametrize("products", [6, g.FP16X3])
@pytest.mark.parametrize("tile", [128, 256])
def test_pair_and_single_cta_modes_agree(orc, products, tile):
    """The pair MMAs (cta_group::2, two CTAs per 256-row tile, each holding half
    of the B tile) and one CTA per 128-row tile give the same result bit for
    bit, for even and odd numbers of row tiles."""
    outs = []
    try:
        assert g.tune_param(g.TUNE_TILE_N, tile) == g.OK
        for mode in (1, 2):
            assert g.tune_param(g.TUNE_PAIR_MMA, mode) == g.OK
            res = []
            for m, n, k in ((256, 300, 200), (640, 520, 333)):
                A = orc.uniform((k, m), np.float32, 77, 0)
                B = orc.uniform((k, n), np.float32, 77, 1)
                C = orc.uniform((m + 3, n), np.float32, 77, 2)
                dA, dB, dC = to_dev(A), to_dev(B), to_dev(C)
                assert g.sgemm_bf16x("T", "N", m, n, k, 1.0, dA.data_ptr(), k, dB.data_ptr(), k,
                                     0.5, dC.data_ptr(), m + 3, products=products) == g.OK
                sync()
                got = from_dev(dC, m + 3)
                assert np.array_equal(got[m:], C[m:])
                res.append(got)
            outs.append(res)
    finally:
        g.tune_param(g.TUNE_PAIR_MMA, 0)
        g.tune_param(g.TUNE_TILE_N, 0)
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
    assert g.device_error() == 0


@pytest.mark.parametrize("k", [1027, 1100, 2048, 4500])
@pytest.mark.parametrize("ta,tb,pad", [("T", "N", 0), ("T", "N", 1), ("T", "T", 4), ("N", "N", 1)])
def test_fused_row_split_bitexact(orc, k, ta, tb, pad):
    """k >= 1024 with k-contiguous rows: the fused max pass and split (both
    operands for TN, one for TT / NN; pad 0 or 4: float4 loads, pad 1: scalar
    loads) write the same exponents and terms as the model, including a row of
    NaN, an Inf column, a zero row and rows scaled by 2^40."""
    m, n = 150, 260
    ar, ac = (m, k) if ta == "N" else (k, m)
    br, bc = (k, n) if tb == "N" else (n, k)
    A = orc.uniform((ar + pad, ac), np.float32, 73, 0)
    B = orc.uniform((br + pad, bc), np.float32, 73, 1)
    Av = A[:m, :k] if ta == "N" else A[:k, :m].T  # op(A) and op(B) as views
    Bv = B[:k, :n] if tb == "N" else B[:n, :k].T
    Av[3, :] *= np.float32(2.0 ** 40)
    Av[5, :] = 0.0
    Av[7, 11] = np.nan
    Bv[17, 9] = np.inf
    C = orc.uniform((m, n), np.float32, 73, 2)
    rc, got, ws = run(ta, tb, m, n, k, 1.0, A, ar + pad, B, br + pad, 0.0, C)
    assert rc == g.OK
    Ap, Bp, eA, eB, Mp, Np, Kp = workspace_parts(ws, m, n, k)
    Aop = np.zeros((Mp, Kp), np.float32)
    Aop[:m, :k] = op(A, ta, m, k)
    Bop = np.zeros((Np, Kp), np.float32)
    Bop[:n, :k] = op(B, tb, k, n).T
    # the rows holding op(A) / op(B) (rows past them are left unwritten)
    assert np.array_equal(eA[:m], osp.row_exponents_f32(Aop)[:m])
    assert np.array_equal(eB[:n], osp.row_exponents_f32(Bop)[:n])
    assert np.array_equal(Ap[:m], osp.fp16x3_operand(Aop, True)[:m])
    assert np.array_equal(Bp[:n], osp.fp16x3_operand(Bop, False)[:n])
    assert np.isnan(got[7]).all() and np.isnan(got[:, 9]).all()
    assert g.device_error() == 0
