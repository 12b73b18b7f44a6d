"""GPU tests of the tensor-core split forms (tcgen05): bit-exact split/slice
kernels against the numpy restatement, and accuracy against the Dot2 oracle."""
import numpy as np
import pytest

import gemm_avx2_gb300 as g
from gpu_util import from_dev, plain_unsplit, sync, to_dev, torch_cuda
from oracle import split as osp
from util import op

pytestmark = pytest.mark.gpu


def ru(x, a):
    return (x + a - 1) // a * a


def ws_tensor(nbytes):
    """A workspace filled with 0xFF bytes (BF16 NaN): padding rows of the split
    operands are never written, and the GEMMs must never read them."""
    torch = torch_cuda()
    return torch.full((nbytes,), 255, dtype=torch.uint8, device="cuda")


def aligned_view(ws, nbytes_needed_from):
    base = ws.data_ptr()
    off = (-base) % 1024
    return off


def rel_errs(x, truth):
    d = np.abs(np.asarray(x, np.float64) - truth)
    fro = np.linalg.norm(d) / np.linalg.norm(truth)
    mx = np.max(d / np.maximum(np.abs(truth), 1e-300))
    return mx, fro


@pytest.mark.parametrize("products", [3, 6])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
def test_bf16x_split_bitexact_and_result(orc, products, ta, tb, tile_n):
    m, n, k = 200, 300, 100
    ar, ac = (m, k) if ta == "N" else (k, m)
    br, bc = (k, n) if tb == "N" else (n, k)
    A = orc.uniform((ar + 1, ac), np.float32, 11, 0)
    B = orc.uniform((br + 3, bc), np.float32, 11, 1)
    C = orc.uniform((m, n), np.float32, 11, 2)
    need = g.split_workspace_bytes(0, m, n, k, products)
    ws = ws_tensor(need)
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C)
    rc = g.sgemm_bf16x(ta, tb, m, n, k, 1.0, dA.data_ptr(), ar + 1, dB.data_ptr(), br + 3, 0.5,
                       dC.data_ptr(), m, products=products, workspace=ws.data_ptr(),
                       workspace_bytes=need)
    assert rc == g.OK
    sync()
    # workspace: A' (Mp x T*Kp) then B' (Np x T*Kp), BF16 terms (T = 2 for P = 3,
    # 3 for P = 6), from the first 1024-aligned byte
    Kp = ru(k, 64)
    Mp, Np = ru(m, 128), ru(n, 256)
    off = aligned_view(ws, need)
    raw = ws.cpu().numpy()[off:]
    kld = (2 if products == 3 else 3) * Kp
    bf = raw[:2 * (Mp + Np) * kld].view(np.uint16).astype(np.uint32) << 16
    vals = bf.view(np.float32)
    Ap = vals[:Mp * kld].reshape(Mp, kld)
    Bp = vals[Mp * kld:(Mp + Np) * kld].reshape(Np, kld)
    Aop = np.zeros((Mp, Kp), np.float32)
    Aop[:m, :k] = op(A, ta, m, k)
    Bop = np.zeros((Np, Kp), np.float32)
    Bop[:n, :k] = op(B, tb, k, n).T
    # the rows holding op(A) / op(B) (rows past them are left unwritten)
    assert np.array_equal(Ap[:m].view(np.uint32),
                          osp.bf16x_operand(Aop, products, True)[:m].view(np.uint32))
    assert np.array_equal(Bp[:n].view(np.uint32),
                          osp.bf16x_operand(Bop, products, False)[:n].view(np.uint32))
    # result vs Dot2 truth
    got = from_dev(dC, m)
    truth = orc.dot2gemm(ta, tb, m, n, k, 1.0, A, ar + 1, B, br + 3, 0.5, C, m)
    mx, fro = rel_errs(got, truth)
    assert fro < (2e-5 if products == 3 else 1e-6), (mx, fro)
    assert g.device_error() == 0


@pytest.mark.parametrize("products", [3, 6])
def test_bf16x_multi_tile_ragged(orc, products, tile_n):
    m, n, k = 300, 520, 333
    A = orc.uniform((k, m), np.float32, 12, 0)   # transa = T
    B = orc.uniform((k, n), np.float32, 12, 1)   # transb = N
    C = orc.uniform((m + 5, n), np.float32, 12, 2)
    dA, dB, dC, dP = to_dev(A), to_dev(B), to_dev(C), to_dev(C)
    assert g.sgemm_bf16x("T", "N", m, n, k, -1.0, dA.data_ptr(), k, dB.data_ptr(), k, 1.0,
                         dC.data_ptr(), m + 5, products=products) == g.OK
    assert g.gemm_device("s", "T", "N", m, n, k, -1.0, dA.data_ptr(), k, dB.data_ptr(), k, 1.0,
                         dP.data_ptr(), m + 5) == g.OK
    sync()
    got = from_dev(dC, m + 5)
    assert np.array_equal(got[m:], C[m:])  # 3 row tiles: the cluster's spare tile writes nothing
    truth = orc.dot2gemm("T", "N", m, n, k, -1.0, A, k, B, k, 1.0, C, m + 5)
    mx, fro = rel_errs(got[:m], truth)
    pmx, pfro = rel_errs(from_dev(dP, m + 5)[:m], truth)
    # 3xBF16 carries ~17 significant bits per operand; 6xBF16 all 24, so its
    # error is of the plain FP32 kernel's order
    if products == 3:
        assert fro < 2e-5, (mx, fro)
    else:
        assert fro < 1e-6 and fro < 4 * pfro, (mx, fro, pfro)
    assert np.array_equal(got[m:], C[m:])


@pytest.mark.parametrize("S", [4, 8])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")])
def test_ozaki_slices_bitexact_and_result(orc, S, ta, tb, tile_n):
    m, n, k = 150, 140, 200
    ar, ac = (m, k) if ta == "N" else (k, m)
    br, bc = (k, n) if tb == "N" else (n, k)
    A = orc.spread((ar + 2, ac), 21, 0, 1.0)
    B = orc.spread((br, bc), 21, 1, 1.0)
    C = orc.uniform((m, n), np.float64, 21, 2)
    need = g.split_workspace_bytes(1, m, n, k, S)
    ws = ws_tensor(need)
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C)
    rc = g.dgemm_ozaki(ta, tb, m, n, k, 1.0, dA.data_ptr(), ar + 2, dB.data_ptr(), br, 0.0,
                       dC.data_ptr(), m, slices=S, workspace=ws.data_ptr(), workspace_bytes=need)
    assert rc == g.OK
    sync()
    Kp, Mp, Np = ru(k, 64), ru(m, 128), ru(n, 256)
    off = aligned_view(ws, need)
    raw = ws.cpu().numpy()[off:]
    bf = raw[:2 * S * (Mp + Np) * Kp].view(np.uint16).astype(np.uint32) << 16
    vals = bf.view(np.float32).astype(np.float64)
    As = vals[:S * Mp * Kp].reshape(S, Mp, Kp)
    Bs = vals[S * Mp * Kp:].reshape(S, Np, Kp)
    Aop = op(A, ta, m, k)
    Bop = op(B, tb, k, n)
    sa, E = osp.ozaki_slices(Aop, S)
    sb, F = osp.ozaki_slices(Bop.T, S)
    for s in range(S):
        assert np.array_equal(As[s, :m, :k], sa[s])
        assert np.array_equal(Bs[s, :n, :k], sb[s])
        # K columns past k of the rows holding data are zeros; rows past m are
        # left unwritten (the GEMM's maps end at m)
        assert not As[s, :m, k:].any() and not Bs[s, :n, k:].any()
    got = from_dev(dC, m)
    model = osp.ozaki_gemm_model(Aop, Bop, S)
    # the kernel's integer sums are exact, so it matches the model up to the
    # FP64 rounding of the final alpha/beta update
    assert np.allclose(got, model, rtol=4e-16, atol=0), np.abs(got - model).max()
    truth = orc.dot2gemm(ta, tb, m, n, k, 1.0, A, ar + 2, B, br, 0.0, C, m)
    mx, fro = rel_errs(got, truth)
    assert fro < (2.0 ** (-7 * S + 12)), (mx, fro)
    assert g.device_error() == 0


@pytest.mark.parametrize("S", [8, 12])
@pytest.mark.parametrize("ta", ["N", "T"])
def test_ozaki_slices_extreme_exponents(orc, S, ta):
    """Digits of subnormals, of rows spanning ~600 decades and of zero rows:
    the slice kernel reads them from the significand bits and must agree with
    the FP64 trunc-by-128 recurrence of the oracle."""
    m, n, k = 70, 40, 90
    rng = np.random.default_rng(5)
    Aop = rng.standard_normal((m, k)) * np.exp2(rng.integers(-40, 40, (m, k)))
    Aop[0] = rng.standard_normal(k) * 5e-324 * rng.integers(1, 2 ** 20, k)   # subnormal row
    Aop[1, :] = 0.0
    Aop[2] = rng.standard_normal(k) * np.exp2(rng.integers(-1000, 1000, k))   # huge spread
    Aop[3, ::3] = 5e-324                                                     # smallest subnormal
    Aop[4] = np.exp2(rng.integers(-1074, -1022, k)) * np.sign(rng.standard_normal(k))
    Aop[5, 0] = np.finfo(np.float64).max
    Aop[6] = -np.exp2(-7.0 * np.arange(k) / 3.0)                             # digit boundaries
    A = np.asfortranarray(Aop if ta == "N" else Aop.T)
    B = orc.uniform((k, n), np.float64, 22, 1)
    need = g.split_workspace_bytes(1, m, n, k, S)
    ws = ws_tensor(need)
    dA, dB = to_dev(A), to_dev(B)
    dC = to_dev(np.zeros((m, n), order="F"))
    rc = g.dgemm_ozaki(ta, "N", m, n, k, 1.0, dA.data_ptr(), A.shape[0], dB.data_ptr(), k, 0.0,
                       dC.data_ptr(), m, slices=S, workspace=ws.data_ptr(), workspace_bytes=need)
    assert rc == g.OK
    sync()
    Kp, Mp = ru(k, 64), ru(m, 128)
    raw = ws.cpu().numpy()[aligned_view(ws, need):]
    bf = raw[:2 * S * Mp * Kp].view(np.uint16).astype(np.uint32) << 16
    As = bf.view(np.float32).astype(np.float64).reshape(S, Mp, Kp)
    sa, _ = osp.ozaki_slices(Aop, S)
    for s in range(S):
        assert np.array_equal(As[s, :m, :k], sa[s]), s
    assert g.device_error() == 0


def test_ozaki_odd_row_tiles(orc, tile_n, cluster_mode):
    """3 row tiles, in each cluster mode: with pair MMAs the spare fourth tile
    runs through the pipeline but must write neither the FP64 scratch nor C."""
    m, n, k = 300, 270, 200
    A = orc.spread((m, k), 23, 0, 1.0)
    B = orc.spread((k, n), 23, 1, 1.0)
    C = orc.uniform((m + 3, n), np.float64, 23, 2)
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C)
    assert g.dgemm_ozaki("N", "N", m, n, k, 1.0, dA.data_ptr(), m, dB.data_ptr(), k, 0.5,
                         dC.data_ptr(), m + 3, slices=8) == g.OK
    sync()
    got = from_dev(dC, m + 3)
    assert np.array_equal(got[m:], C[m:])
    model = osp.ozaki_gemm_model(A, B, 8)
    assert np.allclose(got[:m], model + 0.5 * C[:m], rtol=4e-16, atol=1e-300)
    assert g.device_error() == 0


def test_ozaki_vs_plain_accuracy(orc):
    """At S = 8 the Ozaki form is as accurate as the plain FP64 kernel (uniform data)."""
    m = n = 384
    k = 2048
    A = orc.uniform((m, k), np.float64, 31, 0)
    B = orc.uniform((n, k), np.float64, 31, 1)
    C = orc.uniform((m, n), np.float64, 31, 2)
    dA, dB = to_dev(A), to_dev(B)
    dC1, dC2 = to_dev(C), to_dev(C)
    assert g.dgemm_ozaki("N", "T", m, n, k, 1.0, dA.data_ptr(), m, dB.data_ptr(), n, 1.0,
                         dC1.data_ptr(), m, slices=8) == g.OK
    with plain_unsplit():
        assert g.gemm_device("d", "N", "T", m, n, k, 1.0, dA.data_ptr(), m, dB.data_ptr(), n,
                             1.0, dC2.data_ptr(), m) == g.OK
    sync()
    truth = orc.dot2gemm("N", "T", m, n, k, 1.0, A, m, B, n, 1.0, C, m)
    e_oz = rel_errs(from_dev(dC1, m), truth)
    e_pl = rel_errs(from_dev(dC2, m), truth)
    assert e_oz[1] <= 4 * e_pl[1] + 1e-16, (e_oz, e_pl)


def test_ozaki_edge_semantics(orc):
    m, n, k = 70, 50, 30
    A = orc.uniform((m, k), np.float64, 41, 0)
    B = orc.uniform((k, n), np.float64, 41, 1)
    C = np.ones((m, n), order="F")
    C[2, 3] = np.nan
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C)
    # alpha == 0 -> beta scaling only
    assert g.dgemm_ozaki("N", "N", m, n, k, 0.0, dA.data_ptr(), m, dB.data_ptr(), k, 2.0,
                         dC.data_ptr(), m, slices=6) == g.OK
    sync()
    got = from_dev(dC, m)
    assert np.isnan(got[2, 3]) and np.all(got[~np.isnan(got)] == 2.0)
    # a NaN in A's row 5 poisons C's row 5
    A2 = A.copy(order="F")
    A2[5, 7] = np.nan
    dA2, dC = to_dev(A2), to_dev(np.zeros((m, n), order="F"))
    assert g.dgemm_ozaki("N", "N", m, n, k, 1.0, dA2.data_ptr(), m, dB.data_ptr(), k, 0.0,
                         dC.data_ptr(), m, slices=6) == g.OK
    sync()
    got = from_dev(dC, m)
    assert np.isnan(got[5]).all() and np.isfinite(np.delete(got, 5, axis=0)).all()


def test_ozaki_exact_at_chunk_bound(orc):
    """Worst case for the exact chunks: every slice digit is 127, so a 1024-step
    chunk sums to 1024*127^2 (just below 2^24) and the int32 running sums grow
    the most.  The kernel must reproduce the integer model bit for bit."""
    S = 4
    m, n, k = 130, 140, 3000
    v = 1.0 - 2.0 ** (-7 * S - 3)  # all S digits 127 after scaling by 2^0
    A = np.full((m, k), v, order="F")
    B = np.full((k, n), -v, order="F")
    A[1, 5] = -v
    C = np.zeros((m, n), order="F")
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C)
    assert g.dgemm_ozaki("N", "N", m, n, k, 1.0, dA.data_ptr(), m, dB.data_ptr(), k, 0.0,
                         dC.data_ptr(), m, slices=S) == g.OK
    sync()
    got = from_dev(dC, m)
    sa, _ = osp.ozaki_slices(A, S)
    assert (sa[0] == 127).sum() > 0.99 * m * k
    model = osp.ozaki_gemm_model(A, B, S)
    assert np.array_equal(got, model), np.abs(got - model).max()
    assert g.device_error() == 0


@pytest.mark.parametrize("form", ["bf16x", "ozaki"])
def test_host_pointer_split_forms(orc, form):
    """gb300_host_sgemm_bf16x / gb300_host_dgemm_ozaki on pageable host arrays with
    padded leading dimensions: results within the split forms' bounds and the
    ldc padding rows untouched (the kernels access host memory directly on
    coherent CPU-GPU systems, or stage it otherwise)."""
    dt = np.float32 if form == "bf16x" else np.float64
    m, n, k = 333, 290, 517
    A = orc.uniform((k + 3, m), dt, 71, 0)        # transa = T, lda = k + 3
    B = orc.uniform((n + 1, k), dt, 71, 1)        # transb = T, ldb = n + 1
    C = orc.uniform((m + 2, n), dt, 71, 2)
    C0 = C.copy(order="F")
    param = 6 if form == "bf16x" else 8
    assert g.host_split_gemm(form, "T", "T", m, n, k, 0.75, A, k + 3, B, n + 1, -1.25, C, m + 2,
                             param) == g.OK
    truth = orc.dot2gemm("T", "T", m, n, k, 0.75, A, k + 3, B, n + 1, -1.25, C0, m + 2)
    d = np.linalg.norm(C[:m].astype(np.float64) - truth) / np.linalg.norm(truth)
    assert d < (1e-6 if form == "bf16x" else 1e-15), d
    assert np.array_equal(C[m:], C0[m:])


def staged_c_runs(orc, m, n, k, products, beta, seed):
    """C = -op(A) op(B) + beta C with pair MMAs / aligned ldc, one CTA per tile /
    aligned ldc and pair MMAs / odd ldc (256-wide tiles); the m x n results."""
    A = orc.uniform((m, k), np.float32, seed, 0)
    B = orc.uniform((n, k), np.float32, seed, 1)
    C0 = orc.uniform((m, n), np.float32, seed, 2)
    C0[7, 3], C0[250, 400], C0[0, n - 1] = np.nan, np.inf, -0.0
    dA, dB = to_dev(A), to_dev(B)
    ld4 = ru(m, 4) + 4
    outs = []
    try:
        assert g.tune_param(g.TUNE_TILE_N, 256) == g.OK
        for mode, ldc in ((1, ld4), (2, ld4), (1, ld4 - 1)):
            assert g.tune_param(g.TUNE_PAIR_MMA, mode) == g.OK
            C = np.full((ldc, n), 3.25, np.float32, order="F")
            C[:m] = C0
            dC = to_dev(C)
            assert g.sgemm_bf16x("N", "T", m, n, k, -1.0, dA.data_ptr(), m, dB.data_ptr(), n, beta,
                                 dC.data_ptr(), ldc, products=products) == g.OK
            sync()
            got = from_dev(dC, ldc)
            assert np.all(got[m:] == 3.25)
            outs.append(got[:m])
            del dC
    finally:
        g.tune_param(g.TUNE_PAIR_MMA, 0)
        g.tune_param(g.TUNE_TILE_N, 0)
    return outs


@pytest.mark.parametrize("products,k", [(6, 256), (3, 100), (g.FP16X3, 256), (6, 700)])
@pytest.mark.parametrize("beta", [1.0, 0.0, 0.5])
def test_bf16x_staged_c_bitexact(orc, products, k, beta):
    """Short K (at most 48 K blocks a tile) with pair MMAs, 256-wide tiles and a
    C whose base and column stride are 16-byte multiples: the epilogue reads C
    from shared memory, loaded by TMA.  Its results equal bit for bit those of
    the kernels that read C with plain loads (one CTA per tile; or an odd ldc,
    which no tensor map can describe), NaN and Inf entries of C included, and
    the rows of C past m stay untouched.  k = 700 with 6 products (66 K blocks),
    and m = 298, take the plain-load path in every mode."""
    outs = staged_c_runs(orc, 300, 520, k, products, beta, 31)
    for o in outs[1:]:
        assert np.array_equal(outs[0].view(np.uint32), o.view(np.uint32))
    # m = 298: rows not a multiple of 16 bytes take the plain-load epilogue
    # (a TMA store of the last row tile would write 2 rows of the ld padding)
    outs = staged_c_runs(orc, 298, 520, k, products, beta, 33)
    for o in outs[1:]:
        assert np.array_equal(outs[0].view(np.uint32), o.view(np.uint32))
    assert np.isnan(outs[0][7, 3])   # beta * NaN, whatever beta
    assert g.device_error() == 0


@pytest.mark.parametrize("products", [6, g.FP16X3])
def test_bf16x_staged_c_many_tiles(orc, products):
    """The staged-C epilogue over about four tiles per CTA (4100 x 3900, k = 256:
    272 row-tile pairs x column tiles on 74 clusters), where each C slot is
    loaded, read and released again tile after tile: bit-identical to the
    plain-load kernels."""
    outs = staged_c_runs(orc, 4100, 3900, 256, products, 1.0, 32)
    for o in outs[1:]:
        assert np.array_equal(outs[0].view(np.uint32), o.view(np.uint32))
    assert g.device_error() == 0
