"""GPU tests of complex GEMM (CGEMM / ZGEMM, 4M / 3M / split methods) against
the complex oracle, through the C ABI: device pointers, caller workspaces, the
host-pointer path and the ZGEMM.so / CGEMM.so drop-in symbols."""
import numpy as np
import pytest

import gemm_avx2_gb300 as g
import oracle
from gpu_util import from_dev, sync, to_dev, torch_cuda
from util import U32, U64, cgemm_bound, check_close_c, cop, ctrans, l1

pytestmark = pytest.mark.gpu

TRANS = ["N", "T", "C", "R"]
DT = {"z": np.complex128, "c": np.complex64}
U = {"z": U64, "c": U32}


def inputs(p, ta, tb, m, n, k, seed, pad=0):
    dt = DT[p]
    ar, ac = (k, m) if ctrans(ta) else (m, k)
    br, bc = (n, k) if ctrans(tb) else (k, n)
    A = oracle.cuniform((ar + pad, ac), dt, seed, 0)
    B = oracle.cuniform((br + pad, bc), dt, seed, 1)
    C = oracle.cuniform((m + pad, n), dt, seed, 2)
    return A, B, C


def run_device(p, ta, tb, m, n, k, alpha, A, B, beta, C, method, param=0, ws=None, wsb=0):
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C)
    rc = g.complex_device(p, ta, tb, m, n, k, alpha, dA.data_ptr(), A.shape[0], dB.data_ptr(),
                          B.shape[0], beta, dC.data_ptr(), C.shape[0], method=method, param=param,
                          workspace=ws, workspace_bytes=wsb)
    sync()
    return rc, from_dev(dC, C.shape[0])


def truth_of(ta, tb, m, n, k, alpha, A, B, beta, C):
    return oracle.zgemm_dot2(ta, tb, m, n, k, alpha, A, A.shape[0], B, B.shape[0], beta, C,
                             C.shape[0])


@pytest.mark.parametrize("p", ["z", "c"])
@pytest.mark.parametrize("ta", TRANS)
@pytest.mark.parametrize("tb", TRANS)
def test_4m_all_trans(p, ta, tb):
    m, n, k = 70, 51, 45
    A, B, C = inputs(p, ta, tb, m, n, k, 31, pad=3)
    al, be = 0.75 - 0.5j, -0.5 + 1.25j
    rc, got = run_device(p, ta, tb, m, n, k, al, A, B, be, C, g.CPLX_4M)
    assert rc == g.OK
    truth = truth_of(ta, tb, m, n, k, al, A, B, be, C)
    bound = cgemm_bound(cop(A, ta, m, k), cop(B, tb, k, n), C[:m], al, be, k, U[p])
    check_close_c(got[:m], truth, bound)
    assert np.array_equal(got[m:], C[m:])  # rows past m untouched
    assert g.device_error() == 0


@pytest.mark.parametrize("p", ["z", "c"])
@pytest.mark.parametrize("al,be", [(2.0, 0.5), (1.0, 0.0), (0.5j, 1.0), (-1.0, 0.25 - 0.5j)])
def test_4m_real_and_complex_scalars(p, al, be):
    m, n, k = 129, 130, 67
    A, B, C = inputs(p, "N", "N", m, n, k, 32)
    rc, got = run_device(p, "N", "N", m, n, k, al, A, B, be, C, g.CPLX_4M)
    assert rc == g.OK
    truth = truth_of("N", "N", m, n, k, al, A, B, be, C)
    check_close_c(got, truth, cgemm_bound(cop(A, "N", m, k), cop(B, "N", k, n), C, al, be, k,
                                          U[p]))


@pytest.mark.parametrize("p", ["z", "c"])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("C", "T"), ("R", "C"), ("T", "R")])
def test_3m(p, ta, tb):
    m, n, k = 97, 66, 80
    A, B, C = inputs(p, ta, tb, m, n, k, 33, pad=1)
    al, be = -0.5 + 0.75j, 0.5 - 0.25j
    rc, got = run_device(p, ta, tb, m, n, k, al, A, B, be, C, g.CPLX_3M)
    assert rc == g.OK
    truth = truth_of(ta, tb, m, n, k, al, A, B, be, C)
    # three real products and their differences: three times the 4M bound
    bound = cgemm_bound(cop(A, ta, m, k), cop(B, tb, k, n), C[:m], al, be, k, U[p], factor=3.0)
    check_close_c(got[:m], truth, bound)
    assert np.array_equal(got[m:], C[m:])


def rel_fro(got, truth):
    return float(np.linalg.norm(got - truth) / np.linalg.norm(truth))


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("C", "N"), ("N", "C"), ("T", "R")])
@pytest.mark.parametrize("products", [3, 6])
def test_split_cgemm_bf16x(ta, tb, products):
    m, n, k = 200, 140, 150
    A, B, C = inputs("c", ta, tb, m, n, k, 34)
    al, be = 1.0 - 0.5j, 0.5
    rc, got = run_device("c", ta, tb, m, n, k, al, A, B, be, C, g.CPLX_SPLIT, param=products)
    assert rc == g.OK
    truth = truth_of(ta, tb, m, n, k, al, A, B, be, C)
    if products == 6:
        # 6xBF16 is at least as accurate as the plain FP32 kernel
        bound = cgemm_bound(cop(A, ta, m, k), cop(B, tb, k, n), C, al, be, k, U32)
        check_close_c(got, truth, bound)
    else:
        assert rel_fro(got, truth) < 2e-5


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("C", "N"), ("T", "C"), ("R", "R")])
@pytest.mark.parametrize("S", [6, 8])
def test_split_zgemm_ozaki(ta, tb, S):
    m, n, k = 150, 90, 120
    A, B, C = inputs("z", ta, tb, m, n, k, 35)
    al, be = 0.5 + 0.5j, -1.0
    rc, got = run_device("z", ta, tb, m, n, k, al, A, B, be, C, g.CPLX_SPLIT, param=S)
    assert rc == g.OK
    truth = truth_of(ta, tb, m, n, k, al, A, B, be, C)
    assert rel_fro(got, truth) < 2.0 ** (-7 * S + 12), rel_fro(got, truth)
    if S == 8:  # as accurate as plain FP64 on these inputs
        bound = cgemm_bound(cop(A, ta, m, k), cop(B, tb, k, n), C, al, be, k, U64)
        check_close_c(got, truth, bound)


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("C", "N"), ("T", "C"), ("R", "R")])
@pytest.mark.parametrize("N", [14, 16])
def test_crt_zgemm(ta, tb, N):
    m, n, k = 150, 90, 120
    A, B, C = inputs("z", ta, tb, m, n, k, 43)
    al, be = 0.5 + 0.5j, -1.0
    rc, got = run_device("z", ta, tb, m, n, k, al, A, B, be, C, g.CPLX_CRT, param=N)
    assert rc == g.OK
    truth = truth_of(ta, tb, m, n, k, al, A, B, be, C)
    if N == 16:  # as accurate as plain FP64 on these inputs
        bound = cgemm_bound(cop(A, ta, m, k), cop(B, tb, k, n), C, al, be, k, U64)
        check_close_c(got, truth, bound)
    else:
        assert rel_fro(got, truth) < 1e-13


@pytest.mark.parametrize("p", ["z", "c"])
@pytest.mark.parametrize("method", [g.CPLX_4M, g.CPLX_3M, g.CPLX_SPLIT])
def test_k0_and_alpha0_scale_c_only(p, method):
    m, n, k = 33, 17, 9
    A, B, C = inputs(p, "N", "N", m, n, k, 36)
    be = 0.5 - 2.0j
    dC = to_dev(C)
    # alpha == 0: A and B are never read (null pointers)
    rc = g.complex_device(p, "N", "N", m, n, k, 0.0, 0, m, 0, k, be, dC.data_ptr(), m,
                          method=method)
    assert rc == g.OK
    # k == 0
    rc = g.complex_device(p, "N", "N", m, n, 0, 1.0 + 1j, 0, m, 0, 1, be, dC.data_ptr(), m,
                          method=method)
    assert rc == g.OK
    sync()
    want = be * be * C.astype(np.complex128)
    # two complex multiplies, each within a few units of |beta|_1 |c|_1 per part
    check_close_c(from_dev(dC, m), want, 8 * U[p] * l1(be) ** 2 * l1(C) + 1e-30)


@pytest.mark.parametrize("p", ["z", "c"])
@pytest.mark.parametrize("method", [g.CPLX_4M, g.CPLX_3M])
def test_beta0_propagates_nan(p, method):
    m, n, k = 20, 10, 5
    A, B, C = inputs(p, "N", "N", m, n, k, 37)
    C[3, 4] = np.nan
    rc, got = run_device(p, "N", "N", m, n, k, 1.0, A, B, 0.0, C, method)
    assert rc == g.OK
    assert np.isnan(got[3, 4]) and np.isfinite(np.delete(got.ravel(order="F"), 4 * m + 3)).all()


@pytest.mark.parametrize("p", ["z", "c"])
def test_misaligned_base_and_odd_ld(p):
    """A and B one complex element past an aligned base, ldb odd: for CGEMM the
    embedded B view (real ld 2*ldb) is then not TMA-aligned and the plain kernel
    takes its fallback loads."""
    m, n, k = 45, 38, 29
    A, _, C = inputs(p, "N", "N", m, n, k, 38)
    Bp = oracle.cuniform((k + 2, n), DT[p], 38, 4)  # ldb = k + 2 = 31
    dA = to_dev(np.vstack([np.zeros((1, k), DT[p]), A]))
    dB = to_dev(np.vstack([np.zeros((1, n), DT[p]), Bp]))
    dC = to_dev(C)
    esz = np.dtype(DT[p]).itemsize
    rc = g.complex_device(p, "N", "N", m, n, k, 1.0 - 1j, dA.data_ptr() + esz, m + 1,
                          dB.data_ptr() + esz, k + 3, 0.5, dC.data_ptr(), m)
    assert rc == g.OK
    sync()
    got = from_dev(dC, m)
    truth = truth_of("N", "N", m, n, k, 1.0 - 1j, A, Bp, 0.5, C)
    check_close_c(got, truth, cgemm_bound(A, Bp[:k], C, 1.0 - 1j, 0.5, k, U[p]))


@pytest.mark.parametrize("p", ["z", "c"])
@pytest.mark.parametrize("method", [g.CPLX_4M, g.CPLX_3M, g.CPLX_SPLIT])
def test_caller_workspace(p, method):
    torch = torch_cuda()
    m, n, k = 64, 48, 40
    A, B, C = inputs(p, "C", "T", m, n, k, 39)
    param = (6 if p == "c" else 8) if method == g.CPLX_SPLIT else 0
    need = g.complex_workspace_bytes(p, method, "T", m, n, k, param)
    assert need > 0
    small = torch.zeros(need - 1, dtype=torch.uint8, device="cuda")
    rc, _ = run_device(p, "C", "T", m, n, k, 1.0, A, B, 0.0, C, method, param,
                       ws=small.data_ptr(), wsb=need - 1)
    assert rc == g.ERR_WORKSPACE
    ws = torch.zeros(need, dtype=torch.uint8, device="cuda")
    rc, got = run_device(p, "C", "T", m, n, k, 1.0, A, B, 0.0, C, method, param,
                         ws=ws.data_ptr(), wsb=need)
    assert rc == g.OK
    truth = truth_of("C", "T", m, n, k, 1.0, A, B, 0.0, C)
    fac = 3.0 if method == g.CPLX_3M else 1.0
    check_close_c(got, truth, cgemm_bound(cop(A, "C", m, k), cop(B, "T", k, n), C, 1.0, 0.0, k,
                                          U[p], factor=fac))


@pytest.mark.parametrize("p", ["z", "c"])
@pytest.mark.parametrize("method", [g.CPLX_4M, g.CPLX_3M, g.CPLX_SPLIT])
def test_host_path(p, method):
    m, n, k = 77, 41, 56
    A, B, C = inputs(p, "T", "N", m, n, k, 40, pad=2)
    al, be = 0.25 + 1j, 1.0
    Cg = C.copy(order="F")
    rc = g.host_complex(p, "T", "N", m, n, k, al, A, A.shape[0], B, B.shape[0], be, Cg,
                        C.shape[0], method=method, param=(6 if p == "c" else 8)
                        if method == g.CPLX_SPLIT else 0)
    assert rc == g.OK
    truth = truth_of("T", "N", m, n, k, al, A, B, be, C)
    fac = 3.0 if method == g.CPLX_3M else 1.0
    check_close_c(Cg[:m], truth, cgemm_bound(cop(A, "T", m, k), cop(B, "N", k, n), C[:m], al, be,
                                             k, U[p], factor=fac))
    assert np.array_equal(Cg[m:], C[m:])


@pytest.mark.parametrize("p", ["z", "c"])
@pytest.mark.parametrize("three_m", [False, True])
def test_dropin_symbols(p, three_m):
    m, n, k = 50, 60, 70
    A, B, C = inputs(p, "C", "C", m, n, k, 41)
    al, be = 1.5 - 0.5j, 0.0 + 0.5j
    Cg = C.copy(order="F")
    f = g.zgemm if p == "z" else g.cgemm
    f("C", "C", m, n, k, al, A, A.shape[0], B, B.shape[0], be, Cg, m, method3m=three_m)
    truth = truth_of("C", "C", m, n, k, al, A, B, be, C)
    check_close_c(Cg, truth, cgemm_bound(cop(A, "C", m, k), cop(B, "C", k, n), C, al, be, k, U[p],
                                         factor=3.0 if three_m else 1.0))


@pytest.mark.parametrize("p,method", [("z", g.CPLX_4M), ("z", g.CPLX_SPLIT), ("z", g.CPLX_CRT),
                                      ("c", g.CPLX_4M), ("c", g.CPLX_SPLIT)])
def test_large_sampled(p, method):
    """1024^3 against sampled ground-truth entries."""
    m = n = k = 1024
    A, B, C = inputs(p, "N", "C", m, n, k, 42)
    al, be = 1.0, 1.0
    rc, got = run_device(p, "N", "C", m, n, k, al, A, B, be, C, method,
                         param=(6 if p == "c" else 8) if method == g.CPLX_SPLIT else 0)
    assert rc == g.OK
    rng = np.random.default_rng(0)
    rows, cols = rng.integers(0, m, 256), rng.integers(0, n, 256)
    t = oracle.zgemm_dot2_sampled("N", "C", k, al, A, m, B, n, be, C, m, rows, cols)
    Aop, Bop = cop(A, "N", m, k), cop(B, "C", k, n)
    mag = (np.abs(Aop.real) + np.abs(Aop.imag))[rows] * 1.0
    bsum = (np.abs(Bop.real) + np.abs(Bop.imag))[:, cols]
    bound = (2 * k + 8) * U[p] * (np.einsum("ij,ji->i", mag, bsum) + np.abs(C[rows, cols]) * 2)
    d = got[rows, cols] - t
    assert (np.abs(d.real) <= bound).all() and (np.abs(d.imag) <= bound).all()
