"""The host-pointer split forms on problems large enough that the CRT form
stages C in HBM (a side-stream copy beside the prepare), and the two-pass forms
stage A and B: the result equals the device-pointer path bit for bit and the
padding rows of C stay untouched."""
import numpy as np
import pytest

import gemm_avx2_gb300 as g
from gpu_util import from_dev, sync, to_dev, torch_cuda

pytestmark = pytest.mark.gpu


def device_result(form, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, param):
    torch = torch_cuda()
    kind = {"bf16x": 0, "ozaki": 1, "crt": 2}[form]
    need = g.split_workspace_bytes(kind, m, n, k, param)
    ws = torch.empty(need, dtype=torch.uint8, device="cuda")
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C)
    assert g.split_prepare(form, ta, tb, m, n, k, dA.data_ptr(), lda, dB.data_ptr(), ldb, param,
                           ws.data_ptr(), need) == g.OK
    assert g.split_run(form, m, n, k, alpha, beta, dC.data_ptr(), C.shape[0], param,
                       ws.data_ptr(), need) == g.OK
    sync()
    return from_dev(dC, C.shape[0])


@pytest.mark.parametrize("form,param,dt,size,k", [
    ("crt", 16, np.float64, 1500, 1100),
    ("crt", 16, np.float64, 1500, 200),
    ("ozaki", 8, np.float64, 1500, 200),
    ("bf16x", g.FP16X3, np.float32, 2100, 200),
    ("bf16x", 6, np.float32, 2100, 200),
])
def test_staged_host_path_matches_device(orc, form, param, dt, size, k):
    m, n = size, size - 40
    A = orc.uniform((k, m), dt, 81, 0)       # transa = T
    B = orc.uniform((n + 2, k), dt, 81, 1)   # transb = T, ldb = n + 2
    C = orc.uniform((m + 3, n), dt, 81, 2)   # ldc = m + 3
    ref = device_result(form, "T", "T", m, n, k, 1.5, A, k, B, n + 2, 0.5, C, param)
    Ch = C.copy(order="F")
    assert g.host_split_gemm(form, "T", "T", m, n, k, 1.5, A, k, B, n + 2, 0.5, Ch, m + 3,
                             param) == g.OK
    assert np.array_equal(Ch[m:], C[m:])
    assert np.array_equal(Ch[:m], ref[:m])


@pytest.fixture
def host_parts():
    yield lambda v: g.tune_param(g.TUNE_HOST_PARTS, v)
    g.tune_param(g.TUNE_HOST_PARTS, 0)


@pytest.mark.parametrize("parts", [2, 3])
@pytest.mark.parametrize("param", [g.FP16X3, 6, 3])
@pytest.mark.parametrize("ta,tb", [("T", "N"), ("N", "N"), ("N", "T"), ("T", "T")])
def test_pipelined_host_sgemm_matches_device(orc, host_parts, parts, param, ta, tb):
    """The FP32 split form with op(A) in row parts and op(B) in column parts
    (ragged last parts, padded ld): bit for bit the device-pointer result."""
    m, n, k = 700, 900, 300
    ar, ac = (m, k) if ta == "N" else (k, m)
    br, bc = (k, n) if tb == "N" else (n, k)
    A = orc.uniform((ar + 1, ac), np.float32, 82, 0)
    B = orc.uniform((br + 3, bc), np.float32, 82, 1)
    C = orc.uniform((m + 2, n), np.float32, 82, 2)
    ref = device_result("bf16x", ta, tb, m, n, k, 0.75, A, ar + 1, B, br + 3, -1.0, C, param)
    assert host_parts(parts) == g.OK
    Ch = C.copy(order="F")
    assert g.host_split_gemm("bf16x", ta, tb, m, n, k, 0.75, A, ar + 1, B, br + 3, -1.0, Ch, m + 2,
                             param) == g.OK
    assert np.array_equal(Ch[m:], C[m:])
    assert np.array_equal(Ch[:m], ref[:m])
    assert g.device_error() == 0


def test_pipelined_host_sgemm_pinned_buffers(orc, host_parts):
    """Page-locked host buffers take the copy engines: same result bit for bit,
    including beta = 0 with NaN and Inf in C (C * 0 propagates them, as the
    reference's C_MULT_BETA does)."""
    torch = torch_cuda()
    m, n, k = 1100, 800, 1030
    A = orc.uniform((k, m), np.float32, 83, 0)
    B = orc.uniform((k, n), np.float32, 83, 1)
    C = orc.uniform((m, n), np.float32, 83, 2)
    C[5, 700] = np.nan
    C[1000, 3] = -np.inf
    ref = device_result("bf16x", "T", "N", m, n, k, 1.0, A, k, B, k, 0.0, C, g.FP16X3)
    pa, pb, pc = (torch.from_numpy(x.ravel(order="F").copy()).pin_memory() for x in (A, B, C))
    assert host_parts(4) == g.OK
    assert g.core().gb300_host_sgemm_bf16x(b"T", b"N", m, n, k, 1.0, pa.data_ptr(), k,
                                           pb.data_ptr(), k, 0.0, pc.data_ptr(), m,
                                           g.FP16X3) == g.OK
    got = pc.numpy().reshape((n, m)).T
    assert np.isnan(got[5, 700]) and np.isnan(got[1000, 3])
    assert np.array_equal(got, ref, equal_nan=True)


@pytest.mark.parametrize("parts", [2, 3])
@pytest.mark.parametrize("ta,tb", [("T", "N"), ("N", "N"), ("N", "T"), ("T", "T")])
def test_pipelined_host_crt_matches_device(orc, host_parts, parts, ta, tb):
    """The FP64 CRT form in row / column parts: bit for bit the device-pointer
    result (ragged last parts, padded ld, beta != 0)."""
    m, n, k = 700, 900, 300
    ar, ac = (m, k) if ta == "N" else (k, m)
    br, bc = (k, n) if tb == "N" else (n, k)
    A = orc.spread((ar + 1, ac), 84, 0, 1.0)
    B = orc.spread((br + 3, bc), 84, 1, 1.0)
    C = orc.uniform((m + 2, n), np.float64, 84, 2)
    ref = device_result("crt", ta, tb, m, n, k, -0.5, A, ar + 1, B, br + 3, 0.75, C, 15)
    assert host_parts(parts) == g.OK
    Ch = C.copy(order="F")
    assert g.host_split_gemm("crt", ta, tb, m, n, k, -0.5, A, ar + 1, B, br + 3, 0.75, Ch, m + 2,
                             15) == g.OK
    assert np.array_equal(Ch[m:], C[m:])
    assert np.array_equal(Ch[:m], ref[:m])
    assert g.device_error() == 0


def test_pipelined_host_crt_pinned_beta0_nan(orc, host_parts):
    """Copy-engine path of the CRT form, beta = 0 with NaN / Inf in C."""
    torch = torch_cuda()
    m, n, k = 1100, 800, 530
    A = orc.spread((m, k), 85, 0, 1.0)
    B = orc.spread((n, k), 85, 1, 1.0)
    C = orc.uniform((m, n), np.float64, 85, 2)
    C[7, 650] = np.nan
    C[900, 2] = np.inf
    ref = device_result("crt", "N", "T", m, n, k, 1.0, A, m, B, n, 0.0, C, 16)
    pa, pb, pc = (torch.from_numpy(x.ravel(order="F").copy()).pin_memory() for x in (A, B, C))
    assert host_parts(4) == g.OK
    assert g.core().gb300_host_dgemm_ozaki2(b"N", b"T", m, n, k, 1.0, pa.data_ptr(), m,
                                            pb.data_ptr(), n, 0.0, pc.data_ptr(), m, 16) == g.OK
    got = pc.numpy().reshape((n, m)).T
    assert np.isnan(got[7, 650]) and np.isnan(got[900, 2])
    assert np.array_equal(got, ref, equal_nan=True)


@pytest.mark.parametrize("form", ["bf16x", "crt"])
@pytest.mark.parametrize("sign", [1.0, -1.0])
def test_pipelined_host_beta0_c_unread_or_copied(orc, host_parts, form, sign):
    """beta = 0: when every entry of C is finite and non-negative, 0 * C is +0
    everywhere and the pipelined host path zero-fills its device copy of C
    instead of moving C over the link; otherwise it copies C.  Both give the
    device-pointer call's bits, including the sign of zero: with alpha = -1
    and a zero row of op(A), that row of the result is 0 * C + (-0), +0 for
    C >= 0 and -0 for C < 0."""
    torch = torch_cuda()
    m, n, k = 1100, 800, 1030
    dt = np.float32 if form == "bf16x" else np.float64
    A = orc.uniform((k, m), dt, 87, 0)
    B = orc.uniform((k, n), dt, 87, 1)
    A[:, 9] = 0.0                                    # row 9 of op(A) = A^T
    C = (sign * np.abs(orc.uniform((m, n), dt, 87, 2))).astype(dt)
    C[:, 17] = 0.0 * sign                            # exact zeros (+0, or -0 when negative)
    param = g.FP16X3 if form == "bf16x" else 16
    ref = device_result(form, "T", "N", m, n, k, -1.0, A, k, B, k, 0.0, C, param)
    pa, pb, pc = (torch.from_numpy(x.ravel(order="F").copy()).pin_memory() for x in (A, B, C))
    assert host_parts(4) == g.OK
    f = g.core().gb300_host_sgemm_bf16x if form == "bf16x" else g.core().gb300_host_dgemm_ozaki2
    assert f(b"T", b"N", m, n, k, -1.0, pa.data_ptr(), k, pb.data_ptr(), k, 0.0,
             pc.data_ptr(), m, param) == g.OK
    got = pc.numpy().reshape((n, m)).T
    u = np.uint32 if form == "bf16x" else np.uint64
    assert np.array_equal(np.ascontiguousarray(got).view(u), np.ascontiguousarray(ref).view(u))
    assert np.all(np.signbit(got[9]) == (sign < 0)) and not got[9].any()
