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
