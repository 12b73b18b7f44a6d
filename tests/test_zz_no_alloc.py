"""gb300_sgemm_bf16x_noalloc: the split SGEMM for callers that may not allocate
device memory (a framework that owns all of it, or a latency-critical path).
Its scratch is the library's fixed 32 MiB device array.  Checked through the
C ABI against the allocating entry point gb300_sgemm_bf16x, on two calls in a
row with different shapes, so that whatever the first call left in the shared
array cannot leak into the second.  Collected last (test_zz_*) on purpose."""
import numpy as np
import pytest

import gemm_avx2_gb300 as g
from gpu_util import from_dev, sync, to_dev

pytestmark = pytest.mark.gpu

# same bound as the 3xBF16 / 6xBF16 accuracy tests (relative Frobenius)
TOL = {3: 2e-5, 6: 1e-6}


def run_both(orc, ta, tb, m, n, k, products, seed):
    ar, ac = (m, k) if ta == "N" else (k, m)
    br, bc = (k, n) if tb == "N" else (n, k)
    A = orc.uniform((ar + 1, ac), np.float32, seed, 0)
    B = orc.uniform((br + 2, bc), np.float32, seed, 1)
    C = orc.uniform((m + 3, n), np.float32, seed, 2)
    dA, dB = to_dev(A), to_dev(B)
    dC_ref, dC_na = to_dev(C), to_dev(C)
    assert g.sgemm_bf16x(ta, tb, m, n, k, 0.75, dA.data_ptr(), ar + 1, dB.data_ptr(), br + 2,
                         -0.5, dC_ref.data_ptr(), m + 3, products=products) == g.OK
    assert g.sgemm_bf16x_noalloc(ta, tb, m, n, k, 0.75, dA.data_ptr(), ar + 1, dB.data_ptr(),
                                 br + 2, -0.5, dC_na.data_ptr(), m + 3, products=products) == g.OK
    sync()
    ref = from_dev(dC_ref, m + 3)
    got = from_dev(dC_na, m + 3)
    d = np.linalg.norm(got[:m].astype(np.float64) - ref[:m]) / np.linalg.norm(ref[:m])
    assert d <= TOL[products], d
    assert np.array_equal(got[m:], C[m:])  # rows beyond m untouched


def test_noalloc_matches_allocating_entry_two_calls(orc):
    # first call: a larger problem fills more of the shared scratch
    run_both(orc, "T", "N", 300, 260, 500, 3, 61)
    # second call: smaller, other transposes and products
    run_both(orc, "N", "T", 129, 257, 77, 6, 62)


def test_noalloc_rejects_problems_beyond_its_scratch():
    # 3xBF16 at 4096^3 needs ~200 MB of scratch: rejected before any GPU work
    assert g.split_workspace_bytes(0, 4096, 4096, 4096, 3) > 32 << 20
    assert g.sgemm_bf16x_noalloc("N", "N", 4096, 4096, 4096, 1.0, 0, 4096, 0, 4096, 0.0, 0,
                                 4096, products=3) == g.ERR_NOALLOC_LIMIT
