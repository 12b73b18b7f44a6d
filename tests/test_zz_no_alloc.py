"""gb300_sgemm_bf16x_noalloc: the split SGEMM for callers that may not allocate
device memory (a framework that owns all of it, or a latency-critical path).
Its scratch is the library's fixed 32 MiB device array.  Checked through the
C ABI against the allocating entry point gb300_sgemm_bf16x, on two calls in a
row with different shapes, so that whatever the first call left in the shared
array cannot leak into the second.  Both entry points run the same kernels on
the same inputs, so they must agree bit for bit.  Collected last (test_zz_*)
on purpose."""
import numpy as np
import pytest

import gemm_avx2_gb300 as g
from gpu_util import from_dev, sync, to_dev, torch_cuda

pytestmark = pytest.mark.gpu


def operands(orc, ta, tb, m, n, k, seed):
    ar, ac = (m, k) if ta == "N" else (k, m)
    br, bc = (k, n) if tb == "N" else (n, k)
    A = orc.uniform((ar + 1, ac), np.float32, seed, 0)
    B = orc.uniform((br + 2, bc), np.float32, seed, 1)
    C = orc.uniform((m + 3, n), np.float32, seed, 2)
    return A, B, C, ar + 1, br + 2


def run_both(orc, ta, tb, m, n, k, products, seed):
    A, B, C, lda, ldb = operands(orc, ta, tb, m, n, k, seed)
    dA, dB = to_dev(A), to_dev(B)
    dC_ref, dC_na = to_dev(C), to_dev(C)
    assert g.sgemm_bf16x(ta, tb, m, n, k, 0.75, dA.data_ptr(), lda, dB.data_ptr(), ldb,
                         -0.5, dC_ref.data_ptr(), m + 3, products=products) == g.OK
    assert g.sgemm_bf16x_noalloc(ta, tb, m, n, k, 0.75, dA.data_ptr(), lda, dB.data_ptr(),
                                 ldb, -0.5, dC_na.data_ptr(), m + 3, products=products) == g.OK
    sync()
    ref = from_dev(dC_ref, m + 3)
    got = from_dev(dC_na, m + 3)
    assert np.array_equal(got[:m], ref[:m])
    assert np.array_equal(got[m:], C[m:])  # rows beyond m untouched
    # kernel time-outs of either entry point would show here (0 = none)
    assert g.device_error() == 0


def test_noalloc_matches_allocating_entry_two_calls(orc):
    # first call: a larger problem fills more of the shared scratch
    run_both(orc, "T", "N", 300, 260, 500, 3, 61)
    # second call: smaller, other transposes and products
    run_both(orc, "N", "T", 129, 257, 77, 6, 62)
    # the scaled FP16 form (its scratch also holds the scale exponents)
    run_both(orc, "T", "T", 250, 190, 1100, g.FP16X3, 63)


def test_noalloc_allocates_nothing(orc):
    """After a first call (which sets up the device and loads the kernels), a
    call of a larger shape with the same transposes and form leaves the free
    device memory unchanged: its scratch is the static array, not a buffer
    taken from the driver."""
    torch = torch_cuda()
    shapes = [(200, 180, 300), (640, 700, 900)]
    bufs = []
    for i, (m, n, k) in enumerate(shapes):
        A, B, C, lda, ldb = operands(orc, "N", "N", m, n, k, 70 + i)
        bufs.append((m, n, k, to_dev(A), lda, to_dev(B), ldb, to_dev(C)))
    sync()

    def call(b):
        m, n, k, dA, lda, dB, ldb, dC = b
        assert g.sgemm_bf16x_noalloc("N", "N", m, n, k, 1.0, dA.data_ptr(), lda, dB.data_ptr(),
                                     ldb, 0.0, dC.data_ptr(), m + 3, products=6) == g.OK
        sync()

    call(bufs[0])
    free_before = torch.cuda.mem_get_info()[0]
    call(bufs[1])
    free_after = torch.cuda.mem_get_info()[0]
    assert free_after == free_before, (free_before, free_after)
    assert g.device_error() == 0


def test_noalloc_rejects_problems_beyond_its_scratch():
    # 3xBF16 at 4096^3 needs ~200 MB of scratch: rejected before any GPU work
    assert g.split_workspace_bytes(0, 4096, 4096, 4096, 3) > 32 << 20
    assert g.sgemm_bf16x_noalloc("N", "N", 4096, 4096, 4096, 1.0, 0, 4096, 0, 4096, 0.0, 0,
                                 4096, products=3) == g.ERR_NOALLOC_LIMIT
    assert g.sgemm_bf16x_noalloc("N", "N", 4096, 4096, 4096, 1.0, 0, 4096, 0, 4096, 0.0, 0,
                                 4096, products=g.FP16X3) == g.ERR_NOALLOC_LIMIT
