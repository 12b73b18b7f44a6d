"""Failure detection on the GPU without a GPU fault: a kernel's bounded wait on
an mbarrier that nothing arrives on gives up, records an error code and
returns; the host reads GB300_ERR_TIMEOUT and the context stays usable."""
import numpy as np
import pytest

import gemm_avx2_gb300 as g
from gpu_util import from_dev, sync, to_dev

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_survives():
    g.device_error(clear=True)
    assert g.selftest_wait_timeout(2048) == g.ERR_TIMEOUT
    assert g.device_error() == 0x10
    g.device_error(clear=True)
    assert g.device_error() == 0
    # the context is still usable: a normal GEMM afterwards is correct
    A = np.ones((64, 32), order="F")
    B = np.ones((32, 48), order="F")
    C = np.zeros((64, 48), order="F")
    dA, dB, dC = to_dev(A), to_dev(B), to_dev(C)
    assert g.gemm_device("d", "N", "N", 64, 48, 32, 1.0, dA.data_ptr(), 64, dB.data_ptr(), 32,
                         0.0, dC.data_ptr(), 64) == g.OK
    sync()
    assert np.all(from_dev(dC, 64) == 32.0)
    assert g.device_error() == 0
