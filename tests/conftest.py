import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def orc():
    """The CPU oracle (test infrastructure), built on first use."""
    import oracle

    if not os.path.exists(os.path.join(ROOT, "oracle", "liborc.so")):
        oracle.build()
    return oracle


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    return np.load(os.path.join(ROOT, "tests", "golden", "golden.npz"))


@pytest.fixture(params=[128, 256], ids=["tile128", "tile256"])
def tile_n(request):
    """Runs a split-form test with each output tile width of the tensor-core
    GEMMs (the library picks one by shape otherwise)."""
    import gemm_avx2_gb300 as g

    assert g.tune_param(g.TUNE_TILE_N, request.param) == g.OK
    yield request.param
    assert g.tune_param(g.TUNE_TILE_N, 0) == g.OK


@pytest.fixture(params=[1, 2], ids=["pair", "cta"])
def cluster_mode(request):
    """Runs a split-form test with each cluster mode of the tensor-core GEMMs:
    pair MMAs on 2-CTA clusters (1) and one CTA per tile (2)."""
    import gemm_avx2_gb300 as g

    assert g.tune_param(g.TUNE_PAIR_MMA, request.param) == g.OK
    yield request.param
    assert g.tune_param(g.TUNE_PAIR_MMA, 0) == g.OK
