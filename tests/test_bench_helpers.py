"""CPU tests of bench.py's helpers: pinned layout names, the scaled FP16
prepare's launch count by layout, and the traffic lookup of tuned names."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
import gemm_avx2_gb300 as g  # noqa: E402


@pytest.fixture
def knobs():
    yield
    for knob in (g.TUNE_BF16X_CHUNK, g.TUNE_TILE_N, g.TUNE_PAIR_MMA):
        g.tune_param(knob, 0)


def test_parse_form_names(knobs):
    assert bench.parse_form("crt_n15") == ("crt", 15)
    assert bench.parse_form("ozaki_s8") == ("ozaki", 8)
    assert bench.parse_form("bf16x6") == ("bf16x", 6)
    assert bench.parse_form("fp16x3") == ("bf16x", g.FP16X3)
    # a tuned name pins chunk, tile width and cluster mode as knobs
    assert bench.parse_form("tuned:fp16x3_c8_t256_pair") == ("bf16x", g.FP16X3)
    assert bench.parse_form("bf16x6_c4_t128_cta") == ("bf16x", 6)
    assert bench.parse_form("crt_n15_cta") == ("crt", 15)
    assert bench.parse_form("ozaki_s8_pair_t128") == ("ozaki", 8)
    with pytest.raises(SystemExit):
        bench.parse_form("bf16x6_mc")  # the multicast mode no longer exists
    with pytest.raises(SystemExit):
        bench.parse_form("fp16x3_q9")
    with pytest.raises(SystemExit):
        bench.parse_form("nonsense")


def test_fp16x3_prepare_launches():
    # TN: both operands k-contiguous -> one fused launch
    assert bench.fp16x3_prepare_launches("T", "N", 8192) == 1
    # one k-contiguous operand: fused launch + max pass + tile split
    assert bench.fp16x3_prepare_launches("T", "T", 8192) == 3
    assert bench.fp16x3_prepare_launches("N", "N", 16384) == 3
    # none, or k outside [1024, 16384]: max pass + tile split
    assert bench.fp16x3_prepare_launches("N", "T", 8192) == 2
    assert bench.fp16x3_prepare_launches("T", "N", 1000) == 2
    assert bench.fp16x3_prepare_launches("T", "N", 16385) == 2


def test_traffic_lookup_strips_tuned_prefix():
    a = bench.traffic_from_profile("sgemm_tn_8192", "tuned:fp16x3_c8_t256_pair")
    b = bench.traffic_from_profile("sgemm_tn_8192", "fp16x3_c8_t256_pair")
    assert a == b and a > 0
    assert bench.traffic_from_profile("sgemm_tn_8192", "no_such_form") is None
