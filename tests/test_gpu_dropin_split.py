"""The drop-in symbols with GB300_DROPIN_FORM=split: dgemm_ / sgemm_ (and the
complex ones) run the tensor-core forms for large problems, at no worse error
than the plain kernels, several times faster.  The variable is read once per
process, so each setting runs in a child process."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys, time
import numpy as np
sys.path.insert(0, %(root)r)
import gemm_avx2_gb300 as g
import oracle

out = {}
rng = np.random.default_rng(0)
for p, dt in (("d", np.float64), ("s", np.float32)):
    m = n = k = 2048
    A = oracle.uniform((m, k), dt, 61, 0)
    B = oracle.uniform((k, n), dt, 61, 1)
    C0 = oracle.uniform((m, n), dt, 61, 2)
    f = g.dgemm if p == "d" else g.sgemm
    C = C0.copy(order="F")
    f("N", "N", m, n, k, 1.0, A, m, B, k, 0.5, C, m)          # warm-up / accuracy
    rows, cols = rng.integers(0, m, 512), rng.integers(0, n, 512)
    t = oracle.dot2gemm_sampled("N", "N", m, n, k, 1.0, A, m, B, k, 0.5, C0, m, rows, cols)
    d = np.abs(C[rows, cols].astype(np.float64) - t)
    out[p + "_err"] = float(np.linalg.norm(d) / np.linalg.norm(t))
    t0 = time.perf_counter()
    for _ in range(3):
        f("N", "N", m, n, k, 1.0, A, m, B, k, 0.5, C, m)
    out[p + "_ms"] = (time.perf_counter() - t0) / 3 * 1e3
m = n = k = 768
A = oracle.cuniform((m, k), np.complex128, 62, 0)
B = oracle.cuniform((k, n), np.complex128, 62, 1)
C0 = oracle.cuniform((m, n), np.complex128, 62, 2)
C = C0.copy(order="F")
g.zgemm("C", "N", m, n, k, 1.0 - 0.5j, A, k, B, k, 0.5, C, m)
rows, cols = rng.integers(0, m, 256), rng.integers(0, n, 256)
t = oracle.zgemm_dot2_sampled("C", "N", k, 1.0 - 0.5j, A, k, B, k, 0.5, C0, m, rows, cols)
out["z_err"] = float(np.linalg.norm(C[rows, cols] - t) / np.linalg.norm(t))
print(json.dumps(out))
"""


def run_child(split: bool):
    env = dict(os.environ)
    env.pop("GB300_DROPIN_FORM", None)
    if split:
        env["GB300_DROPIN_FORM"] = "split"
    r = subprocess.run([sys.executable, "-c", CHILD % {"root": ROOT}], env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_dropin_split_form_is_faster_at_equal_error():
    plain = run_child(False)
    split = run_child(True)
    for p in ("d", "s", "z"):
        assert split[p + "_err"] <= plain[p + "_err"] * 1.0 + 1e-300, (p, split, plain)
    # FP64 pipe against the tensor pipe (FP32 at this size is mostly host transfer)
    assert split["d_ms"] * 4 < plain["d_ms"], (split, plain)
