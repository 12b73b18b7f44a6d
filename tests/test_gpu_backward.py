"""The backward pass of C = alpha*op(A)*op(B) + beta*C needs no adjoint kernel:
dL/dA and dL/dB are two more GEMMs through the same transa/transb paths of the
library.  Checked against torch autograd (FP64, CPU) for all transposes, with
the plain FP64 kernel and with the FP32 6xBF16 split form."""
import numpy as np
import pytest
import torch

import gemm_avx2_gb300 as g
from gpu_util import from_dev, sync, to_dev

pytestmark = pytest.mark.gpu


def grads_via_gemm(prec, ta, tb, m, n, k, alpha, A, B, G, split=False):
    """dA (stored like A) and dB (stored like B) with two GEMM calls each."""
    dt = np.float64 if prec == "d" else np.float32
    ar, ac = (m, k) if ta == "N" else (k, m)
    br, bc = (k, n) if tb == "N" else (n, k)
    dA_ = to_dev(np.zeros((ar, ac), dt, order="F"))
    dB_ = to_dev(np.zeros((br, bc), dt, order="F"))
    dAd, dBd, dG = to_dev(A), to_dev(B), to_dev(G)

    def gemm(tx, ty, mm, nn, kk, X, ldx, Y, ldy, Z, ldz):
        if split:
            rc = g.sgemm_bf16x(tx, ty, mm, nn, kk, alpha, X.data_ptr(), ldx, Y.data_ptr(), ldy,
                               0.0, Z.data_ptr(), ldz, products=6)
        else:
            rc = g.gemm_device(prec, tx, ty, mm, nn, kk, alpha, X.data_ptr(), ldx, Y.data_ptr(),
                               ldy, 0.0, Z.data_ptr(), ldz)
        assert rc == g.OK

    flip = {"N": "T", "T": "N"}
    # dL/dop(A) = alpha * G * op(B)^T   (m x k)
    if ta == "N":   # A is m x k: dA = alpha * G * op(B)^T
        gemm("N", flip[tb], m, k, n, dG, m, dBd, br, dA_, m)
    else:           # A is k x m: dA = (alpha * G * op(B)^T)^T = alpha * op(B) * G^T
        gemm(tb, "T", k, m, n, dBd, br, dG, m, dA_, k)
    # dL/dop(B) = alpha * op(A)^T * G   (k x n)
    if tb == "N":   # B is k x n
        gemm(flip[ta], "N", k, n, m, dAd, ar, dG, m, dB_, k)
    else:           # B is n x k: dB = alpha * G^T * op(A)
        gemm("T", ta, n, k, m, dG, m, dAd, ar, dB_, n)
    sync()
    return from_dev(dA_, ar), from_dev(dB_, br)


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
@pytest.mark.parametrize("prec,split", [("d", False), ("s", True)])
def test_backward_is_two_gemms(orc, ta, tb, prec, split):
    m, n, k = 150, 130, 170
    dt = np.float64 if prec == "d" else np.float32
    ar, ac = (m, k) if ta == "N" else (k, m)
    br, bc = (k, n) if tb == "N" else (n, k)
    A = orc.uniform((ar, ac), dt, 81, 0)
    B = orc.uniform((br, bc), dt, 81, 1)
    G = orc.uniform((m, n), dt, 81, 2)          # upstream gradient dL/dC
    alpha = 0.75
    tA = torch.tensor(A.astype(np.float64), requires_grad=True)
    tB = torch.tensor(B.astype(np.float64), requires_grad=True)
    opA = tA if ta == "N" else tA.T
    opB = tB if tb == "N" else tB.T
    C = alpha * opA @ opB
    C.backward(torch.tensor(G.astype(np.float64)))
    dA, dB = grads_via_gemm(prec, ta, tb, m, n, k, alpha, A, B, G, split)
    tol = 1e-13 if prec == "d" else 2e-6
    for got, want in ((dA, tA.grad.numpy()), (dB, tB.grad.numpy())):
        d = np.linalg.norm(got.astype(np.float64) - want) / np.linalg.norm(want)
        assert d < tol, (ta, tb, prec, d)
