"""CPU tests of the complex oracle: the ground truth against exact and numpy
results, and its conventions pinned to the reference's own OpenBLAS-style
complex kernels (four conjugation variants, and the 3M kernels), compiled from
their sources into oracle/_ref/libcplx.so where that is possible (x86-64)."""
import numpy as np
import pytest

import oracle
from util import U32, U64, cgemm_bound, check_close_c, cop

TRANS = ["N", "T", "C", "R"]


def test_cuniform_storage_order():
    Z = oracle.cuniform((5, 3), np.complex128, 1, 0)
    R = oracle.uniform((10, 3), np.float64, 1, 0)
    assert Z.flags.f_contiguous and Z.shape == (5, 3)
    assert np.array_equal(Z.real, R[0::2]) and np.array_equal(Z.imag, R[1::2])
    C = oracle.cuniform((4, 2), np.complex64, 1, 0)
    assert np.array_equal(C.real, oracle.uniform((8, 2), np.float32, 1, 0)[0::2])


@pytest.mark.parametrize("ta", TRANS)
@pytest.mark.parametrize("tb", TRANS)
def test_dot2_matches_numpy_all_trans(ta, tb):
    m, n, k = 9, 7, 13
    A = oracle.cuniform((m, k) if ta in "NR" else (k, m), np.complex128, 5, 0)
    B = oracle.cuniform((k, n) if tb in "NR" else (n, k), np.complex128, 5, 1)
    C = oracle.cuniform((m, n), np.complex128, 5, 2)
    al, be = 0.5 - 1.25j, -0.75 + 0.5j
    got = oracle.zgemm_dot2(ta, tb, m, n, k, al, A, A.shape[0], B, B.shape[0], be, C, m)
    want = al * (cop(A, ta, m, k) @ cop(B, tb, k, n)) + be * C
    assert np.allclose(got, want, rtol=1e-14, atol=1e-14)


def test_dot2_exact_on_integer_data():
    """Small integers: every product and partial sum is exact, so the ground
    truth must equal the integer result."""
    rng = np.random.default_rng(3)
    m, n, k = 6, 5, 40
    A = (rng.integers(-9, 9, (m, k)) + 1j * rng.integers(-9, 9, (m, k))).astype(np.complex128)
    B = (rng.integers(-9, 9, (k, n)) + 1j * rng.integers(-9, 9, (k, n))).astype(np.complex128)
    C = (rng.integers(-9, 9, (m, n)) + 1j * rng.integers(-9, 9, (m, n))).astype(np.complex128)
    A, B, C = (np.asfortranarray(x) for x in (A, B, C))
    got = oracle.zgemm_dot2("N", "C", m, n, k, 2 - 3j, A, m, np.asfortranarray(B.T), n, 1 + 1j,
                            C, m)
    want = (2 - 3j) * (A @ B.conj()) + (1 + 1j) * C
    assert np.array_equal(got, want)


def test_sampled_equals_full():
    m, n, k = 11, 6, 17
    A = oracle.cuniform((k, m), np.complex64, 7, 0)
    B = oracle.cuniform((k, n), np.complex64, 7, 1)
    C = oracle.cuniform((m, n), np.complex64, 7, 2)
    full = oracle.zgemm_dot2("C", "N", m, n, k, 1.5j, A, k, B, k, 0.5, C, m)
    rows = np.array([0, 10, 3, 5]), np.array([0, 5, 2, 4])
    s = oracle.zgemm_dot2_sampled("C", "N", k, 1.5j, A, k, B, k, 0.5, C, m, *rows)
    assert np.array_equal(s, full[rows])


needs_ref = pytest.mark.skipif(not oracle.RefCplx.available(),
                               reason="reference complex kernels not built (x86-64 only)")


@needs_ref
@pytest.mark.parametrize("dt", [np.complex128, np.complex64])
@pytest.mark.parametrize("conj_a,conj_b", [(0, 0), (1, 0), (0, 1), (1, 1)])
@pytest.mark.parametrize("shape", [(15, 11, 9), (7, 9, 33), (1, 1, 1), (16, 6, 2), (300, 13, 700)])
def test_reference_kernels_pin_conj_variants(dt, conj_a, conj_b, shape):
    """The reference's NN/RN/NR/RR kernels add alpha * conj_a(A) conj_b(B) to C:
    the oracle's 'R' trans code, within the kernels' rounding bound."""
    m, n, k = shape
    ref = oracle.RefCplx()
    A = oracle.cuniform((m, k), dt, 13, 0)
    B = oracle.cuniform((k, n), dt, 13, 1)
    C0 = oracle.cuniform((m, n), dt, 13, 2)
    al = 0.625 - 1.5j
    C = C0.copy(order="F")
    ref.gemm_conj(conj_a, conj_b, al, A, B, C)
    ta, tb = ("R" if conj_a else "N"), ("R" if conj_b else "N")
    truth = oracle.zgemm_dot2(ta, tb, m, n, k, al, A, m, B, k, 1.0, C0, m)
    u = U64 if dt == np.complex128 else U32
    check_close_c(C, truth, cgemm_bound(cop(A, ta, m, k), cop(B, tb, k, n), C0, al, 1.0, k, u))


@needs_ref
@pytest.mark.parametrize("dt", [np.complex128, np.complex64])
@pytest.mark.parametrize("shape", [(15, 23, 9), (7, 4, 33), (1, 1, 1), (400, 9, 700)])
def test_reference_3m_kernel_adds_alpha_times_real_product(dt, shape):
    m, n, k = shape
    ref = oracle.RefCplx()
    rdt = np.float64 if dt == np.complex128 else np.float32
    A = oracle.uniform((m, k), rdt, 17, 0)
    B = oracle.uniform((k, n), rdt, 17, 1)
    C0 = oracle.cuniform((m, n), dt, 17, 2)
    al = -0.75 + 0.25j
    C = C0.copy(order="F")
    ref.gemm3m(al, A, B, C)
    Ac, Bc = A.astype(np.complex128, order="F"), B.astype(np.complex128, order="F")
    truth = oracle.zgemm_dot2("N", "N", m, n, k, al, Ac, m, Bc, k, 1.0, C0.astype(np.complex128),
                              m)
    u = U64 if dt == np.complex128 else U32
    check_close_c(C, truth, cgemm_bound(Ac, Bc, C0, al, 1.0, k, u))


@pytest.mark.parametrize("dt", [np.complex128, np.complex64])
@pytest.mark.parametrize("conj_a,conj_b", [(0, 0), (1, 1), (1, 0)])
def test_port_matches_truth(dt, conj_a, conj_b):
    """The portable restatement of the complex kernels' arithmetic computes
    C += alpha * conj_a(A) conj_b(B) within the kernels' rounding bound."""
    m, n, k = 37, 13, 50
    A = oracle.cuniform((m, k), dt, 19, 0)
    B = oracle.cuniform((k, n), dt, 19, 1)
    C0 = oracle.cuniform((m, n), dt, 19, 2)
    C = C0.copy(order="F")
    oracle.zgemm_port(conj_a, conj_b, 0.5 + 2j, A, B, C)
    ta, tb = ("R" if conj_a else "N"), ("R" if conj_b else "N")
    truth = oracle.zgemm_dot2(ta, tb, m, n, k, 0.5 + 2j, A, m, B, k, 1.0, C0, m)
    u = U64 if dt == np.complex128 else U32
    check_close_c(C, truth, cgemm_bound(cop(A, ta, m, k), cop(B, tb, k, n), C0, 0.5 + 2j, 1.0, k, u))


@needs_ref
def test_port_agrees_with_reference_kernel():
    """Same inputs through the reference's NN kernel and the port: both within
    a few ulps of each other (the kernels' contracted n>=4 path sums in a
    different order, so not bit for bit)."""
    m, n, k = 15, 11, 64
    A = oracle.cuniform((m, k), np.complex128, 23, 0)
    B = oracle.cuniform((k, n), np.complex128, 23, 1)
    C1 = oracle.cuniform((m, n), np.complex128, 23, 2)
    C2 = C1.copy(order="F")
    oracle.RefCplx().gemm_conj(0, 0, 1.0, A, B, C1)
    oracle.zgemm_port(0, 0, 1.0, A, B, C2)
    assert np.max(np.abs(C1 - C2)) < 64 * k * U64
