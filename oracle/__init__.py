"""CPU oracle for the sgemm_/dgemm_ path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, and only as the checker.  The product library
(``gemm_avx2_gb300``) never loads it.

Contents (all thin ctypes wrappers over ``oracle/liborc.so``, built from
``oracle/oracle.c`` by ``oracle/build.sh``):

* ``uniform`` / ``spread``: the portable counter-based input generator.
* ``refgemm``: bit-exact restatement of the reference's GEMM algorithm
  (wjc404/GEMM_AVX2 ``src/gemm_driver.c:118-197``; see ``oracle.c`` header).
* ``dot2gemm`` / ``dot2gemm_sampled``: compensated FP64 ground truth
  (Ogita-Rump-Oishi Dot2).
* ``RefLib``: the reference library itself (``oracle/_ref/{D,S}GEMM.so``) when
  it was compiled here from the reference sources (x86-64 only).
* ``cuniform`` / ``zgemm_dot2`` / ``zgemm_dot2_sampled``: complex inputs and
  the complex ground truth (trans N/T/C/R, complex alpha and beta).
* ``zgemm_port``: the complex kernels' arithmetic in portable C (CPU baseline).
* ``RefCplx``: the reference's OpenBLAS-style complex and 3M kernels
  (``oracle/_ref/libcplx.so``, x86-64 only) behind ``oracle/ref_cplx.c``.
* ``RefBlas3``: the reference's OpenBLAS-style TRSM and TRMM kernels
  (``oracle/_ref/libblas3.so``, x86-64 only) behind ``oracle/ref_blas3.c``.
* ``split``: numpy restatements of the split-precision decompositions
  (3xBF16 hi/lo and the int8-valued Ozaki slices) used to check the GPU split
  kernels bit for bit.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import c_char, c_double, c_float, c_int, c_int64, c_uint64, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def build(reference_dir: str | None = None) -> None:
    """Compile liborc.so (and the reference into _ref/ when its sources exist)."""
    import subprocess

    cmd = ["sh", os.path.join(HERE, "build.sh")]
    if reference_dir:
        cmd.append(reference_dir)
    subprocess.check_call(cmd)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liborc.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.orc_fill_uniform_d.argtypes = [c_void_p, c_int64, c_uint64, c_uint64]
        L.orc_fill_uniform_s.argtypes = [c_void_p, c_int64, c_uint64, c_uint64]
        L.orc_fill_spread_d.argtypes = [c_void_p, c_int64, c_uint64, c_uint64, c_double]
        L.orc_draw.argtypes = [c_uint64, c_uint64, c_uint64]
        L.orc_draw.restype = c_uint64
        gemm_args = [c_char, c_char, c_int, c_int, c_int]
        L.orc_refgemm_d.argtypes = gemm_args + [c_double, c_void_p, c_int, c_void_p, c_int,
                                                c_double, c_void_p, c_int, c_int]
        L.orc_refgemm_s.argtypes = gemm_args + [c_float, c_void_p, c_int, c_void_p, c_int,
                                                c_float, c_void_p, c_int, c_int]
        d2 = gemm_args + [c_double, c_void_p, c_int, c_void_p, c_int, c_double, c_void_p, c_int]
        L.orc_dot2gemm_d.argtypes = d2 + [c_void_p, c_int]
        L.orc_dot2gemm_s.argtypes = d2 + [c_void_p, c_int]
        L.orc_dot2gemm_sampled_d.argtypes = d2 + [c_void_p, c_void_p, c_int64, c_void_p]
        L.orc_dot2gemm_sampled_s.argtypes = d2 + [c_void_p, c_void_p, c_int64, c_void_p]
        L.orc_geometry.argtypes = [c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                                   ctypes.POINTER(c_int)]
        L.orc_max_threads.restype = c_int
        z2 = gemm_args + [c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p, c_int]
        L.orc_zgemm_dot2.argtypes = z2 + [c_void_p, c_int]
        L.orc_cgemm_dot2.argtypes = z2 + [c_void_p, c_int]
        zs = [c_char, c_char, c_int, c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p,
              c_void_p, c_int, c_void_p, c_void_p, c_int64, c_void_p]
        L.orc_zgemm_dot2_sampled.argtypes = zs
        L.orc_cgemm_dot2_sampled.argtypes = zs
        zp = [c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_int,
              c_void_p, c_int]
        L.orc_zgemm_port.argtypes = zp
        L.orc_cgemm_port.argtypes = zp
        _LIB = L
    return _LIB


def _ptr(x: np.ndarray | None):
    return None if x is None else c_void_p(x.ctypes.data)


# ---------------------------------------------------------------- generator
def uniform(shape, dtype, seed: int, stream: int) -> np.ndarray:
    """U[-1,1) matrix in Fortran (column-major) order; element order = storage order."""
    dtype = np.dtype(dtype)
    out = np.empty(shape, dtype=dtype, order="F")
    n = out.size
    if dtype == np.float64:
        lib().orc_fill_uniform_d(_ptr(out), n, seed, stream)
    elif dtype == np.float32:
        lib().orc_fill_uniform_s(_ptr(out), n, seed, stream)
    else:
        raise TypeError(dtype)
    return out


def spread(shape, seed: int, stream: int, phi: float) -> np.ndarray:
    """(u-0.5)*exp(phi*g) FP64 matrix, column-major."""
    out = np.empty(shape, dtype=np.float64, order="F")
    lib().orc_fill_spread_d(_ptr(out), out.size, seed, stream, float(phi))
    return out


def storage(rows: int, cols: int, ld: int, dtype, seed: int, stream: int,
            phi: float | None = None) -> np.ndarray:
    """A column-major buffer of ld x cols (ld >= rows); pad rows are generated too."""
    shape = (max(ld, 1), cols)
    if phi is None:
        return uniform(shape, dtype, seed, stream)
    return spread(shape, seed, stream, phi).astype(dtype, order="F")


def geometry(is_double: bool):
    u, n, k = c_int(), c_int(), c_int()
    lib().orc_geometry(1 if is_double else 0, ctypes.byref(u), ctypes.byref(n), ctypes.byref(k))
    return u.value, n.value, k.value


# ---------------------------------------------------------------- reference restatement
def _check_f(x: np.ndarray, dtype):
    if x.dtype != dtype or not (x.flags.f_contiguous or x.ndim == 1):
        raise TypeError("expected a Fortran-ordered %s array" % dtype)


def refgemm(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, threads: int) -> None:
    """In place on c: the reference algorithm with a team of `threads` threads."""
    dt = c.dtype
    for x in (a, b, c):
        _check_f(x, dt)
    f = lib().orc_refgemm_d if dt == np.float64 else lib().orc_refgemm_s
    f(ta.encode() if isinstance(ta, str) else ta, tb.encode() if isinstance(tb, str) else tb,
      m, n, k, alpha, _ptr(a), lda, _ptr(b), ldb, beta, _ptr(c), ldc, threads)


def dot2gemm(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc) -> np.ndarray:
    """FP64 m x n result of alpha*op(A)op(B)+beta*C with compensated dots."""
    out = np.empty((m, n), dtype=np.float64, order="F")
    if m == 0 or n == 0:
        return out
    f = lib().orc_dot2gemm_d if a.dtype == np.float64 else lib().orc_dot2gemm_s
    f(ta.encode(), tb.encode(), m, n, k, float(alpha), _ptr(a), lda, _ptr(b), ldb, float(beta),
      _ptr(c), ldc, _ptr(out), max(m, 1))
    return out


def dot2gemm_sampled(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, rows, cols):
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    out = np.empty(rows.shape[0], dtype=np.float64)
    f = lib().orc_dot2gemm_sampled_d if a.dtype == np.float64 else lib().orc_dot2gemm_sampled_s
    f(ta.encode(), tb.encode(), m, n, k, float(alpha), _ptr(a), lda, _ptr(b), ldb, float(beta),
      _ptr(c), ldc, _ptr(rows), _ptr(cols), rows.shape[0], _ptr(out))
    return out


# ---------------------------------------------------------------- complex
_REAL_OF = {np.dtype(np.complex128): np.float64, np.dtype(np.complex64): np.float32}


def cuniform(shape, dtype, seed: int, stream: int) -> np.ndarray:
    """Complex column-major matrix whose (re, im) pairs are consecutive U[-1,1)
    draws of the portable generator (storage order)."""
    dtype = np.dtype(dtype)
    rows, cols = shape
    re = uniform((2 * rows, cols), _REAL_OF[dtype], seed, stream)
    return re.T.view(dtype).T


def _cpair(v) -> np.ndarray:
    v = complex(v)
    return np.array([v.real, v.imag], dtype=np.float64)


def zgemm_dot2(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc) -> np.ndarray:
    """complex128 m x n result of alpha*op(A)op(B)+beta*C (Dot2 real and
    imaginary parts); a, b, c complex64 or complex128 column-major, c may be None."""
    out = np.zeros((m, n), dtype=np.complex128, order="F")
    if m == 0 or n == 0:
        return out
    f = lib().orc_zgemm_dot2 if a.dtype == np.complex128 else lib().orc_cgemm_dot2
    al, be = _cpair(alpha), _cpair(beta)
    f(ta.encode(), tb.encode(), m, n, k, _ptr(al), _ptr(a), lda, _ptr(b), ldb, _ptr(be),
      _ptr(c), ldc, _ptr(out), max(m, 1))
    return out


def zgemm_dot2_sampled(ta, tb, k, alpha, a, lda, b, ldb, beta, c, ldc, rows, cols):
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    out = np.empty(rows.shape[0], dtype=np.complex128)
    f = lib().orc_zgemm_dot2_sampled if a.dtype == np.complex128 else lib().orc_cgemm_dot2_sampled
    al, be = _cpair(alpha), _cpair(beta)
    f(ta.encode(), tb.encode(), k, _ptr(al), _ptr(a), lda, _ptr(b), ldb, _ptr(be), _ptr(c), ldc,
      _ptr(rows), _ptr(cols), rows.shape[0], _ptr(out))
    return out


def zgemm_port(conj_a, conj_b, alpha, A, B, C) -> None:
    """In place: C += alpha * conj_a(A) conj_b(B) with the reference complex
    kernels' operation sequence in portable C (OpenMP over columns of C)."""
    m, k = A.shape
    n = B.shape[1]
    if C.dtype == np.complex128:
        al, f = np.array([complex(alpha).real, complex(alpha).imag]), lib().orc_zgemm_port
    else:
        al = np.array([complex(alpha).real, complex(alpha).imag], np.float32)
        f = lib().orc_cgemm_port
    f(int(conj_a), int(conj_b), m, n, k, _ptr(al), _ptr(A), A.shape[0], _ptr(B), B.shape[0],
      _ptr(C), C.shape[0])


class RefCplx:
    """The reference's complex GEMM kernels and 3M kernels, compiled from their
    sources into oracle/_ref/libcplx.so (x86-64 only)."""

    PATH = os.path.join(HERE, "_ref", "libcplx.so")

    def __init__(self):
        if not os.path.exists(self.PATH):
            raise FileNotFoundError("reference complex kernels not built (x86-64 with sources only)")
        L = ctypes.CDLL(self.PATH)
        for name, F in (("ref_zgemm_conj", c_double), ("ref_cgemm_conj", c_float)):
            getattr(L, name).argtypes = [c_int, c_int, ctypes.c_long, ctypes.c_long, ctypes.c_long,
                                         F, F, c_void_p, ctypes.c_long, c_void_p, ctypes.c_long,
                                         c_void_p, ctypes.c_long]
        for name, F in (("ref_zgemm3m_conj", c_double), ("ref_cgemm3m_conj", c_float)):
            getattr(L, name).argtypes = [c_int, c_int, ctypes.c_long, ctypes.c_long, ctypes.c_long,
                                         F, F, c_void_p, ctypes.c_long, c_void_p, ctypes.c_long,
                                         c_void_p, ctypes.c_long]
        self.L = L

    @classmethod
    def available(cls) -> bool:
        return os.path.exists(cls.PATH)

    def gemm_conj(self, conj_a: bool, conj_b: bool, alpha, A, B, C) -> None:
        """In place: C += alpha * conj_a(A) * conj_b(B) (A m x k, B k x n, complex F arrays)."""
        m, k = A.shape
        n = B.shape[1]
        f = self.L.ref_zgemm_conj if C.dtype == np.complex128 else self.L.ref_cgemm_conj
        rc = f(int(conj_a), int(conj_b), m, n, k, complex(alpha).real, complex(alpha).imag,
               _ptr(A), A.shape[0], _ptr(B), B.shape[0], _ptr(C), C.shape[0])
        assert rc == 0

    def gemm3m(self, alpha, A, B, C) -> None:
        """In place: C (complex) += alpha * (A @ B) with real A (m x k) and B (k x n)."""
        m, k = A.shape
        n = B.shape[1]
        f = self.L.ref_zgemm3m_conj if C.dtype == np.complex128 else self.L.ref_cgemm3m_conj
        rc = f(0, 0, m, n, k, complex(alpha).real, complex(alpha).imag, _ptr(A), A.shape[0],
               _ptr(B), B.shape[0], _ptr(C), C.shape[0])
        assert rc == 0


class RefBlas3:
    """The reference's TRSM kernels (TRSM_KERNEL_*_simplified.c over its
    dgemm_kernel_4x4_haswell.c; strsm_kernel_8x4_haswell_*.c) and TRMM kernel
    (trmm_kernel_4x8_simplified.c), compiled from their sources into
    oracle/_ref/libblas3.so (x86-64 only), called on the whole problem as one
    packed block."""

    PATH = os.path.join(HERE, "_ref", "libblas3.so")

    def __init__(self):
        if not os.path.exists(self.PATH):
            raise FileNotFoundError("reference TRSM/TRMM kernels not built (x86-64 with sources only)")
        L = ctypes.CDLL(self.PATH)
        lng = ctypes.c_long
        for r in ("trsm", "trmm"):
            for p, F in (("d", c_double), ("s", c_float)):
                getattr(L, "ref_%s_%s" % (r, p)).argtypes = [c_char, c_char, c_char, c_char, lng,
                                                             lng, F, c_void_p, lng, c_void_p, lng]
        self.L = L

    @classmethod
    def available(cls) -> bool:
        return os.path.exists(cls.PATH)

    def call(self, routine, side, uplo, transa, diag, m, n, alpha, A, B) -> np.ndarray:
        """B := alpha inv(op(A)) B / B inv(op(A)) (trsm) or alpha op(A) B / B op(A)
        (trmm); A and B Fortran arrays of one dtype; returns the updated copy of B."""
        assert A.dtype == B.dtype and A.flags.f_contiguous and B.flags.f_contiguous
        out = np.array(B, order="F", copy=True)
        f = getattr(self.L, "ref_%s_%s" % (routine, "d" if B.dtype == np.float64 else "s"))
        rc = f(side.encode(), uplo.encode(), transa.encode(), diag.encode(), m, n, alpha,
               _ptr(A), A.shape[0], _ptr(out), out.shape[0])
        assert rc == 0
        return out


def set_threads(n: int) -> None:
    """Set the OpenMP team size of this process (shared by liborc and the reference)."""
    lib()
    try:
        gomp = ctypes.CDLL("libgomp.so.1")
        gomp.omp_set_num_threads(int(n))
    except OSError:
        pass


def max_threads() -> int:
    return lib().orc_max_threads()


# ---------------------------------------------------------------- the reference library
class RefLib:
    """The reference's own dgemm_/sgemm_, compiled from its sources into oracle/_ref/."""

    def __init__(self):
        d = os.path.join(HERE, "_ref", "DGEMM.so")
        s = os.path.join(HERE, "_ref", "SGEMM.so")
        if not (os.path.exists(d) and os.path.exists(s)):
            raise FileNotFoundError("reference library not built (x86-64 with sources only)")
        self.d = ctypes.CDLL(d)
        self.s = ctypes.CDLL(s)

    @staticmethod
    def available() -> bool:
        return os.path.exists(os.path.join(HERE, "_ref", "DGEMM.so"))

    def gemm(self, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc) -> None:
        dt = c.dtype
        F = c_double if dt == np.float64 else c_float
        fn = self.d.dgemm_ if dt == np.float64 else self.s.sgemm_
        ci = lambda v: ctypes.byref(c_int(v))
        fn(ctypes.c_char_p(ta.encode()), ctypes.c_char_p(tb.encode()), ci(m), ci(n), ci(k),
           ctypes.byref(F(alpha)), _ptr(a), ci(lda), _ptr(b), ci(ldb), ctypes.byref(F(beta)),
           _ptr(c), ci(ldc))


# ---------------------------------------------------------------- error metrics
def rel_errors(x: np.ndarray, truth: np.ndarray):
    """(max elementwise relative error, Frobenius relative error) of x vs truth."""
    x = np.asarray(x, dtype=np.float64)
    t = np.asarray(truth, dtype=np.float64)
    d = np.abs(x - t)
    denom = np.abs(t)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(denom > 0, d / np.where(denom > 0, denom, 1.0), np.where(d > 0, np.inf, 0.0))
    mx = float(np.max(r)) if r.size else 0.0
    nt = float(np.linalg.norm(t))
    fro = float(np.linalg.norm(d)) / nt if nt > 0 else float(np.linalg.norm(d))
    return mx, fro


def exponent_spread(x: np.ndarray) -> int:
    """max - min of ilogb over the nonzero finite entries."""
    v = np.abs(np.asarray(x, dtype=np.float64).ravel())
    v = v[(v > 0) & np.isfinite(v)]
    if v.size == 0:
        return 0
    e = np.frexp(v)[1]
    return int(e.max() - e.min())
