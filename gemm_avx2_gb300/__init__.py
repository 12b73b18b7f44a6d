"""GB300 (sm_103a) drop-in for the sgemm_/dgemm_ path of wjc404/GEMM_AVX2.

The product is native code in this directory:

* ``DGEMM.so`` / ``SGEMM.so`` export exactly ``dgemm_`` / ``sgemm_`` with the
  reference's Fortran-style ABI (reference ``src/gemm_driver.c:118``).
* ``ZGEMM.so`` / ``CGEMM.so`` export the complex BLAS symbols ``zgemm_`` /
  ``zgemm3m_`` and ``cgemm_`` / ``cgemm3m_``.
* ``libgemm_gb300.so`` holds every CUDA kernel and the ``gb300_*`` C ABI
  declared in ``include/gemm_gb300.h`` (device pointers, streams, split forms).

This module is a thin ctypes mirror of that ABI so that tests and the
benchmark call the library exactly as a C or Fortran caller would:

* ``dgemm`` / ``sgemm`` mirror the reference interface argument for argument
  (host arrays, column-major, ``lda``/``ldb``/``ldc``) and go through the
  drop-in ``DGEMM.so``/``SGEMM.so``.
* ``gemm_device`` and friends take device pointers (integers, e.g. from
  ``torch.Tensor.data_ptr()``) and a stream handle.

There is no CPU fallback: if the native library is missing, loading fails
with an error.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import c_char, c_double, c_float, c_int, c_size_t, c_uint, c_void_p

PKG = os.path.dirname(os.path.abspath(__file__))

OK = 0
ERR_ARG = 1
ERR_CUDA = 2
ERR_TIMEOUT = 3
ERR_NOMEM = 4
ERR_UNSUPPORTED = 5
ERR_WORKSPACE = 6
ERR_NOALLOC_LIMIT = 7

# complex GEMM methods (gb300_cgemm / gb300_zgemm)
# `products` code of the scaled 3xFP16 split SGEMM (GB300_SPLIT_FP16X3)
FP16X3 = 0x103
CPLX_4M = 0
CPLX_3M = 1
CPLX_SPLIT = 2
CPLX_CRT = 3

_core = None
_drop = {}


class NativeLibraryMissing(RuntimeError):
    pass


def build() -> None:
    """Compile the native library in place (nvcc, sm_103a)."""
    from . import native_build

    native_build.build()


def _load(name: str) -> ctypes.CDLL:
    path = os.path.join(PKG, name)
    if not os.path.exists(path):
        raise NativeLibraryMissing(
            "%s not built: run gemm_avx2_gb300.build() (or __graft_entry__.build())" % path)
    return ctypes.CDLL(path, mode=ctypes.RTLD_GLOBAL)


def core() -> ctypes.CDLL:
    """libgemm_gb300.so with argument types declared."""
    global _core
    if _core is None:
        L = _load("libgemm_gb300.so")
        g = [c_char, c_char, c_int, c_int, c_int]
        L.gb300_dgemm.argtypes = g + [c_double, c_void_p, c_int, c_void_p, c_int, c_double,
                                      c_void_p, c_int, c_void_p]
        L.gb300_sgemm.argtypes = g + [c_float, c_void_p, c_int, c_void_p, c_int, c_float,
                                      c_void_p, c_int, c_void_p]
        L.gb300_host_dgemm.argtypes = g + [c_double, c_void_p, c_int, c_void_p, c_int, c_double,
                                           c_void_p, c_int]
        L.gb300_host_sgemm.argtypes = g + [c_float, c_void_p, c_int, c_void_p, c_int, c_float,
                                           c_void_p, c_int]
        L.gb300_sgemm_bf16x.argtypes = g + [c_float, c_void_p, c_int, c_void_p, c_int, c_float,
                                            c_void_p, c_int, c_int, c_void_p]
        L.gb300_sgemm_bf16x_ws.argtypes = g + [c_float, c_void_p, c_int, c_void_p, c_int,
                                               c_float, c_void_p, c_int, c_int, c_void_p,
                                               c_size_t, c_void_p]
        L.gb300_dgemm_ozaki.argtypes = g + [c_double, c_void_p, c_int, c_void_p, c_int,
                                            c_double, c_void_p, c_int, c_int, c_void_p]
        L.gb300_dgemm_ozaki_ws.argtypes = g + [c_double, c_void_p, c_int, c_void_p, c_int,
                                               c_double, c_void_p, c_int, c_int, c_void_p,
                                               c_size_t, c_void_p]
        L.gb300_sgemm_bf16x_prepare.argtypes = g + [c_void_p, c_int, c_void_p, c_int, c_int,
                                                    c_void_p, c_size_t, c_void_p]
        L.gb300_sgemm_bf16x_run.argtypes = [c_int, c_int, c_int, c_float, c_float, c_void_p,
                                            c_int, c_int, c_void_p, c_size_t, c_void_p]
        L.gb300_dgemm_ozaki_prepare.argtypes = g + [c_void_p, c_int, c_void_p, c_int, c_int,
                                                    c_void_p, c_size_t, c_void_p]
        L.gb300_dgemm_ozaki_run.argtypes = [c_int, c_int, c_int, c_double, c_double, c_void_p,
                                            c_int, c_int, c_void_p, c_size_t, c_void_p]
        L.gb300_host_sgemm_bf16x.argtypes = g + [c_float, c_void_p, c_int, c_void_p, c_int,
                                                 c_float, c_void_p, c_int, c_int]
        L.gb300_host_dgemm_ozaki.argtypes = g + [c_double, c_void_p, c_int, c_void_p, c_int,
                                                 c_double, c_void_p, c_int, c_int]
        L.gb300_split_workspace_bytes.argtypes = [c_int, c_int, c_int, c_int, c_int]
        L.gb300_split_workspace_bytes.restype = c_size_t
        L.gb300_device_error.argtypes = [c_int]
        L.gb300_device_error.restype = c_uint
        L.gb300_version.restype = ctypes.c_char_p
        L.gb300_selftest_wait_timeout.argtypes = [c_uint]
        L.gb300_tune_param.argtypes = [c_int, c_int]
        L.gb300_autotune.argtypes = [c_int, c_char, c_char, c_int, c_int, c_int, c_void_p, c_int,
                                     c_void_p, c_int, c_void_p, ctypes.POINTER(c_int)]
        L.gb300_tune_lookup.argtypes = [c_int, c_int, c_int, c_int, ctypes.POINTER(c_int),
                                        ctypes.POINTER(c_int)]
        L.gb300_tune_layout.argtypes = [c_int, c_int, c_int, c_int, ctypes.POINTER(c_int),
                                        ctypes.POINTER(c_int)]
        L.gb300_plain_layout.argtypes = [c_int, c_int, c_int, c_int, ctypes.POINTER(c_int),
                                         ctypes.POINTER(c_int)]
        L.gb300_tune_cache_save.argtypes = [ctypes.c_char_p]
        L.gb300_tune_cache_load.argtypes = [ctypes.c_char_p, ctypes.POINTER(c_int)]
        L.gb300_tune_cache_clear.restype = None
        for nm, F in (("gb300_dtrsm", c_double), ("gb300_strsm", c_float),
                      ("gb300_dtrmm", c_double), ("gb300_strmm", c_float)):
            getattr(L, nm).argtypes = [c_char, c_char, c_char, c_char, c_int, c_int, F, c_void_p,
                                       c_int, c_void_p, c_int, c_int, c_void_p]
        L.gb300_grouped_workspace_bytes.argtypes = [c_int]
        L.gb300_grouped_workspace_bytes.restype = c_size_t
        L.gb300_gemm_grouped.argtypes = [c_void_p, c_int, c_void_p]
        L.gb300_gemm_grouped_ws.argtypes = [c_void_p, c_int, c_void_p, c_size_t, c_void_p]
        L.gb300_grouped_graph_create.argtypes = [c_void_p, c_int, c_int, ctypes.POINTER(c_void_p)]
        L.gb300_grouped_graph_launch.argtypes = [c_void_p, c_void_p]
        L.gb300_grouped_graph_destroy.argtypes = [c_void_p]
        L.gb300_sgemm_bf16x_noalloc.argtypes = g + [c_float, c_void_p, c_int, c_void_p, c_int,
                                                    c_float, c_void_p, c_int, c_int, c_void_p]
        L.gb300_dgemm_ozaki2.argtypes = g + [c_double, c_void_p, c_int, c_void_p, c_int,
                                             c_double, c_void_p, c_int, c_int, c_void_p, c_size_t,
                                             c_void_p]
        L.gb300_host_dgemm_ozaki2.argtypes = g + [c_double, c_void_p, c_int, c_void_p, c_int,
                                                  c_double, c_void_p, c_int, c_int]
        L.gb300_dgemm_ozaki2_prepare.argtypes = g + [c_void_p, c_int, c_void_p, c_int, c_int,
                                                     c_void_p, c_size_t, c_void_p]
        L.gb300_dgemm_ozaki2_run.argtypes = [c_int, c_int, c_int, c_double, c_double, c_void_p,
                                             c_int, c_int, c_void_p, c_size_t, c_void_p]
        cg = [c_char, c_char, c_int, c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_int,
              c_void_p, c_void_p, c_int, c_int, c_int]
        L.gb300_cgemm.argtypes = cg + [c_void_p, c_size_t, c_void_p]
        L.gb300_zgemm.argtypes = cg + [c_void_p, c_size_t, c_void_p]
        L.gb300_host_cgemm.argtypes = cg
        L.gb300_host_zgemm.argtypes = cg
        L.gb300_complex_workspace_bytes.argtypes = [c_int, c_int, c_char, c_int, c_int, c_int,
                                                    c_int]
        L.gb300_complex_workspace_bytes.restype = c_size_t
        _core = L
    return _core


_DROPIN = {"d": "DGEMM.so", "s": "SGEMM.so", "z": "ZGEMM.so", "c": "CGEMM.so"}


def dropin(precision: str) -> ctypes.CDLL:
    """The drop-in library: 'd' DGEMM.so, 's' SGEMM.so, 'z' ZGEMM.so, 'c' CGEMM.so."""
    if precision not in _drop:
        core()  # resolve libgemm_gb300.so first (RTLD_GLOBAL)
        _drop[precision] = _load(_DROPIN[precision])
    return _drop[precision]


def _b(c) -> bytes:
    return c.encode() if isinstance(c, str) else bytes(c)


def _ptr(x):
    """Address of a numpy array, torch tensor or raw integer pointer."""
    if x is None:
        return None
    if isinstance(x, int):
        return c_void_p(x)
    if hasattr(x, "data_ptr"):
        return c_void_p(x.data_ptr())
    return c_void_p(x.ctypes.data)


# ---------------------------------------------------------------------------
# Reference interface mirror (host arrays, drop-in libraries)
# ---------------------------------------------------------------------------
def dgemm(transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc) -> None:
    """dgemm_ of DGEMM.so: C = alpha*op(A)*op(B) + beta*C on host column-major arrays.

    Same argument meaning as the reference (``src/gemm_driver.c:118``); returns
    nothing; invalid arguments leave ``c`` untouched.
    """
    L = dropin("d")
    i = lambda v: ctypes.byref(c_int(int(v)))
    L.dgemm_(ctypes.c_char_p(_b(transa)), ctypes.c_char_p(_b(transb)), i(m), i(n), i(k),
             ctypes.byref(c_double(alpha)), _ptr(a), i(lda), _ptr(b), i(ldb),
             ctypes.byref(c_double(beta)), _ptr(c), i(ldc))


def sgemm(transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc) -> None:
    """sgemm_ of SGEMM.so (FP32), same contract as :func:`dgemm`."""
    L = dropin("s")
    i = lambda v: ctypes.byref(c_int(int(v)))
    L.sgemm_(ctypes.c_char_p(_b(transa)), ctypes.c_char_p(_b(transb)), i(m), i(n), i(k),
             ctypes.byref(c_float(alpha)), _ptr(a), i(lda), _ptr(b), i(ldb),
             ctypes.byref(c_float(beta)), _ptr(c), i(ldc))


def host_gemm(precision, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc) -> int:
    """Host-pointer path with a status code (gb300_host_dgemm / gb300_host_sgemm)."""
    L = core()
    f = L.gb300_host_dgemm if precision == "d" else L.gb300_host_sgemm
    return f(_b(transa), _b(transb), m, n, k, alpha, _ptr(a), lda, _ptr(b), ldb, beta, _ptr(c),
             ldc)


def _cscalar(v, precision):
    """(re, im) of a Python number as a ctypes array (complex scalars by pointer)."""
    v = complex(v)
    T = c_double if precision == "z" else c_float
    return (T * 2)(v.real, v.imag)


def zgemm(transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, method3m=False) -> None:
    """zgemm_ (or zgemm3m_) of ZGEMM.so on host complex128 column-major arrays:
    C = alpha*op(A)*op(B) + beta*C, trans 'N', 'T', 'C' (conjugate transpose) or
    'R' (conjugate).  Returns nothing; invalid arguments leave ``c`` untouched."""
    _complex_dropin("z", transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, method3m)


def cgemm(transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, method3m=False) -> None:
    """cgemm_ (or cgemm3m_) of CGEMM.so on complex64 arrays, as :func:`zgemm`."""
    _complex_dropin("c", transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, method3m)


def _complex_dropin(p, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, method3m):
    L = dropin(p)
    f = getattr(L, p + ("gemm3m_" if method3m else "gemm_"))
    i = lambda v: ctypes.byref(c_int(int(v)))
    al, be = _cscalar(alpha, p), _cscalar(beta, p)
    f(ctypes.c_char_p(_b(transa)), ctypes.c_char_p(_b(transb)), i(m), i(n), i(k), al, _ptr(a),
      i(lda), _ptr(b), i(ldb), be, _ptr(c), i(ldc))


def host_complex(precision, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc,
                 method=CPLX_4M, param=0) -> int:
    """gb300_host_zgemm / gb300_host_cgemm ('z' / 'c') with a status code."""
    L = core()
    f = L.gb300_host_zgemm if precision == "z" else L.gb300_host_cgemm
    return f(_b(transa), _b(transb), m, n, k, _cscalar(alpha, precision), _ptr(a), lda, _ptr(b),
             ldb, _cscalar(beta, precision), _ptr(c), ldc, method, param)


# ---------------------------------------------------------------------------
# Device-pointer entry points
# ---------------------------------------------------------------------------
def gemm_device(precision, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                stream=0) -> int:
    """gb300_dgemm / gb300_sgemm on device buffers; stream-ordered, returns a status."""
    L = core()
    f = L.gb300_dgemm if precision == "d" else L.gb300_sgemm
    return f(_b(transa), _b(transb), m, n, k, alpha, _ptr(A), lda, _ptr(B), ldb, beta, _ptr(C),
             ldc, c_void_p(stream))


def sgemm_bf16x(transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, products=3,
                stream=0, workspace=None, workspace_bytes=0) -> int:
    """Split-precision SGEMM on the tensor cores: products 3 / 6 (3xBF16 / 6xBF16)
    or FP16X3 (row/column-scaled 3xFP16)."""
    L = core()
    if workspace is None:
        return L.gb300_sgemm_bf16x(_b(transa), _b(transb), m, n, k, alpha, _ptr(A), lda,
                                   _ptr(B), ldb, beta, _ptr(C), ldc, products, c_void_p(stream))
    return L.gb300_sgemm_bf16x_ws(_b(transa), _b(transb), m, n, k, alpha, _ptr(A), lda, _ptr(B),
                                  ldb, beta, _ptr(C), ldc, products, _ptr(workspace),
                                  workspace_bytes, c_void_p(stream))


def dgemm_ozaki(transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, slices=0,
                stream=0, workspace=None, workspace_bytes=0) -> int:
    """Ozaki-scheme DGEMM (int8-range slices, exact products) on the tensor cores."""
    L = core()
    if workspace is None:
        return L.gb300_dgemm_ozaki(_b(transa), _b(transb), m, n, k, alpha, _ptr(A), lda,
                                   _ptr(B), ldb, beta, _ptr(C), ldc, slices, c_void_p(stream))
    return L.gb300_dgemm_ozaki_ws(_b(transa), _b(transb), m, n, k, alpha, _ptr(A), lda, _ptr(B),
                                  ldb, beta, _ptr(C), ldc, slices, _ptr(workspace),
                                  workspace_bytes, c_void_p(stream))


def dgemm_ozaki2(transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, moduli=0,
                 stream=0, workspace=None, workspace_bytes=0) -> int:
    """CRT (modular-integer) DGEMM on the tensor cores: the exact integer product
    of b-bit scaled operands from `moduli` residue GEMMs (0 = 16)."""
    return core().gb300_dgemm_ozaki2(_b(transa), _b(transb), m, n, k, alpha, _ptr(A), lda,
                                     _ptr(B), ldb, beta, _ptr(C), ldc, moduli, _ptr(workspace),
                                     workspace_bytes, c_void_p(stream))


def sgemm_bf16x_noalloc(transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                        products=3, stream=0) -> int:
    """BF16xP split SGEMM whose scratch is the library's fixed 32 MiB device array
    (no allocation; for callers that may not call cudaMalloc)."""
    L = core()
    return L.gb300_sgemm_bf16x_noalloc(_b(transa), _b(transb), m, n, k, alpha, _ptr(A), lda,
                                       _ptr(B), ldb, beta, _ptr(C), ldc, products,
                                       c_void_p(stream))


def split_prepare(form, transa, transb, m, n, k, A, lda, B, ldb, param, workspace,
                  workspace_bytes, stream=0) -> int:
    """Phase 1 of a split form ('bf16x', 'ozaki' or 'crt'): split op(A), op(B)
    into the workspace."""
    L = core()
    f = {"bf16x": L.gb300_sgemm_bf16x_prepare, "ozaki": L.gb300_dgemm_ozaki_prepare,
         "crt": L.gb300_dgemm_ozaki2_prepare}[form]
    return f(_b(transa), _b(transb), m, n, k, _ptr(A), lda, _ptr(B), ldb, param, _ptr(workspace),
             workspace_bytes, c_void_p(stream))


def split_run(form, m, n, k, alpha, beta, C, ldc, param, workspace, workspace_bytes,
              stream=0) -> int:
    """Phase 2 of a split form: the tensor-core GEMM from a prepared workspace."""
    L = core()
    f = {"bf16x": L.gb300_sgemm_bf16x_run, "ozaki": L.gb300_dgemm_ozaki_run,
         "crt": L.gb300_dgemm_ozaki2_run}[form]
    return f(m, n, k, alpha, beta, _ptr(C), ldc, param, _ptr(workspace), workspace_bytes,
             c_void_p(stream))


def host_split_gemm(form, transa, transb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc,
                    param) -> int:
    """Host-pointer split forms ("bf16x", "ozaki" slices, "crt"; synchronous)."""
    L = core()
    f = {"bf16x": L.gb300_host_sgemm_bf16x, "ozaki": L.gb300_host_dgemm_ozaki,
         "crt": L.gb300_host_dgemm_ozaki2}[form]
    return f(_b(transa), _b(transb), m, n, k, alpha, _ptr(a), lda, _ptr(b), ldb, beta, _ptr(c),
             ldc, param)


def trsm(precision, side, uplo, transa, diag, m, n, alpha, A, lda, B, ldb, form=0,
         stream=0) -> int:
    """Triangular solve on device buffers (BLAS TRSM semantics); X overwrites B."""
    f = core().gb300_dtrsm if precision == "d" else core().gb300_strsm
    return f(_b(side), _b(uplo), _b(transa), _b(diag), m, n, alpha, _ptr(A), lda, _ptr(B), ldb,
             form, c_void_p(stream))


def trmm(precision, side, uplo, transa, diag, m, n, alpha, A, lda, B, ldb, form=0,
         stream=0) -> int:
    """Triangular multiply on device buffers (BLAS TRMM semantics), in place on B."""
    f = core().gb300_dtrmm if precision == "d" else core().gb300_strmm
    return f(_b(side), _b(uplo), _b(transa), _b(diag), m, n, alpha, _ptr(A), lda, _ptr(B), ldb,
             form, c_void_p(stream))


def complex_device(precision, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc,
                   method=CPLX_4M, param=0, workspace=None, workspace_bytes=0, stream=0) -> int:
    """gb300_zgemm / gb300_cgemm on device buffers (complex interleaved, ld in
    complex elements); stream-ordered, returns a status."""
    L = core()
    f = L.gb300_zgemm if precision == "z" else L.gb300_cgemm
    return f(_b(transa), _b(transb), m, n, k, _cscalar(alpha, precision), _ptr(A), lda, _ptr(B),
             ldb, _cscalar(beta, precision), _ptr(C), ldc, method, param, _ptr(workspace),
             workspace_bytes, c_void_p(stream))


def complex_workspace_bytes(precision, method, transb, m, n, k, param=0) -> int:
    return core().gb300_complex_workspace_bytes(1 if precision == "z" else 0, method, _b(transb),
                                                m, n, k, param)


def split_workspace_bytes(kind: int, m: int, n: int, k: int, param: int) -> int:
    return core().gb300_split_workspace_bytes(kind, m, n, k, param)


def device_error(clear: bool = False) -> int:
    return core().gb300_device_error(1 if clear else 0)


def selftest_wait_timeout(poll_limit: int = 4096) -> int:
    """Bounded-wait self-test: a kernel waits on an mbarrier nothing arrives on."""
    return core().gb300_selftest_wait_timeout(poll_limit)


TUNE_BF16X_CHUNK = 1
TUNE_GRAPH_BRANCHES = 2
TUNE_TILE_N = 3
TUNE_PAIR_MMA = 4
TUNE_HOST_PARTS = 5
TUNE_MODULUS_SPLIT = 6
TUNE_SPLIT_K = 7
TUNE_PLAIN_STAGES = 8
TUNE_BF16X = 0     # autotuner kinds
TUNE_OZAKI = 1
TUNE_CRT = 2
TUNE_PLAIN_D = 3
TUNE_PLAIN_S = 4


def autotune(kind, transa, transb, m, n, k, A, lda, B, ldb, stream=0):
    """Tune the split form for this shape class on these device operands.
    Returns (status, chosen products or slices)."""
    out = c_int(0)
    rc = core().gb300_autotune(kind, _b(transa), _b(transb), m, n, k, _ptr(A), lda, _ptr(B),
                               ldb, c_void_p(stream), ctypes.byref(out))
    return rc, out.value


def tune_lookup(kind, m, n, k):
    """(status, param, chunk) that products/slices = 0 resolve to for this shape."""
    p, c = c_int(0), c_int(0)
    rc = core().gb300_tune_lookup(kind, m, n, k, ctypes.byref(p), ctypes.byref(c))
    return rc, p.value, c.value


def tune_layout(kind, m, n, k):
    """(status, tile width, cluster mode) the split GEMMs use for this shape."""
    t, pm = c_int(0), c_int(0)
    rc = core().gb300_tune_layout(kind, m, n, k, ctypes.byref(t), ctypes.byref(pm))
    return rc, t.value, pm.value


def plain_layout(precision, m, n, k):
    """(status, split-K factor, ring depth) the plain kernels use for this shape."""
    sk, st = c_int(0), c_int(0)
    rc = core().gb300_plain_layout(1 if precision == "d" else 0, m, n, k, ctypes.byref(sk),
                                   ctypes.byref(st))
    return rc, sk.value, st.value


def tune_cache_save(path=None) -> int:
    return core().gb300_tune_cache_save(path.encode() if path else None)


def tune_cache_load(path=None):
    n = c_int(0)
    rc = core().gb300_tune_cache_load(path.encode() if path else None, ctypes.byref(n))
    return rc, n.value


def tune_cache_clear() -> None:
    core().gb300_tune_cache_clear()


class GemmProblem(ctypes.Structure):
    """gb300_gemm_problem of include/gemm_gb300.h (one problem of a grouped call)."""

    _fields_ = [("transa", c_char), ("transb", c_char), ("precision", c_char),
                ("m", c_int), ("n", c_int), ("k", c_int),
                ("alpha", c_double), ("beta", c_double),
                ("A", c_void_p), ("lda", c_int), ("B", c_void_p), ("ldb", c_int),
                ("C", c_void_p), ("ldc", c_int)]


def problem_array(problems):
    """A ctypes array of GemmProblem from dicts with keys precision, transa,
    transb, m, n, k, alpha, beta, A, lda, B, ldb, C, ldc (A/B/C device pointers)."""
    arr = (GemmProblem * len(problems))()
    for i, p in enumerate(problems):
        arr[i] = GemmProblem(_b(p["transa"]), _b(p["transb"]), _b(p["precision"]), p["m"],
                             p["n"], p["k"], p["alpha"], p["beta"], p["A"], p["lda"], p["B"],
                             p["ldb"], p["C"], p["ldc"])
    return arr


def gemm_grouped(problems, stream=0, workspace=None, workspace_bytes=0) -> int:
    """All problems' plain forms in one persistent launch (device-side tile scheduler)."""
    arr = problem_array(problems)
    L = core()
    if workspace is None:
        return L.gb300_gemm_grouped(ctypes.cast(arr, c_void_p), len(problems), c_void_p(stream))
    return L.gb300_gemm_grouped_ws(ctypes.cast(arr, c_void_p), len(problems), _ptr(workspace),
                                   workspace_bytes, c_void_p(stream))


def grouped_workspace_bytes(count: int) -> int:
    return core().gb300_grouped_workspace_bytes(count)


class GroupedGraph:
    """A fixed grouped batch captured into a CUDA graph (form 0 plain, 1 split)."""

    def __init__(self, problems, form=0):
        self.handle = c_void_p()
        arr = problem_array(problems)
        rc = core().gb300_grouped_graph_create(ctypes.cast(arr, c_void_p), len(problems), form,
                                               ctypes.byref(self.handle))
        if rc != OK:
            raise RuntimeError("gb300_grouped_graph_create failed: status %d" % rc)

    def launch(self, stream=0) -> int:
        return core().gb300_grouped_graph_launch(self.handle, c_void_p(stream))

    def stats(self):
        """(kernel nodes of the graph, of which GEMM launches)."""
        kn, gl = ctypes.c_int(0), ctypes.c_int(0)
        rc = core().gb300_grouped_graph_stats(self.handle, ctypes.byref(kn), ctypes.byref(gl))
        if rc != OK:
            raise RuntimeError("gb300_grouped_graph_stats failed: status %d" % rc)
        return kn.value, gl.value

    def destroy(self) -> None:
        if self.handle:
            core().gb300_grouped_graph_destroy(self.handle)
            self.handle = c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:  # noqa: BLE001
            pass


def tune_param(param: int, value: int) -> int:
    """Set a process-wide tuning knob (see include/gemm_gb300.h)."""
    return core().gb300_tune_param(param, value)


def version() -> str:
    return core().gb300_version().decode()


# Symbols every library must export (checked by the CPU tests).
CORE_SYMBOLS = [
    "gb300_host_dgemm", "gb300_host_sgemm", "gb300_dgemm", "gb300_sgemm", "gb300_sgemm_bf16x",
    "gb300_sgemm_bf16x_ws", "gb300_dgemm_ozaki", "gb300_dgemm_ozaki_ws",
    "gb300_split_workspace_bytes", "gb300_device_error", "gb300_version",
    "gb300_sgemm_bf16x_prepare", "gb300_sgemm_bf16x_run", "gb300_dgemm_ozaki_prepare",
    "gb300_dgemm_ozaki_run", "gb300_host_sgemm_bf16x", "gb300_host_dgemm_ozaki",
    "gb300_selftest_wait_timeout", "gb300_sgemm_bf16x_noalloc", "gb300_tune_param",
    "gb300_grouped_workspace_bytes", "gb300_gemm_grouped", "gb300_gemm_grouped_ws",
    "gb300_autotune", "gb300_tune_lookup", "gb300_tune_layout", "gb300_plain_layout",
    "gb300_tune_cache_save",
    "gb300_tune_cache_load",
    "gb300_tune_cache_clear", "gb300_dtrsm", "gb300_strsm", "gb300_dtrmm", "gb300_strmm",
    "gb300_grouped_graph_create", "gb300_grouped_graph_launch", "gb300_grouped_graph_destroy",
    "gb300_grouped_graph_stats",
    "gb300_cgemm", "gb300_zgemm", "gb300_host_cgemm", "gb300_host_zgemm",
    "gb300_complex_workspace_bytes", "gb300_dgemm_ozaki2", "gb300_host_dgemm_ozaki2",
    "gb300_dgemm_ozaki2_prepare", "gb300_dgemm_ozaki2_run",
]
