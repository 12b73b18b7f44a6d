"""CPU tests of the C-ABI boundary: the libraries load, export exactly what
include/*.h declares (the drop-in libraries exactly one symbol each, like the
reference's DGEMM.so/SGEMM.so), and report argument errors without a GPU."""
import os
import re
import subprocess

import pytest

import gemm_avx2_gb300 as g

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    return {l.split()[-1] for l in out.splitlines() if re.match(r"^[0-9a-f]+ [TW] ", l)}


def header_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b((?:gb300_|[dszc]gemm(?:3m)?_)\w*)\s*\(", src))
    return names


@pytest.fixture(scope="module", autouse=True)
def built():
    if not os.path.exists(os.path.join(g.PKG, "libgemm_gb300.so")):
        g.build()


def test_dropin_exports_exactly_one_symbol():
    assert exported(os.path.join(g.PKG, "DGEMM.so")) == {"dgemm_"}
    assert exported(os.path.join(g.PKG, "SGEMM.so")) == {"sgemm_"}
    # the complex libraries: the BLAS symbol and its 3M twin, nothing else
    assert exported(os.path.join(g.PKG, "ZGEMM.so")) == {"zgemm_", "zgemm3m_"}
    assert exported(os.path.join(g.PKG, "CGEMM.so")) == {"cgemm_", "cgemm3m_"}


def test_core_exports_every_declared_function():
    decl = header_functions()
    assert {"dgemm_", "sgemm_", "gb300_dgemm", "gb300_sgemm"} <= decl
    core = exported(os.path.join(g.PKG, "libgemm_gb300.so"))
    dropin = set()
    for lib in ("DGEMM.so", "SGEMM.so", "ZGEMM.so", "CGEMM.so"):
        dropin |= exported(os.path.join(g.PKG, lib))
    missing = {n for n in decl if n not in core and n not in dropin}
    assert not missing, missing
    # nothing but the declared ABI is exported from the core library
    extra = {n for n in core if n.startswith("gb300_")} - decl
    assert not extra, extra
    assert set(g.CORE_SYMBOLS) <= core


def test_libraries_load_and_version():
    assert "sm_103a" in g.version()
    for p in "dszc":
        g.dropin(p)


def test_argument_errors_need_no_gpu():
    # invalid sizes / leading dimensions are rejected before any CUDA call
    assert g.gemm_device("d", "N", "N", -1, 4, 4, 1.0, 0, 4, 0, 4, 0.0, 0, 4) == g.ERR_ARG
    assert g.gemm_device("s", "N", "N", 8, 4, 4, 1.0, 0, 7, 0, 4, 0.0, 0, 8) == g.ERR_ARG
    assert g.gemm_device("s", "T", "N", 8, 4, 4, 1.0, 0, 3, 0, 4, 0.0, 0, 8) == g.ERR_ARG
    assert g.gemm_device("d", "N", "T", 8, 4, 4, 1.0, 0, 8, 0, 3, 0.0, 0, 8) == g.ERR_ARG
    assert g.gemm_device("d", "N", "N", 8, 4, 4, 1.0, 0, 8, 0, 4, 0.0, 0, 7) == g.ERR_ARG
    assert g.sgemm_bf16x("N", "N", 8, 8, 8, 1.0, 0, 8, 0, 8, 0.0, 0, 8, products=4) == g.ERR_ARG
    assert g.dgemm_ozaki("N", "N", 8, 8, 8, 1.0, 0, 8, 0, 8, 0.0, 0, 8, slices=1) == g.ERR_ARG
    assert g.dgemm_ozaki("N", "N", 8, 8, 8, 1.0, 0, 8, 0, 8, 0.0, 0, 8, slices=13) == g.ERR_ARG
    # empty problems are valid no-ops
    assert g.gemm_device("d", "N", "N", 0, 4, 4, 1.0, 0, 1, 0, 4, 0.0, 0, 1) == g.OK


@pytest.mark.parametrize("p", ["z", "c"])
def test_complex_argument_errors_need_no_gpu(p):
    cd = g.complex_device
    assert cd(p, "N", "N", -1, 4, 4, 1, 0, 4, 0, 4, 0, 0, 4) == g.ERR_ARG
    assert cd(p, "N", "N", 8, 4, 4, 1, 0, 7, 0, 4, 0, 0, 8) == g.ERR_ARG       # lda < m
    assert cd(p, "C", "N", 8, 4, 4, 1, 0, 3, 0, 4, 0, 0, 8) == g.ERR_ARG       # lda < k
    assert cd(p, "R", "N", 8, 4, 4, 1, 0, 7, 0, 4, 0, 0, 8) == g.ERR_ARG       # 'R' keeps m rows
    assert cd(p, "N", "C", 8, 4, 4, 1, 0, 8, 0, 3, 0, 0, 8) == g.ERR_ARG       # ldb < n
    assert cd(p, "N", "N", 8, 4, 4, 1, 0, 8, 0, 4, 0, 0, 7) == g.ERR_ARG       # ldc < m
    assert cd(p, "N", "N", 8, 4, 4, 1, 0, 8, 0, 4, 0, 0, 8, method=4) == g.ERR_ARG
    if p == "c":  # the CRT form is FP64 only
        assert cd(p, "N", "N", 8, 4, 4, 1, 0, 8, 0, 4, 0, 0, 8, method=g.CPLX_CRT) == g.ERR_ARG
    else:
        assert cd(p, "N", "N", 8, 4, 4, 1, 0, 8, 0, 4, 0, 0, 8, method=g.CPLX_CRT,
                  param=25) == g.ERR_ARG
    bad = 5 if p == "c" else 13
    assert cd(p, "N", "N", 8, 4, 4, 1, 0, 8, 0, 4, 0, 0, 8, method=g.CPLX_SPLIT,
              param=bad) == g.ERR_ARG
    assert g.host_complex(p, "N", "N", 8, 4, 4, 1, None, 7, None, 4, 0, None, 8) == g.ERR_ARG
    assert cd(p, "N", "N", 0, 4, 4, 1, 0, 1, 0, 4, 0, 0, 1) == g.OK


def test_complex_workspace_sizes():
    m, n, k = 300, 200, 100
    for p, e in (("z", 8), ("c", 4)):
        w4 = g.complex_workspace_bytes(p, g.CPLX_4M, "N", m, n, k)
        assert w4 >= 2 * m * 2 * k * e                       # the embedded op(A)
        if p == "z":   # B is used in place when transb is 'N'
            assert g.complex_workspace_bytes(p, g.CPLX_4M, "T", m, n, k) >= w4 + 2 * k * n * e
        else:          # FP32 4M always stores op(B) transposed (MN-major for the FFMA kernel)
            assert w4 >= (2 * m + n) * 2 * k * e
        w3 = g.complex_workspace_bytes(p, g.CPLX_3M, "N", m, n, k)
        assert w3 >= 3 * (m * k + k * n + m * n) * e
        ws = g.complex_workspace_bytes(p, g.CPLX_SPLIT, "N", m, n, k, 8 if p == "z" else 6)
        assert ws > w4
        assert g.complex_workspace_bytes(p, g.CPLX_4M, "N", 0, n, k) == 0


def test_workspace_sizes():
    assert g.split_workspace_bytes(0, 0, 8, 8, 3) == 0
    w3 = g.split_workspace_bytes(0, 8192, 8192, 8192, 3)
    w6 = g.split_workspace_bytes(0, 8192, 8192, 8192, 6)
    # each split term stored once: 2 BF16 terms per element for P = 3, 3 for P = 6
    assert w3 >= (8192 + 8192) * 2 * 8192 * 2 and w6 >= (8192 + 8192) * 3 * 8192 * 2
    assert w6 >= w3 * 3 // 2 - 4096
    assert g.split_workspace_bytes(0, 10, 10, 10, 5) == 0
    wo = g.split_workspace_bytes(1, 1000, 1000, 1000, 8)
    assert wo >= 8 * (1024 + 1024) * 1024 * 2


def test_dropin_invalid_args_leave_c_untouched():
    import numpy as np
    c = np.arange(12, dtype=np.float64).reshape(3, 4, order="F").copy(order="F")
    before = c.copy()
    a = np.ones((3, 3), order="F")
    g.dgemm("N", "N", 3, 4, 3, 1.0, a, 2, a, 3, 0.0, c, 3)  # lda < m
    assert np.array_equal(c, before)
    g.dgemm("N", "N", 3, -4, 3, 1.0, a, 3, a, 3, 0.0, c, 3)
    assert np.array_equal(c, before)
    z = (np.arange(12) + 1j).reshape(3, 4, order="F").astype(np.complex128, order="F")
    zb = z.copy()
    za = np.ones((3, 3), np.complex128, order="F")
    g.zgemm("N", "N", 3, 4, 3, 1.0, za, 2, za, 3, 0.0, z, 3)   # lda < m
    g.zgemm("C", "N", 3, 4, 3, 1.0, za, 3, za, 3, 0.0, z, 2, method3m=True)  # ldc < m
    assert np.array_equal(z, zb)


def test_grouped_problem_struct_layout_and_args():
    import ctypes
    P = g.GemmProblem
    # LP64 layout of gb300_gemm_problem (x86-64 and aarch64 alike)
    assert ctypes.sizeof(P) == 80
    assert (P.m.offset, P.alpha.offset, P.A.offset, P.lda.offset, P.B.offset, P.C.offset,
            P.ldc.offset) == (4, 16, 32, 40, 48, 64, 72)
    bad = dict(precision="d", transa="N", transb="N", m=4, n=4, k=4, alpha=1.0, beta=0.0,
               A=0, lda=3, B=0, ldb=4, C=0, ldc=4)
    assert g.gemm_grouped([bad]) == g.ERR_ARG          # lda < m, checked before any CUDA call
    bad2 = dict(bad, lda=4, precision="z")
    assert g.gemm_grouped([bad2]) == g.ERR_ARG
    assert g.gemm_grouped([]) == g.OK


def test_tune_cache_roundtrip_and_corruption(tmp_path):
    g.tune_cache_clear()
    # defaults without a tuned entry
    assert g.tune_lookup(g.TUNE_OZAKI, 1000, 1000, 1000) == (g.ERR_UNSUPPORTED, 8, 0)
    assert g.tune_lookup(g.TUNE_BF16X, 1000, 1000, 1000) == (g.ERR_UNSUPPORTED, 6, 0)
    assert g.tune_lookup(g.TUNE_CRT, 1000, 1000, 1000) == (g.ERR_UNSUPPORTED, 16, 0)
    # a hand-written cache file with good, malformed and out-of-range lines
    f = tmp_path / "tune.json"
    f.write_text('{"version": 1, "entries": [\n'
                 '  {"key": "ozaki:9:9:9", "param": 10, "chunk": 0, "ms": 1, "err_max": 1e-14, '
                 '"err_fro": 1e-16, "plain_max": 2e-14, "plain_fro": 1e-15},\n'
                 '  {"key": "bf16x:9:9:9", "param": 3, "chunk": 8, "ms": 1, "err_max": 1e-5, '
                 '"err_fro": 1e-7, "plain_max": 2e-5, "plain_fro": 1e-6},\n'
                 '  {"key": "bf16x:12:12:12", "param": 259, "chunk": 4, "ms": 1, "err_max": 1e-5, '
                 '"err_fro": 1e-7, "plain_max": 2e-5, "plain_fro": 1e-6, "tile": 128},\n'
                 '  {"key": "ozaki:8:8:8", "param": 99, "chunk": 0, "ms": 1, "err_max": 0, '
                 '"err_fro": 0, "plain_max": 0, "plain_fro": 0},\n'
                 '  {"key": "crt:9:9:9", "param": 14, "chunk": 0, "ms": 1, "err_max": 1e-14, '
                 '"err_fro": 1e-16, "plain_max": 2e-14, "plain_fro": 1e-15},\n'
                 '  {"key": "crt:8:8:8", "param": 25, "chunk": 0, "ms": 1, "err_max": 0, '
                 '"err_fro": 0, "plain_max": 0, "plain_fro": 0},\n'
                 '  garbage line\n]}\n')
    assert g.tune_cache_load(str(f)) == (g.OK, 4)
    assert g.tune_lookup(g.TUNE_CRT, 1000, 600, 700) == (g.OK, 14, 0)
    # the scaled FP16 form is a valid tuned choice and sizes the workspace
    assert g.tune_lookup(g.TUNE_BF16X, 4096, 5000, 8000) == (g.OK, g.FP16X3, 4)
    assert g.split_workspace_bytes(0, 4096, 5000, 8000, 0) == \
        g.split_workspace_bytes(0, 4096, 5000, 8000, g.FP16X3)
    assert g.tune_lookup(g.TUNE_CRT, 300, 300, 300)[0] == g.ERR_UNSUPPORTED   # 25 rejected
    # moduli = 0 sizes the workspace with the tuned count
    assert g.split_workspace_bytes(2, 1000, 600, 700, 0) == g.split_workspace_bytes(2, 1000, 600, 700, 14)
    assert g.tune_lookup(g.TUNE_OZAKI, 1000, 600, 700) == (g.OK, 10, 0)      # log2 buckets 9
    assert g.tune_lookup(g.TUNE_BF16X, 512, 1023, 600) == (g.OK, 3, 8)
    assert g.tune_lookup(g.TUNE_OZAKI, 300, 300, 300)[0] == g.ERR_UNSUPPORTED  # rejected entry
    assert g.split_workspace_bytes(0, 512, 512, 512, 0) == g.split_workspace_bytes(0, 512, 512, 512, 3)
    out = tmp_path / "saved.json"
    assert g.tune_cache_save(str(out)) == g.OK
    assert '"key": "bf16x:12:12:12", "param": 259, "chunk": 4' in out.read_text()
    assert '"tile": 128, "pair": 0, "stages": 0}' in out.read_text()
    g.tune_cache_clear()
    assert g.tune_cache_load(str(out)) == (g.OK, 4)
    assert g.tune_cache_load(str(tmp_path / "missing.json"))[0] == g.ERR_ARG
    assert g.tune_lookup(g.TUNE_OZAKI, 1000, 600, 700) == (g.OK, 10, 0)        # cache kept
    g.tune_cache_clear()


def test_tuning_knobs_validate():
    assert g.tune_param(g.TUNE_TILE_N, 128) == g.OK
    assert g.tune_param(g.TUNE_TILE_N, 192) == g.ERR_ARG
    assert g.tune_param(g.TUNE_TILE_N, 0) == g.OK
    assert g.tune_param(g.TUNE_PAIR_MMA, 2) == g.OK
    assert g.tune_param(g.TUNE_PAIR_MMA, 3) == g.ERR_ARG
    assert g.tune_param(g.TUNE_PAIR_MMA, 0) == g.OK
    assert g.tune_param(g.TUNE_GRAPH_BRANCHES, 64) == g.OK
    assert g.tune_param(g.TUNE_GRAPH_BRANCHES, 65) == g.ERR_ARG
    assert g.tune_param(g.TUNE_GRAPH_BRANCHES, -1) == g.ERR_ARG
    assert g.tune_param(g.TUNE_GRAPH_BRANCHES, 0) == g.OK   # back to the default
    assert g.tune_param(g.TUNE_HOST_PARTS, 8) == g.OK
    assert g.tune_param(g.TUNE_HOST_PARTS, 9) == g.ERR_ARG
    assert g.tune_param(g.TUNE_HOST_PARTS, 0) == g.OK
    assert g.tune_param(g.TUNE_MODULUS_SPLIT, 2) == g.OK
    assert g.tune_param(g.TUNE_MODULUS_SPLIT, 3) == g.ERR_ARG
    assert g.tune_param(g.TUNE_MODULUS_SPLIT, 0) == g.OK
    assert g.tune_param(g.TUNE_SPLIT_K, 65535) == g.OK
    assert g.tune_param(g.TUNE_SPLIT_K, 65536) == g.ERR_ARG
    assert g.tune_param(g.TUNE_SPLIT_K, -1) == g.ERR_ARG
    assert g.tune_param(g.TUNE_SPLIT_K, 0) == g.OK
    assert g.tune_param(g.TUNE_PLAIN_STAGES, 6) == g.OK
    assert g.tune_param(g.TUNE_PLAIN_STAGES, 5) == g.ERR_ARG
    assert g.tune_param(g.TUNE_PLAIN_STAGES, 0) == g.OK
    assert g.tune_param(99, 1) == g.ERR_ARG


def test_plain_split_k_by_shape_and_cache(tmp_path):
    """Host logic of the plain kernels' split-K (no GPU needed): many waves of
    128 x 128 tiles stay unsplit; a few tiles with a long K are split, at
    least 8 k-tiles a slice; a tuned entry and the knob win."""
    g.tune_cache_clear()
    assert g.plain_layout("d", 8192, 8192, 8192)[1:] == (1, 4)     # 4096 tiles
    assert g.plain_layout("d", 32768, 32768, 256)[1] == 1           # rank-256 update
    assert g.plain_layout("d", 2048, 2048, 2048)[1] > 1             # 1.7 waves
    rc, sk, st = g.plain_layout("d", 256, 256, 65536)               # 4 tiles, 4096 k-tiles
    assert rc == g.ERR_UNSUPPORTED and 16 <= sk <= 32 and st == 4
    assert g.plain_layout("s", 256, 256, 100)[1] == 1               # 4 k-tiles: too short
    sk = g.plain_layout("s", 300, 200, 20000)[1]
    assert 2 <= sk <= 32 and (20000 + 31) // 32 // sk >= 8
    assert g.tune_param(g.TUNE_SPLIT_K, 5) == g.OK
    try:
        assert g.plain_layout("d", 8192, 8192, 8192)[1] == 5
        assert g.plain_layout("d", 100, 100, 40)[1] == 3            # at most one per k-tile
    finally:
        g.tune_param(g.TUNE_SPLIT_K, 0)
    f = tmp_path / "plain.json"
    f.write_text('{"version": 1, "entries": [\n'
                 '  {"key": "plain_d:8:8:16", "param": 6, "chunk": 0, "ms": 1, "err_max": 0, '
                 '"err_fro": 0, "plain_max": 0, "plain_fro": 0, "tile": 0, "pair": 0, '
                 '"stages": 6},\n'
                 '  {"key": "plain_s:8:8:16", "param": 33, "chunk": 0, "ms": 1, "err_max": 0, '
                 '"err_fro": 0, "plain_max": 0, "plain_fro": 0},\n'
                 ']}\n')
    assert g.tune_cache_load(str(f)) == (g.OK, 1)                   # split 33 rejected
    assert g.plain_layout("d", 256, 256, 65536) == (g.OK, 6, 6)
    assert g.tune_lookup(g.TUNE_PLAIN_D, 256, 256, 65536) == (g.OK, 6, 0)
    g.tune_cache_clear()
