"""Build recipe of the native library (nvcc + gcc, no cmake).

Produces, in this package directory:
  libgemm_gb300.so  all CUDA kernels (sm_103a) + the gb300_* C ABI
  DGEMM.so          exports only dgemm_ (drop-in for the reference's DGEMM.so)
  SGEMM.so          exports only sgemm_ (drop-in for the reference's SGEMM.so)
  ZGEMM.so          exports zgemm_ and zgemm3m_ (complex BLAS symbols)
  CGEMM.so          exports cgemm_ and cgemm3m_
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
CU_SOURCES = ["plain_gemm.cu", "tc_gemm.cu", "grouped.cu", "autotune.cu", "trsm.cu", "api.cu",
              "noalloc.cu", "cplx.cu", "crt.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
                    "-I" + os.path.join(PKG, "..", "include")]
    if ptxas_info:
        flags += ["-Xptxas", "-v"]

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        out = _run([nvcc, *flags, "-c", os.path.join(CSRC, src), "-o", obj])
        return obj, out

    with ThreadPoolExecutor(max_workers=len(CU_SOURCES)) as ex:
        results = list(ex.map(compile_one, CU_SOURCES))
    log = "".join(o for _, o in results)
    objs = [o for o, _ in results]
    lib = os.path.join(PKG, "libgemm_gb300.so")
    _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", lib, *objs, "-lpthread", "-ldl"])
    cc = os.environ.get("CC", "gcc")
    for name, defs in (("DGEMM.so", ["-DDOUBLE"]), ("SGEMM.so", []),
                       ("ZGEMM.so", ["-DZCOMPLEX"]), ("CGEMM.so", ["-DCCOMPLEX"])):
        _run([cc, *defs, "-O2", "-fPIC", "-shared", "-fvisibility=hidden",
              os.path.join(CSRC, "dropin.c"), "-o", os.path.join(PKG, name),
              "-L" + PKG, "-lgemm_gb300", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        sys.stdout.write(log)
    return log


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
