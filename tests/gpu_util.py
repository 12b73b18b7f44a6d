"""GPU test helpers: column-major numpy <-> device buffers (torch is only the
device-memory allocator here) and calls through the C ABI."""
from __future__ import annotations

import contextlib

import numpy as np


def torch_cuda():
    import torch

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch


def to_dev(X: np.ndarray):
    """Column-major (ld x cols) numpy array -> device buffer with the same layout."""
    torch = torch_cuda()
    Xf = np.asfortranarray(X)
    return torch.from_numpy(np.ascontiguousarray(Xf.T)).cuda()


def from_dev(t, rows: int) -> np.ndarray:
    """Device buffer written by to_dev -> column-major numpy (ld x cols)."""
    return np.asfortranarray(t.cpu().numpy().T)[:rows, :]


def sync():
    torch_cuda().cuda.synchronize()


@contextlib.contextmanager
def plain_unsplit():
    """The plain kernels with one K slice (split-K off): the full-K FMA / DMMA
    chain whose error the split forms' equal-error rule is measured against
    (the autotuner's bar; the plain kernel also runs unsplit at the benchmark
    shapes).  Split-K shortens the chains of few-tile shapes and lowers the
    plain kernel's own error there."""
    import gemm_avx2_gb300 as g

    assert g.tune_param(g.TUNE_SPLIT_K, 1) == g.OK
    try:
        yield
    finally:
        g.tune_param(g.TUNE_SPLIT_K, 0)
