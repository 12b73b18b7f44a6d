"""GPU test helpers: column-major numpy <-> device buffers (torch is only the
device-memory allocator here) and calls through the C ABI."""
from __future__ import annotations

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
