"""Array plumbing: accept torch tensors, CUDA arrays (``__cuda_array_interface__``
or DLPack, e.g. CuPy) and NumPy arrays; hand device tensors to the library."""
from __future__ import annotations

import numpy as np
import torch


def as_device(a, dtype=None, device=None):
    """Returns a CUDA torch tensor viewing (or holding a copy of) ``a``."""
    if isinstance(a, torch.Tensor):
        t = a
    elif hasattr(a, "__cuda_array_interface__") or hasattr(a, "__dlpack__") and not isinstance(a, np.ndarray):
        t = torch.as_tensor(a, device="cuda")
    else:
        t = torch.from_numpy(np.ascontiguousarray(a))
    if not t.is_cuda:
        t = t.to(device or "cuda", non_blocking=False)
    if dtype is not None and t.dtype != dtype:
        t = t.to(dtype)
    return t


def torch_dtype(np_dtype):
    return {np.dtype(np.float32): torch.float32, np.dtype(np.uint16): torch.uint16,
            np.dtype(np.float64): torch.float64, np.dtype(np.int32): torch.int32}[np.dtype(np_dtype)]


def dense_yz(t):
    """True if the last axis is contiguous (the layout the kernels take)."""
    return t.dim() == 0 or t.stride(-1) == 1 or t.shape[-1] == 1


def elem_strides(t):
    return [int(s) for s in t.stride()]
