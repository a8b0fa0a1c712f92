"""``reflect`` with the reference's call surface (mermake/fill.py:54-111),
computed by ``k_mirror`` in ``csrc/misc.cu``."""
from __future__ import annotations

import torch

from . import _lib
from ._arrays import as_device


def reflect(arr, i, axis=0, mode="out", out=None):
    """Mirror about index ``i`` along ``axis``: 'out' sets a[j] = a[2i-j] for
    j > i, 'in' for j < i; sources outside the axis are skipped."""
    a = as_device(arr)
    if out is None:
        result = a.clone()
        ret = result
    else:
        o = as_device(out)
        if tuple(o.shape) != tuple(a.shape):
            raise ValueError(f"output array shape {tuple(o.shape)} does not match input shape {tuple(a.shape)}")
        if o.dtype != a.dtype:
            raise ValueError(f"output array dtype {o.dtype} does not match input dtype {a.dtype}")
        if o.data_ptr() != a.data_ptr() or o.stride() != a.stride():
            o.copy_(a)
        result, ret = o, out
    if axis < 0:
        axis += result.dim()
    if axis < 0 or axis >= result.dim():
        raise IndexError(f"axis {axis} is out of bounds for array of dimension {result.dim()}")
    n = result.shape[axis]
    if i < 0:
        i += n
    if i < 0 or i >= n:
        raise IndexError(f"index {i} is out of bounds for axis {axis} with size {n}")
    if mode == "out":
        m = 0
    elif mode == "in":
        m = 1
    else:
        raise ValueError("mode must be 'out' or 'in'")
    if result.dtype != torch.float32:
        raise TypeError("reflect supports float32 arrays (the reference kernel is float-only)")
    _lib.check(_lib.lib().mm_reflect_f32(_lib.ptr(result), result.dim(), _lib.i64arr(result.shape),
                                         _lib.i64arr(result.stride()), axis, int(i), m, _lib.stream_ptr()),
               IndexError)
    return ret
