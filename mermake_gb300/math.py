"""uint16 subtraction without wrap-around (mermake/math.py:1-33), computed by
``k_subtract_u16`` in ``csrc/misc.cu``."""
from __future__ import annotations

import torch

from . import _lib
from ._arrays import as_device


def _sub(x, y, out, mode):
    a = as_device(x)
    b = as_device(y)
    if a.dtype != torch.uint16 or b.dtype != torch.uint16:
        raise TypeError("subtract_* take uint16 arrays")
    if tuple(a.shape) != tuple(b.shape):
        raise ValueError("operands must have the same shape")
    if out is None:
        out = torch.empty(a.shape, dtype=torch.uint16, device=a.device)
    o = as_device(out)
    shape = list(a.shape) or [1]
    _lib.check(_lib.lib().mm_subtract_u16(_lib.ptr(a), _lib.i64arr(a.stride() or [1]), _lib.ptr(b),
                                          _lib.i64arr(b.stride() or [1]), _lib.ptr(o), _lib.i64arr(o.stride() or [1]),
                                          len(shape), _lib.i64arr(shape), mode, _lib.stream_ptr()))
    return out


def subtract_clamp(x, y, out=None):
    """math.py:4-17: x - y, floored at 0."""
    return _sub(x, y, out, 0)


def subtract_reflect(x, y, out=None):
    """math.py:20-33: |x - y|."""
    return _sub(x, y, out, 1)
