"""Separable box blur with the reference's call surface (mermake/blur.py:15-188),
computed by ``k_box_1d`` in ``csrc/misc.cu``."""
from __future__ import annotations

import torch

from . import _lib
from ._arrays import as_device


def _launch(src, dst, size, axis):
    """One box_1d pass; src/dst are float32 2-D or 3-D CUDA tensors."""
    if src.dim() == 2:
        sz, (sx, sy) = 1, src.shape
        ins = [0] + list(src.stride())
        outs = [0] + list(dst.stride())
        axis = axis + 1
    else:
        sz, sx, sy = src.shape
        ins = list(src.stride())
        outs = list(dst.stride())
    _lib.check(_lib.lib().mm_box_1d_f32(_lib.ptr(src), _lib.i64arr(ins), _lib.ptr(dst), _lib.i64arr(outs),
                                        sz, sx, sy, int(size) // 2, axis, _lib.stream_ptr()))


def _overlaps(a, b):
    sa = a.untyped_storage().data_ptr()
    sb = b.untyped_storage().data_ptr()
    if sa != sb:
        return False
    ea = a.data_ptr() + (a.numel() and sum((n - 1) * s for n, s in zip(a.shape, a.stride())) + 1) * a.element_size()
    eb = b.data_ptr() + (b.numel() and sum((n - 1) * s for n, s in zip(b.shape, b.stride())) + 1) * b.element_size()
    return a.data_ptr() < eb and b.data_ptr() < ea


def box_1d(image, size, axis=0, out=None):
    """blur.py:157-188: mean over ``[c - size//2, c + size//2]`` clipped to the
    axis.  As in the reference, any negative axis means the last axis."""
    img = as_device(image)
    if img.dtype != torch.float32:
        raise AssertionError("Input must be float32")
    if out is None:
        out = torch.empty_like(img)
    o = as_device(out)
    if o.dtype != torch.float32:
        raise AssertionError("Output must be float32")
    if _overlaps(img, o):
        raise ValueError("In-place operation not supported - input and output must be different")
    if axis < 0:
        axis = img.dim() - 1
    if img.dim() == 2:
        if axis >= 2:
            raise AssertionError(f"axis {axis} is out of bounds for array of dimension 2")
    elif img.dim() != 3:
        raise ValueError("Only 2D or 3D arrays are supported")
    _launch(img, o, size, axis)
    return out


def box(image, size, axes=None, out=None, temp=None):
    """blur.py:15-129: blur along several axes in ascending order."""
    img = as_device(image)
    if img.dtype != torch.float32:
        img = img.to(torch.float32)
    if img.dim() not in (2, 3):
        raise ValueError("Only 2D or 3D arrays are supported")
    if axes is None:
        axes = tuple(range(img.dim()))
    elif isinstance(axes, int):
        axes = (axes,)
    elif not isinstance(axes, (tuple, list)):
        raise TypeError("axes must be None, int, tuple, or list")
    norm = []
    for a in axes:
        if a < 0:
            a = img.dim() + a
        if a < 0 or a >= img.dim():
            raise ValueError(f"axis {a} is out of bounds for array of dimension {img.dim()}")
        norm.append(a)
    axes = tuple(sorted(set(norm)))
    if len(axes) == 0:
        if out is None:
            return img.clone()
        as_device(out).copy_(img)
        return out
    if isinstance(size, int):
        sizes = {a: size for a in axes}
    elif isinstance(size, (tuple, list)):
        if len(size) != len(axes):
            raise ValueError(f"Size must have {len(axes)} elements for {len(axes)} axes")
        sizes = dict(zip(axes, size))
    else:
        raise TypeError("size must be an int, tuple, or list of ints")
    if out is None:
        out = torch.empty_like(img)
    o = as_device(out)
    if len(axes) == 1:
        _launch(img, o, sizes[axes[0]], axes[0])
        return out
    if temp is None:
        temp = torch.empty_like(img)
    elif tuple(temp.shape) != tuple(img.shape) or as_device(temp).dtype != img.dtype:
        raise ValueError("temp buffer must have same shape and dtype as input")
    t = as_device(temp)
    _launch(img, o, sizes[axes[0]], axes[0])
    for i in range(1, len(axes)):
        a = axes[i]
        if i % 2 == 1:
            _launch(o, t, sizes[a], a)
        else:
            _launch(t, o, sizes[a], a)
    if len(axes) % 2 == 0:
        o.copy_(t)
    return out


def box_2d(image, size, axes=(-2, -1), out=None):
    """blur.py:132-155."""
    if len(axes) != 2:
        raise ValueError("axes must contain exactly 2 elements for 2D blur")
    return box(image, size, axes=axes, out=out)
