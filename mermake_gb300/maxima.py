"""``find_local_maxima`` with the reference's signature (mermake/maxima.py:17-98),
computed by the sm_103a kernels of ``csrc/maxima.cu``."""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from ._arrays import as_device


def _prep(t):
    if t.dim() != 3:
        raise ValueError("find_local_maxima expects a 3-D (z, x, y) volume")
    if t.stride(-1) != 1 and t.shape[-1] > 1:
        t = t.contiguous()
    return t


def find_local_maxima(image, threshold=None, delta=1, delta_fit=0, raw=None, sigmaZ=1, sigmaXY=1.5, *,
                      norm_div=0.0, negate=False, stream=None, **kwargs):
    """Local maxima of a float32 (Z, X, Y) volume with the per-spot fit.

    Returns a (N, 8) float32 CUDA tensor of rows
    ``[zc, xc, yc, background, a, habs, hn, h]`` (row order unspecified, as in
    the reference).  ``threshold=None`` admits every voxel (the reference's
    ``float32(None)`` is NaN and its ``<=`` test never rejects).  ``raw`` of
    any dtype is read as float32; ``raw=None`` uses the image itself.
    ``norm_div`` / ``negate`` read the image as ``-(v / norm_div)`` without
    writing it (the DAPI normalisation, mermake/__main__.py:221-225).
    """
    if delta > 5:
        raise TypeError("Delta must be an less than or equal to 5 due to MAX_KERNEL_POINTS")
    img = _prep(as_device(image, torch.float32))
    Z, X, Y = img.shape
    if raw is None:
        raw = img
    rw = as_device(raw)
    if rw.dtype not in (torch.float32, torch.uint16):
        rw = rw.to(torch.float32)
    rw = _prep(rw)
    if tuple(rw.shape) != (Z, X, Y):
        raise ValueError("raw must have the image's shape")
    th = float("nan") if threshold is None else float(threshold)
    L = _lib.lib()
    ctx = _lib.ctx(img.device.index)
    st = _lib.stream_ptr(stream)
    cap = 1 << 16
    for _ in range(2):
        out = torch.zeros((cap, 8), dtype=torch.float32, device=img.device)
        n = C.c_uint32(0)
        rc = L.mm_find_local_maxima(ctx, _lib.ptr(img), Z, X, Y, img.stride(0), img.stride(1), _lib.ptr(rw),
                                    1 if rw.dtype == torch.uint16 else 0, rw.stride(0), rw.stride(1), th,
                                    int(delta), int(delta_fit), float(sigmaZ), float(sigmaXY), float(norm_div),
                                    int(bool(negate)), _lib.ptr(out), cap, C.byref(n), st)
        if rc == _lib.MM_EOVERFLOW:
            cap = int(n.value)
            continue
        _lib.check(rc)
        return out[: n.value]
    raise _lib.MermakeError("maxima output did not fit after resizing")
