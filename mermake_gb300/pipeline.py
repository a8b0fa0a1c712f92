"""Batched per-FOV drivers (mermake/__main__.py:211-283 per image):

* ``hyb_spots``  -- one colour: every tile deconvolved, blurred, spot-called
  and keep-filtered in batches of tiles, rows appended on the device
  (``mm_hyb_spots``), instead of one Python iteration per tile.
* ``dapi_spots`` -- the DAPI block: stitched deconvolution, RMS, maxima of
  ``v/rms`` and of ``-v/rms`` (``mm_dapi_spots``), normalisation applied on read.

Both take the reference's TOML section as keyword arguments
(``**vars(args.hybs)`` / ``**vars(args.dapi)``), like the reference's ops.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from ._arrays import as_device


def _u16_channel(image):
    t = as_device(image)
    if t.dtype != torch.uint16:
        raise TypeError("the per-FOV drivers take uint16 channels (mermake/io.py:read_im)")
    if t.dim() != 3:
        raise ValueError("expected a (z, x, y) channel")
    if t.stride(-1) != 1:
        t = t.contiguous()
    return t


def _flat(flat, shape):
    if flat is None:
        return None
    f = as_device(flat, torch.float32)
    if f.dim() == 3:
        f = f[0]
    if tuple(f.shape) != tuple(shape[-2:]):
        raise ValueError("flat field must be (X, Y)")
    return f if f.stride(-1) == 1 else f.contiguous()


def _check_delta(delta):
    if delta > 5:
        raise TypeError("Delta must be an less than or equal to 5 due to MAX_KERNEL_POINTS")


def hyb_spots(dec, image, flat_field=None, *, threshold=None, delta=1, delta_fit=0, sigmaZ=1, sigmaXY=1.5,
              blur_radius=None, batch=0, capacity=1 << 18, stream=None, **kwargs):
    """Rows ``[zc, xc, yc, bg, a, habs, hn, h]`` of one colour, in FOV coordinates
    (mermake/__main__.py:253-265).  ``dec`` is a ``Deconvolver``."""
    _check_delta(delta)
    img = _u16_channel(image)
    fl = _flat(flat_field, img.shape)
    Z, X, Y = img.shape
    L = _lib.lib()
    th = float("nan") if threshold is None else float(threshold)
    br = -1 if blur_radius is None else int(blur_radius)
    cap = int(capacity)
    for _ in range(2):
        out = torch.empty((cap, 8), dtype=torch.float32, device=img.device)
        n = C.c_uint32(0)
        rc = L.mm_hyb_spots(_lib.ctx(img.device.index), _lib.ptr(img), Z, X, Y, img.stride(0), img.stride(1),
                            _lib.ptr(fl), fl.stride(0) if fl is not None else 0, _lib.ptr(dec.psf_fft),
                            dec.psf_fft.shape[0], _lib.ptr(dec.z_operator), dec.tile_size, dec.zpad, dec.overlap,
                            br, th, int(delta), int(delta_fit), float(sigmaZ), float(sigmaXY), int(batch),
                            _lib.ptr(out), cap, C.byref(n), _lib.stream_ptr(stream))
        if rc == _lib.MM_EOVERFLOW:
            cap = int(n.value)
            continue
        _lib.check(rc)
        return out[: n.value]
    raise _lib.MermakeError("spot rows did not fit after resizing")


def dapi_spots(dec, image, flat_field=None, *, threshold=None, delta=1, delta_fit=0, sigmaZ=1, sigmaXY=1.5,
               blur_radius=None, batch=0, buffer=None, capacity=1 << 16, stream=None, **kwargs):
    """``(Xh_plus, Xh_minus, buffer, rms)`` of the DAPI block
    (mermake/__main__.py:215-225); ``buffer`` holds the stitched deconvolution
    before normalisation."""
    _check_delta(delta)
    img = _u16_channel(image)
    fl = _flat(flat_field, img.shape)
    Z, X, Y = img.shape
    if buffer is None:
        buffer = torch.empty((Z, X, Y), dtype=torch.float32, device=img.device)
    L = _lib.lib()
    th = float("nan") if threshold is None else float(threshold)
    br = -1 if blur_radius is None else int(blur_radius)
    cp, cm = int(capacity), int(capacity)
    for _ in range(2):
        op = torch.empty((cp, 8), dtype=torch.float32, device=img.device)
        om = torch.empty((cm, 8), dtype=torch.float32, device=img.device)
        n_p, n_m, rms = C.c_uint32(0), C.c_uint32(0), C.c_float(0)
        rc = L.mm_dapi_spots(_lib.ctx(img.device.index), _lib.ptr(img), Z, X, Y, img.stride(0), img.stride(1),
                             _lib.ptr(fl), fl.stride(0) if fl is not None else 0, _lib.ptr(dec.psf_fft),
                             dec.psf_fft.shape[0], _lib.ptr(dec.z_operator), dec.tile_size, dec.zpad,
                             dec.overlap, br, th, int(delta), int(delta_fit), float(sigmaZ), float(sigmaXY),
                             int(batch), _lib.ptr(buffer), _lib.ptr(op), cp, C.byref(n_p), _lib.ptr(om), cm, C.byref(n_m), C.byref(rms),
                             _lib.stream_ptr(stream))
        if rc == _lib.MM_EOVERFLOW:
            cp, cm = max(cp, int(n_p.value)), max(cm, int(n_m.value))
            continue
        _lib.check(rc)
        return op[: n_p.value], om[: n_m.value], buffer, float(rms.value)
    raise _lib.MermakeError("spot rows did not fit after resizing")
