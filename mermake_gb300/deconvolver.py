"""``Deconvolver`` / ``full_deconv`` with the reference's call surface
(mermake/deconvolver.py:47-287), computed by the sm_103a kernels of
``csrc/deconv.cu`` and ``csrc/wiener.cu``.

Differences a caller can see:

* ``psf_fft`` holds the Wiener spectra as Hermitian half spectra
  ``(n_psf, Zp, P, P//2+1)`` complex64, pre-divided by ``Zp*P*P`` (the
  inverse transform's normalisation), instead of full spectra.
* Yielded tiles and outputs are torch CUDA tensors.
* ``zpad = 0`` raises ``ValueError`` up front (the reference fails later
  with a broadcast error, because ``[zpad:-zpad]`` is empty).
"""
from __future__ import annotations

import gc

import numpy as np
import torch

from . import _lib
from ._arrays import as_device

MM_DTYPE_F32, MM_DTYPE_U16 = 0, 1


def laplacian_3d(shape):
    """deconvolver.py:24-36 (host array, float16 like the reference)."""
    lap = np.zeros(shape, dtype=np.float16)
    z_c, y_c, x_c = shape[0] // 2, shape[1] // 2, shape[2] // 2
    lap[z_c, y_c, x_c] = 6
    lap[z_c - 1, y_c, x_c] = -1
    lap[z_c + 1, y_c, x_c] = -1
    lap[z_c, y_c - 1, x_c] = -1
    lap[z_c, y_c + 1, x_c] = -1
    lap[z_c, y_c, x_c - 1] = -1
    return lap


def _channel(image):
    """Device view of a (Z, X, Y) channel as uint16 or float32 with y contiguous."""
    t = as_device(image)
    if t.dim() != 3:
        raise ValueError("expected a 3-D (z, x, y) image")
    if t.dtype == torch.uint16:
        dt = MM_DTYPE_U16
    else:
        if t.dtype != torch.float32:
            t = t.to(torch.float32)
        dt = MM_DTYPE_F32
    if t.stride(-1) != 1 and t.shape[-1] > 1:
        t = t.contiguous()
    return t, dt


def _flat2d(flat_field, shape):
    if flat_field is None:
        return None
    f = as_device(flat_field, torch.float32)
    if f.dim() == 3:
        if f.shape[0] != 1:
            raise NotImplementedError("per-plane flat fields are not supported; pass (X, Y) or (1, X, Y)")
        f = f[0]
    if f.dim() != 2 or tuple(f.shape) != tuple(shape[-2:]):
        raise ValueError("flat_field must be (X, Y) matching the image")
    if f.stride(-1) != 1:
        f = f.contiguous()
    return f


class Deconvolver:
    """Tiled Wiener deconvolution (deconvolver.py:47-236)."""

    def __init__(self, psfs, channel_shape, tile_size=300, zpad=0, overlap=89, beta=0.001, xp=None, **kwargs):
        self.tile_size = int(tile_size)
        self.tile_height = int(channel_shape[0])
        self.overlap = int(overlap)
        self.zpad = int(zpad)
        self.beta = float(beta)
        self.Zp = self.tile_height + 2 * self.zpad
        self.P = self.tile_size + 2 * self.overlap
        self.H = self.P // 2 + 1
        if isinstance(psfs, dict):
            plist = list(psfs.values())
        else:
            plist = [psfs]
        L = _lib.lib()
        ctx = _lib.ctx()
        st = _lib.stream_ptr()
        self.psf_fft = torch.empty((len(plist), self.Zp, self.P, self.H, 2), dtype=torch.float32, device="cuda")
        for i, p in enumerate(plist):
            pd = as_device(np.asarray(p, dtype=np.float32) if not isinstance(p, torch.Tensor) else p,
                           torch.float32).contiguous()
            if pd.dim() != 3:
                raise ValueError("a PSF must be 3-D")
            _lib.check(L.mm_wiener_spectrum(ctx, _lib.ptr(pd), *pd.shape, self.tile_height, self.tile_size,
                                            self.zpad, self.overlap, self.beta, _lib.ptr(self.psf_fft[i]), st))
        self.psf_fft = torch.view_as_complex(self.psf_fft)
        self.z_operator = None
        if self._want_z_operator(kwargs.get("z_operator")):
            self.z_operator = torch.empty_like(self.psf_fft)
            for i in range(self.psf_fft.shape[0]):
                _lib.check(L.mm_wiener_zop(ctx, _lib.ptr(self.psf_fft[i]), self.tile_height, self.zpad,
                                           self.tile_size, self.overlap, _lib.ptr(self.z_operator[i]), st))
        if self.tile_size:
            shape = (self.tile_height, self.P, self.P)
            self.tile_res = torch.empty(shape, dtype=torch.float32, device="cuda")
            self.tile_raw = torch.empty(shape, dtype=torch.float32, device="cuda")

    # z kernels: the z step of a tile (padding by reflection, transforms over
    # Zp, times the spectrum, crop) is, per (x, y) frequency, a sum over the
    # padded planes weighted by the inverse DFT of the spectrum along z
    # (csrc/zop.cu).  One kernel per spectrum, the size of psf_fft, kept
    # beside it.  With one PSF and batches of >= 10 tiles the sum runs as a
    # Z x Z matrix per frequency over the batch; otherwise directly per tile.
    def _want_z_operator(self, request):
        ok = bool(self.tile_size) and bool(_lib.lib().mm_zkernel_supported(self.tile_height, self.zpad))
        if request is True and not ok:
            raise ValueError("z_operator needs zpad >= 1, tile height <= 128 and padded depth <= 400 "
                             "(with the z kernel's staging in shared memory)")
        return ok and request is not False

    # -- geometry ------------------------------------------------------------
    def tile_boxes(self, shape):
        """(x, y, x0, x1, y0, y1) per tile, x-major (deconvolver.py:186-206)."""
        _, sx, sy = shape
        ts, ov = self.tile_size, self.overlap
        return [(x, y, max(x - ov, 0), min(x + ts + ov, sx), max(y - ov, 0), min(y + ts + ov, sy))
                for x in range(0, sx, ts) for y in range(0, sy, ts)]

    def tiled(self, image):
        """deconvolver.py:186-206: yields (x, y, tile view)."""
        sz, sx, sy = image.shape
        self.nx = -(-sx // self.tile_size)
        self.ny = -(-sy // self.tile_size)
        for x, y, x0, x1, y0, y1 in self.tile_boxes(image.shape):
            yield x, y, image[:, x0:x1, y0:y1]

    def _extent(self, box):
        x, y, x0, x1, y0, y1 = box
        xd, yd = x1 - x0, y1 - y0
        xend = xd + (self.overlap if (x == 0 or xd < self.P) else 0)
        yend = yd + (self.overlap if (y == 0 or yd < self.P) else 0)
        # the reference's tile_res[:, :xend, :yend] clips at the padded size
        return min(xend, self.P), min(yend, self.P)

    def n_tiles(self, shape):
        n = len(self.tile_boxes(shape))
        npsf = self.psf_fft.shape[0]
        return n if npsf == 1 else min(n, npsf)

    def _call(self, img, dt, flat, t0, nt, blur_radius, res_out=None, raw_out=None, stitch=None, stream=None):
        L = _lib.lib()
        Z, X, Y = img.shape
        br = -1 if blur_radius is None else int(blur_radius)
        _lib.check(L.mm_deconv_tiles(
            _lib.ctx(), _lib.ptr(img), dt, Z, X, Y, img.stride(0), img.stride(1), _lib.ptr(flat),
            flat.stride(0) if flat is not None else 0, _lib.ptr(self.psf_fft), self.psf_fft.shape[0],
            _lib.ptr(self.z_operator), self.tile_size, self.zpad, self.overlap, t0, nt, br, _lib.ptr(res_out),
            _lib.ptr(raw_out), _lib.ptr(stitch), stitch.stride(0) if stitch is not None else 0,
            stitch.stride(1) if stitch is not None else 0, _lib.stream_ptr(stream)))

    def _check_image(self, img):
        if img.shape[0] != self.tile_height:
            raise ValueError("image depth %d does not match the Deconvolver's %d" % (img.shape[0], self.tile_height))

    # -- reference surface -----------------------------------------------------
    def tile_wise(self, image, flat_field=None, blur_radius=None, **kwargs):
        """deconvolver.py:98-170.  Yields ``(x, y, tile_res[:, :xend, :yend],
        raw[:, :xend, :yend])``; both are views of this object's buffers, valid
        until the next iteration, as in the reference."""
        img, dt = _channel(image)
        self._check_image(img)
        flat = _flat2d(flat_field, img.shape)
        boxes = self.tile_boxes(img.shape)[: self.n_tiles(img.shape)]
        for i, box in enumerate(boxes):
            self._call(img, dt, flat, i, 1, blur_radius, res_out=self.tile_res, raw_out=self.tile_raw)
            xend, yend = self._extent(box)
            yield box[0], box[1], self.tile_res[:, :xend, :yend], self.tile_raw[:, :xend, :yend]

    def apply(self, image, flat_field=None, blur_radius=None, output=None, batch=None, **kwargs):
        """deconvolver.py:172-184: every tile's centre stitched into ``output``
        (float32 (Z, X, Y); allocated when None).  Tiles run ``batch`` at a time
        (default: all)."""
        img, dt = _channel(image)
        self._check_image(img)
        flat = _flat2d(flat_field, img.shape)
        if output is None:
            output = torch.empty(img.shape, dtype=torch.float32, device=img.device)
        out = as_device(output)
        if out.dtype != torch.float32 or tuple(out.shape) != tuple(img.shape) or out.stride(-1) != 1:
            raise ValueError("output must be a float32 (Z, X, Y) CUDA array with y contiguous")
        n = self.n_tiles(img.shape)
        b = n if not batch else int(batch)
        for t0 in range(0, n, b):
            self._call(img, dt, flat, t0, min(b, n - t0), blur_radius, stitch=out)
        return output

    def center_psf(self, psf):
        """deconvolver.py:238-270 (host NumPy utility, as in the reference)."""
        psf = np.asarray(psf)
        tgt = np.array([self.tile_height, self.tile_size, self.tile_size])
        ps = np.array(psf.shape)
        out = np.zeros(tuple(tgt), dtype=psf.dtype)
        s0 = np.maximum(0, (tgt - ps) // 2)
        e0 = s0 + np.minimum(tgt, ps)
        s1 = np.maximum(0, (ps - tgt) // 2)
        e1 = s1 + np.minimum(tgt, ps)
        out[tuple(slice(int(a), int(b)) for a, b in zip(s0, e0))] = \
            psf[tuple(slice(int(a), int(b)) for a, b in zip(s1, e1))]
        out /= out.sum()
        return out


def full_deconv(image, psfs, flat_field=None, tile_size=300, zpad=None, overlap=1, beta=0.001):
    """deconvolver.py:272-287."""
    shape = tuple(image.shape)
    if zpad is None:
        zpad = shape[0]
    d = Deconvolver(psfs, channel_shape=shape, zpad=zpad, tile_size=tile_size, overlap=overlap, beta=beta)
    out = d.apply(image, flat_field)
    del d
    gc.collect()
    return out
