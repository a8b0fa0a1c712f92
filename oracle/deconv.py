"""FP64 NumPy/SciPy restatement of ``mermake/deconvolver.py`` (test oracle only).

Every function names the reference lines it restates.  Arithmetic follows the
reference's order of operations where it is observable (the tile is placed and
flat-divided in float32, reflect padding copies float32 values, the raw view is
re-multiplied in float32); the FFT, Wiener multiply and box blur run in float64
so that the oracle is more accurate than either implementation under test.
"""
from __future__ import annotations

import os

import numpy as np
import scipy.fft as sfft

WORKERS = os.cpu_count() or 1


# --------------------------------------------------------------------------
# Wiener spectrum (deconvolver.py:24-36, 48-75, 238-270)
# --------------------------------------------------------------------------
def laplacian_3d(shape):
    """deconvolver.py:24-36.  6 at the centre, -1 at axis-0 +-1, axis-1 +-1 and
    axis-2 -1 only (the reference writes the axis-2 -1 entry twice)."""
    lap = np.zeros(shape, dtype=np.float64)
    zc, yc, xc = shape[0] // 2, shape[1] // 2, shape[2] // 2
    lap[zc, yc, xc] = 6
    lap[zc - 1, yc, xc] = -1
    lap[zc + 1, yc, xc] = -1
    lap[zc, yc - 1, xc] = -1
    lap[zc, yc + 1, xc] = -1
    lap[zc, yc, xc - 1] = -1
    return lap


def center_psf(psf, tile_height, tile_size):
    """deconvolver.py:238-270: crop/zero-pad the PSF into (Z, ts, ts) about its
    centre (integer floor halves), then normalise to unit sum in the PSF dtype."""
    psf = np.asarray(psf)
    tgt = np.array([tile_height, tile_size, tile_size])
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


def padded_psf(psf, tile_height, tile_size, zpad, overlap):
    """deconvolver.py:52-62 for one PSF: centre, pad (zpad, ov, ov), roll by
    ``-np.array(shape)//2`` (floor of the negated shape)."""
    p = center_psf(psf, tile_height, tile_size)
    p = np.pad(p, ((zpad, zpad), (overlap, overlap), (overlap, overlap)), mode="constant")
    shift = -np.array(p.shape) // 2
    return np.roll(p, shift=tuple(int(s) for s in shift), axis=(0, 1, 2))


def wiener_half(psf, tile_height, tile_size, zpad, overlap, beta):
    """deconvolver.py:64-74 for one PSF, as the Hermitian half spectrum along the
    last axis: ``W = conj(H) / (H conj(H) + beta |L|^2)`` in complex128."""
    p = padded_psf(psf, tile_height, tile_size, zpad, overlap).astype(np.float64)
    H = sfft.rfftn(p, workers=WORKERS)
    L = sfft.rfftn(laplacian_3d(p.shape), workers=WORKERS)
    D = (H * np.conj(H)).real + beta * (L * np.conj(L)).real
    return np.conj(H) / D


def psf_list(psfs):
    """deconvolver.py:52-59: a dict gives one PSF per tile in dict order; an
    array is a single PSF reused for every tile."""
    if isinstance(psfs, dict):
        return [np.asarray(v) for v in psfs.values()]
    return [np.asarray(psfs)]


# --------------------------------------------------------------------------
# Tiling and padding (deconvolver.py:98-170, 186-206; fill.py:6-52)
# --------------------------------------------------------------------------
def tiles(shape, tile_size, overlap):
    """deconvolver.py:186-206: tile origins x-major, slices clipped with overlap."""
    _, sx, sy = shape
    out = []
    for x in range(0, sx, tile_size):
        for y in range(0, sy, tile_size):
            out.append((x, y,
                        max(x - overlap, 0), min(x + tile_size + overlap, sx),
                        max(y - overlap, 0), min(y + tile_size + overlap, sy)))
    return out


def mirror_inplace(a, i, axis, mode):
    """fill.py:6-52 (kernel ``mirror``): 'in' sets a[j] = a[2i-j] for j < i when
    2i-j < n; 'out' sets a[j] = a[2i-j] for j > i when 2i-j >= 0."""
    n = a.shape[axis]
    if mode == "in":
        js = np.arange(0, i)
    else:
        js = np.arange(i + 1, n)
    src = 2 * i - js
    ok = (src >= 0) & (src < n)
    js, src = js[ok], src[ok]
    if len(js) == 0:
        return a
    idx_dst = [slice(None)] * a.ndim
    idx_src = [slice(None)] * a.ndim
    idx_dst[axis] = js
    idx_src[axis] = src
    a[tuple(idx_dst)] = a[tuple(idx_src)]
    return a


def pad_tile(tile, flat, x, y, tile_size, zpad, overlap):
    """deconvolver.py:117-148: place the (float32) tile, divide by the flat in
    float32, then reflect x, y, z.  Returns the padded float32 tile and the
    yielded extents (xend, yend) and placement offsets (xstart, ystart)."""
    zdim, xdim, ydim = tile.shape
    P = tile_size + 2 * overlap
    xstart = overlap if x == 0 else 0
    ystart = overlap if y == 0 else 0
    xend, yend = xdim, ydim
    pad = np.zeros((zdim + 2 * zpad, P, P), dtype=np.float32)
    pad[zpad:zpad + zdim, xstart:xstart + xdim, ystart:ystart + ydim] = tile
    if flat is not None:
        m = (slice(zpad, zpad + zdim), slice(xstart, xstart + xdim), slice(ystart, ystart + ydim))
        pad[m] = pad[m] / np.asarray(flat, dtype=np.float32)
    if x == 0:
        mirror_inplace(pad, overlap, 1, "in")
        xend += overlap
    elif xdim < P:
        mirror_inplace(pad, xdim - 1, 1, "out")
        xend += overlap
    if y == 0:
        mirror_inplace(pad, overlap, 2, "in")
        yend += overlap
    elif ydim < P:
        mirror_inplace(pad, ydim - 1, 2, "out")
        yend += overlap
    mirror_inplace(pad, zpad, 0, "in")
    mirror_inplace(pad, zpad + zdim - 1, 0, "out")
    return pad, xstart, ystart, xend, yend


def box_mean_f64(a, delta, axis):
    """blur.cu:1-52 semantics in float64: mean over [c-delta, c+delta] clipped to
    the axis, divided by the number of in-range samples."""
    a = np.asarray(a, dtype=np.float64)
    n = a.shape[axis]
    c = np.cumsum(a, axis=axis)
    zshape = list(a.shape)
    zshape[axis] = 1
    c = np.concatenate([np.zeros(zshape), c], axis=axis)
    idx = np.arange(n)
    lo = np.maximum(idx - delta, 0)
    hi = np.minimum(idx + delta + 1, n)
    s = np.take(c, hi, axis=axis) - np.take(c, lo, axis=axis)
    cnt = (hi - lo).astype(np.float64)
    shp = [1] * a.ndim
    shp[axis] = n
    return s / cnt.reshape(shp)


def deconv_tile(image, flat, tile_box, W, tile_size, zpad, overlap, blur_radius=None):
    """One iteration of ``Deconvolver.tile_wise`` (deconvolver.py:116-170).

    Returns ``(res, raw)``: ``res`` is the float64 result over the yielded
    extent (Z, xend, yend) (float32 in the reference: ``tile_res[:, :xend, :yend]``),
    ``raw`` the float32 ``tile_pad[zpad:-zpad, :xend, :yend]`` after the flat
    is multiplied back (deconvolver.py:165-170)."""
    x, y, x0, x1, y0, y1 = tile_box
    tile = np.asarray(image[:, x0:x1, y0:y1], dtype=np.float32)
    ftile = None if flat is None else np.asarray(flat[x0:x1, y0:y1], dtype=np.float32)
    pad, xstart, ystart, xend, yend = pad_tile(tile, ftile, x, y, tile_size, zpad, overlap)
    zdim, xdim, ydim = tile.shape
    F = sfft.rfftn(pad.astype(np.float64), workers=WORKERS)
    F *= W
    res = sfft.irfftn(F, s=pad.shape, workers=WORKERS)[zpad:zpad + zdim]
    if blur_radius is not None:
        d = blur_radius // 2
        res = res - box_mean_f64(box_mean_f64(res, d, 1), d, 2)
    if ftile is not None:
        m = (slice(zpad, zpad + zdim), slice(xstart, xstart + xdim), slice(ystart, ystart + ydim))
        pad[m] = pad[m] * ftile
    raw = pad[zpad:zpad + zdim]
    return res[:, :xend, :yend], raw[:, :xend, :yend]


class Deconvolver:
    """Oracle counterpart of ``Deconvolver`` (deconvolver.py:47-236) with the
    Wiener spectra held as float64 Hermitian halves."""

    def __init__(self, psfs, channel_shape, tile_size=300, zpad=0, overlap=89, beta=0.001, **kwargs):
        self.tile_size = tile_size
        self.tile_height = channel_shape[0]
        self.zpad = zpad
        self.overlap = overlap
        self.W = [wiener_half(p, self.tile_height, tile_size, zpad, overlap, beta)
                  for p in psf_list(psfs)]

    def tile_wise(self, image, flat_field=None, blur_radius=None, **kwargs):
        """deconvolver.py:98-170; the PSF list is cycled when it has one entry and
        zipped (truncating) otherwise (deconvolver.py:110, 116)."""
        boxes = tiles(image.shape, self.tile_size, self.overlap)
        if len(self.W) != 1:
            boxes = boxes[:len(self.W)]
        for i, b in enumerate(boxes):
            W = self.W[0] if len(self.W) == 1 else self.W[i]
            res, raw = deconv_tile(image, flat_field, b, W, self.tile_size, self.zpad,
                                   self.overlap, blur_radius)
            yield b[0], b[1], res, raw

    def apply(self, image, flat_field=None, blur_radius=None, output=None, **kwargs):
        """deconvolver.py:172-184: stitch the tile centres into the output.
        Voxels no tile writes (the last ``overlap`` columns of a single-tile
        axis) are left as NaN here (uninitialised memory in the reference)."""
        if output is None:
            output = np.full(image.shape, np.nan, dtype=np.float64)
        ov = self.overlap
        for x, y, tile, _ in self.tile_wise(image, flat_field, blur_radius):
            _, xdim, ydim = tile.shape
            xdim -= 2 * ov
            ydim -= 2 * ov
            output[:, x:x + xdim, y:y + ydim] = tile[:, ov:-ov, ov:-ov]
        return output


def full_deconv(image, psfs, flat_field=None, tile_size=300, zpad=None, overlap=1, beta=0.001):
    """deconvolver.py:272-287."""
    if zpad is None:
        zpad = image.shape[0]
    d = Deconvolver(psfs, image.shape, tile_size=tile_size, zpad=zpad, overlap=overlap, beta=beta)
    return d.apply(image, flat_field)
