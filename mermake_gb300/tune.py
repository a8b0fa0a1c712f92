"""Tuning of the per-FOV drivers (``pipeline.hyb_spots`` / ``dapi_spots``):
the tile batch size and the form of the z step, per geometry.

A tile batch's working set is its spectrum (Z x P x (P/2+1) complex64) plus
the float32 result and blur copy (2 x Z x P x P).  One batch of all tiles
amortises the launches and, with one PSF, lets the z step run as a matrix
product over the batch.  Measured on GB300, that beats batches small enough
to stay in the L2 cache even where a tile is only 110 MB (Z 40, tiles of 300,
100 PSFs: 170.5 ms per FOV for one batch against 183.7 ms for one tile at a
time).  ``default_batch`` therefore takes all tiles, up to a scratch budget
(``SCRATCH_BYTES``), and the library picks the z form (``MM_ZFORM_AUTO``).

``autotune`` times, on a real channel, every candidate batch size with every
z form the geometry qualifies for (the matrix in registers, over one shared
spectrum or per tile, the matrix on the tensor cores or in shared memory, the
direct sum per tile, the transforms over the padded depth;
``mm_ctx_set_option(MM_OPT_ZFORM)``) and keeps the fastest pair on the
Deconvolver, where the drivers find it (``settings_for``).

With several PSFs every batch size gives the same rows.  The z forms, and
with one PSF batches on either side of the matrix forms' 10 tiles, give the
same voxels within float32 rounding (about 1e-7 relative), which can move a
spot that sits on the threshold.
"""
from __future__ import annotations

import time

import torch

SCRATCH_BYTES = 32 << 30  # device bytes of tile scratch one batch may take


def tile_bytes(dec):
    """Device bytes one tile of a batch holds (spectrum, result, blur copy)."""
    Z, P, H = dec.tile_height, dec.P, dec.H
    return Z * P * H * 8 + 2 * Z * P * P * 4


def _key(dec, shape, dapi):
    return (tuple(int(v) for v in shape), bool(dapi))


def default_batch(dec, shape):
    """All tiles in one batch (-1), or as many as fit ``SCRATCH_BYTES``."""
    nt = dec.n_tiles(shape)
    b = max(1, SCRATCH_BYTES // tile_bytes(dec))
    return -1 if b >= nt else int(b)


def batch_for(dec, shape, dapi=False):
    """The tuned batch of this geometry, else ``default_batch``."""
    tuned = getattr(dec, "_tuned", {}).get(_key(dec, shape, dapi))
    return default_batch(dec, shape) if tuned is None else tuned[0]


def zform_for(dec, shape, dapi=False):
    """The tuned z form of this geometry (``_lib.MM_ZFORM_*``), else AUTO."""
    from . import _lib
    tuned = getattr(dec, "_tuned", {}).get(_key(dec, shape, dapi))
    return _lib.MM_ZFORM_AUTO if tuned is None else tuned[1]


def zforms(dec):
    """The z forms worth timing for a Deconvolver: those of its z kernels when
    it has them, and the transforms over the padded depth."""
    from . import _lib
    forms = [_lib.MM_ZFORM_TRANSFORMS]
    if dec.z_operator is not None:
        forms = [_lib.MM_ZFORM_REGISTERS, _lib.MM_ZFORM_DIRECT] + forms
        if dec.psf_fft.shape[0] == 1:
            forms = forms[:1] + [_lib.MM_ZFORM_TENSOR, _lib.MM_ZFORM_SHARED] + forms[1:]
    return forms


def autotune(dec, image, flat_field=None, settings=None, dapi=False, candidates=None, forms=None, reps=2):
    """Times ``hyb_spots`` (or ``dapi_spots`` with ``dapi=True``) on ``image``
    for every candidate batch size (-1: all tiles) with every z form, and keeps
    the fastest pair for this geometry on ``dec``.  Returns
    ``{(batch, form): ms}``; the choice is ``settings_for(dec, shape, dapi)``."""
    from . import _lib, pipeline
    settings = dict(settings or {})
    settings.pop("batch", None)
    shape = tuple(int(v) for v in image.shape)
    nt = dec.n_tiles(shape)
    if candidates is None:
        candidates = sorted({c for c in (1, 4, 10, default_batch(dec, shape)) if 0 < c < nt} | {-1})
    forms = zforms(dec) if forms is None else list(forms)
    times = {}
    buf = None
    for b in candidates:
        for f in forms:
            def run():
                nonlocal buf
                with _lib.zform(f):
                    if dapi:
                        out = pipeline.dapi_spots(dec, image, flat_field, batch=b, buffer=buf, tuned=False, **settings)
                        buf = out[2]
                    else:
                        pipeline.hyb_spots(dec, image, flat_field, batch=b, tuned=False, **settings)
            run()  # warm-up (scratch sized for this batch)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(reps):
                run()
            torch.cuda.synchronize()
            times[(b, f)] = 1e3 * (time.perf_counter() - t0) / reps
    best = min(times, key=times.get)
    dec.__dict__.setdefault("_tuned", {})[_key(dec, shape, dapi)] = best
    return times


def settings_for(dec, shape, dapi=False):
    """(batch, z form) the drivers use for this geometry."""
    return batch_for(dec, shape, dapi), zform_for(dec, shape, dapi)
