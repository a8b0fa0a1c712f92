"""Batch-size tuning for the per-FOV drivers (``pipeline.hyb_spots`` /
``dapi_spots``, ``batch=0``).

A tile batch's working set is its spectrum (Z x P x (P/2+1) complex64) plus
the float32 result and blur copies (2 x Z x P x P).  One batch of all tiles
amortises the launches and, with one PSF, lets the z step run as a matrix
product over the batch.  Measured on GB300, that beats batches small enough
to stay in the L2 cache even where a tile is only 110 MB (Z 40, tiles of 300,
100 PSFs: 170.5 ms per FOV for one batch against 183.7 ms for one tile at a
time).  ``default_batch`` therefore takes all tiles, up to a scratch budget
(``SCRATCH_BYTES``); ``autotune`` times candidate sizes on a real channel once
per geometry and keeps the fastest on the Deconvolver, where the drivers find
it.

With several PSFs every batch size gives the same rows.  With one PSF, batches
of fewer than 10 tiles use the padded-depth transforms instead of the z
operator; the voxels then differ in the float32 rounding (about 1e-7
relative), which can move a spot that sits on the threshold.
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
    tuned = getattr(dec, "_tuned_batch", {}).get(_key(dec, shape, dapi))
    return default_batch(dec, shape) if tuned is None else tuned


def autotune(dec, image, flat_field=None, settings=None, dapi=False, candidates=None, reps=2):
    """Times ``hyb_spots`` (or ``dapi_spots`` with ``dapi=True``) on ``image``
    for each candidate batch size (-1: all tiles) and keeps the fastest for
    this geometry on ``dec``.  Returns ``{batch: ms}``; the chosen one is
    ``batch_for(dec, image.shape, dapi)``."""
    from . import pipeline
    settings = dict(settings or {})
    settings.pop("batch", None)
    shape = tuple(int(v) for v in image.shape)
    nt = dec.n_tiles(shape)
    if candidates is None:
        candidates = sorted({c for c in (1, 4, 10, default_batch(dec, shape)) if 0 < c < nt} | {-1})
    times = {}
    buf = None
    for b in candidates:
        def run():
            nonlocal buf
            if dapi:
                out = pipeline.dapi_spots(dec, image, flat_field, batch=b, buffer=buf, **settings)
                buf = out[2]
            else:
                pipeline.hyb_spots(dec, image, flat_field, batch=b, **settings)
        run()  # warm-up (scratch sized for this batch)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            run()
        torch.cuda.synchronize()
        times[b] = 1e3 * (time.perf_counter() - t0) / reps
    best = min(times, key=times.get)
    if not hasattr(dec, "_tuned_batch"):
        dec._tuned_batch = {}
    dec._tuned_batch[_key(dec, shape, dapi)] = best
    return times

