"""I/O around the per-FOV path (mermake/io.py): flat fields, the FOV reader and
the output writers.

* ``load_flats`` (io.py:42-54): centre crop, 21 x 21 box mean
  (``blur.box(size=(20, 20))``) and division by the median, on the GPU.
* ``read_im`` (io.py:116-146): a zarr v2 directory store (bz2 / zlib / raw
  chunks) read with the standard library, frame 0 dropped, frames split into
  channels from the ``<z_offsets>`` tag of the FOV's xml, uint8 widened to
  ``uint16 ** 2`` -- the reference reads the same layout through dask/zarr.
* ``save_xfits`` / ``save_dapi`` (io.py:561-575): ``np.savez_compressed`` with
  ``version``, ``args`` and the ``Xh`` / ``Xh_plus`` / ``Xh_minus`` tables;
  ``drift_save`` is in ``align``.
"""
from __future__ import annotations

import bz2
import ctypes as C
import glob
import json
import os
import zlib

import numpy as np
import torch

from . import __version__, _lib
from . import blur as _blur
from ._arrays import as_device


def center_crop(A, shape):
    """io.py:34-40: crop the last two axes of A to shape[-2:] about the centre."""
    h, w = shape[-2:]
    H, W = A.shape[-2:]
    top = (H - h) // 2
    left = (W - w) // 2
    return A[top:top + h, left:left + w]


def median(x):
    """cp.median of a float32 CUDA array (radix selection on the GPU)."""
    t = as_device(x, torch.float32).contiguous()
    m = C.c_float()
    _lib.check(_lib.lib().mm_median_f32(_lib.ctx(), _lib.ptr(t), t.numel(), C.byref(m), None, _lib.stream_ptr()))
    return m.value


def normalise_by_median(x):
    """x / median(x) in float32 (io.py:52)."""
    t = as_device(x, torch.float32).contiguous()
    out = torch.empty_like(t)
    m = C.c_float()
    _lib.check(_lib.lib().mm_median_f32(_lib.ctx(), _lib.ptr(t), t.numel(), C.byref(m), _lib.ptr(out),
                                        _lib.stream_ptr()))
    return out


def flat_from_image(im, shape=None):
    """One flat field (io.py:46-53) from a 2-D image: crop, blur, / median."""
    im = np.asarray(im)
    if shape is not None:
        assert im.shape[-1] >= shape[-1] and im.shape[-2] >= shape[-2], "flat field smaller than image"
        im = center_crop(im, shape)
    cim = torch.from_numpy(np.ascontiguousarray(im, dtype=np.float32)).cuda()
    blurred = _blur.box(cim, (20, 20), axes=(-1, -2))
    return normalise_by_median(blurred)


def load_flats(flat_field_tag, shape=None, **kwargs):
    """io.py:42-54: every ``flat_field_tag*`` .npz (key 'im'), in sorted order,
    stacked as a (ncol, X, Y) float32 CUDA tensor."""
    files = sorted(glob.glob(flat_field_tag + "*"))
    return torch.stack([flat_from_image(np.load(f)["im"], shape) for f in files])


# ---------------------------------------------------------------------------
# zarr v2 reader
# ---------------------------------------------------------------------------
def _decompress(buf, comp):
    if comp is None:
        return buf
    cid = comp.get("id")
    if cid == "bz2":
        return bz2.decompress(buf)
    if cid in ("zlib", "gzip"):
        return zlib.decompress(buf, 15 + (16 if cid == "gzip" else 0))
    raise NotImplementedError("zarr compressor %r" % cid)


def read_zarr(folder):
    """Whole zarr v2 array in a directory store (C order, '.'-separated chunk
    keys, missing chunks are fill_value)."""
    meta = json.load(open(os.path.join(folder, ".zarray")))
    if meta.get("order", "C") != "C" or meta.get("filters"):
        raise NotImplementedError("only C-order zarr arrays without filters")
    dtype = np.dtype(meta["dtype"])
    shape, chunks = meta["shape"], meta["chunks"]
    sep = meta.get("dimension_separator", ".")
    out = np.full(shape, meta.get("fill_value") or 0, dtype=dtype)
    grid = [-(-s // c) for s, c in zip(shape, chunks)]
    for idx in np.ndindex(*grid):
        f = os.path.join(folder, sep.join(str(i) for i in idx))
        if not os.path.exists(f):
            continue
        data = np.frombuffer(_decompress(open(f, "rb").read(), meta.get("compressor")), dtype=dtype)
        block = data.reshape(chunks)
        sl = tuple(slice(i * c, min((i + 1) * c, s)) for i, c, s in zip(idx, chunks, shape))
        out[sl] = block[tuple(slice(0, s.stop - s.start) for s in sl)]
    return out


def read_im(path, return_pos=False):
    """io.py:116-146: (ncol, Z, X, Y) uint16 channels of one FOV."""
    dirname = os.path.dirname(path)
    fov = os.path.basename(path).split("_")[-1].split(".")[0]
    image = read_zarr(os.path.join(dirname, fov, "data"))[1:]
    shape = image.shape
    x = y = None
    xml_file = os.path.splitext(path)[0] + ".xml"
    if os.path.exists(xml_file):
        txt = open(xml_file, "r").read()
        zstack = txt.split('<z_offsets type="string">')[-1].split("</")[0]
        pos = txt.split('<stage_position type="custom">')[-1].split("</")[0]
        try:
            x, y = [float(v) for v in pos.replace("[", "").replace("]", "").split(",")[:2]]
        except ValueError:
            x = y = None
        nch = int(zstack.split(":")[-1])
        nzs = (shape[0] // nch) * nch
        image = image[:nzs].reshape([shape[0] // nch, nch, shape[-2], shape[-1]]).swapaxes(0, 1)
    if image.dtype == np.uint8:
        image = image.astype(np.uint16) ** 2
    if return_pos:
        return image, x, y
    return image


# ---------------------------------------------------------------------------
# writers
# ---------------------------------------------------------------------------
def _host(a):
    return a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)


def save_xfits(filepath, args_array, Xh):
    """io.py:561-575 for a colour: never overwrites an existing file."""
    if not os.path.exists(filepath):
        np.savez_compressed(filepath, version=__version__, args=args_array, Xh=_host(Xh))


def save_dapi(filepath, args_array, Xh_plus, Xh_minus):
    """io.py:561-575 for the DAPI channel."""
    if not os.path.exists(filepath):
        np.savez_compressed(filepath, version=__version__, args=args_array, Xh_plus=_host(Xh_plus),
                            Xh_minus=_host(Xh_minus))
