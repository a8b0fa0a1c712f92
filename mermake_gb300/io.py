"""I/O around the per-FOV path (mermake/io.py): flat fields, the FOV reader and
the output writers.

* ``load_flats`` (io.py:42-54): centre crop, 21 x 21 box mean
  (``blur.box(size=(20, 20))``) and division by the median, on the GPU.
* ``read_im`` (io.py:116-146): a zarr v2 directory store (bz2 / zlib / raw
  chunks) read with the standard library, frame 0 dropped, frames split into
  channels from the ``<z_offsets>`` tag of the FOV's xml, uint8 widened to
  ``uint16 ** 2`` -- the reference reads the same layout through dask/zarr.
* ``FovPrefetcher``: the prefetching reader in the role of ``ImageQueue``'s
  worker thread (io.py:321-463): FOVs decoded ahead of use, chunks
  decompressed in parallel, into pinned host memory ready for
  ``pipeline.FovRunner``.
* ``save_xfits`` / ``save_dapi`` (io.py:561-575): ``np.savez_compressed`` with
  ``version``, ``args`` and the ``Xh`` / ``Xh_plus`` / ``Xh_minus`` tables;
  ``drift_save`` is in ``align``.  ``namespace_to_array`` (io.py:619-637)
  makes the ``args`` table from the TOML settings, ``output_name``
  (io.py:535-546) the file names.
"""
from __future__ import annotations

import bz2
import concurrent.futures as cf
import ctypes as C
import glob
import json
import os
import queue
import re
import threading
import types
import zlib
from pathlib import Path

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


def _zarr_meta(folder):
    meta = json.load(open(os.path.join(folder, ".zarray")))
    if meta.get("order", "C") != "C" or meta.get("filters"):
        raise NotImplementedError("only C-order zarr arrays without filters")
    return meta


def _zarr_chunks(folder, meta):
    """(chunk file, destination slices, source slices) of every chunk."""
    shape, chunks = meta["shape"], meta["chunks"]
    sep = meta.get("dimension_separator", ".")
    grid = [-(-s // c) for s, c in zip(shape, chunks)]
    for idx in np.ndindex(*grid):
        sl = tuple(slice(i * c, min((i + 1) * c, s)) for i, c, s in zip(idx, chunks, shape))
        yield os.path.join(folder, sep.join(str(i) for i in idx)), sl, tuple(slice(0, s.stop - s.start) for s in sl)


def _read_chunk(f, meta, dtype):
    if not os.path.exists(f):
        return None
    data = np.frombuffer(_decompress(open(f, "rb").read(), meta.get("compressor")), dtype=dtype)
    return data.reshape(meta["chunks"])


def read_zarr(folder, pool=None):
    """Whole zarr v2 array in a directory store (C order, '.'-separated chunk
    keys, missing chunks are fill_value).  ``pool``: an executor that
    decompresses chunks in parallel (bz2 and zlib release the GIL)."""
    meta = _zarr_meta(folder)
    dtype = np.dtype(meta["dtype"])
    out = np.full(meta["shape"], meta.get("fill_value") or 0, dtype=dtype)

    def one(job):
        f, dst, src = job
        block = _read_chunk(f, meta, dtype)
        if block is not None:
            out[dst] = block[src]

    jobs = list(_zarr_chunks(folder, meta))
    if pool is None:
        for j in jobs:
            one(j)
    else:
        list(pool.map(one, jobs))
    return out


def _fov_layout(path):
    """The FOV's zarr folder, channel count and stage position from its xml
    (io.py:116-146)."""
    dirname = os.path.dirname(path)
    fov = os.path.basename(path).split("_")[-1].split(".")[0]
    folder = os.path.join(dirname, fov, "data")
    nch = x = y = None
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
    return folder, nch, x, y


def read_im(path, return_pos=False, pool=None):
    """io.py:116-146: (ncol, Z, X, Y) uint16 channels of one FOV."""
    folder, nch, x, y = _fov_layout(path)
    image = read_zarr(folder, pool)[1:]
    shape = image.shape
    if nch is not None:
        nzs = (shape[0] // nch) * nch
        image = image[:nzs].reshape([shape[0] // nch, nch, shape[-2], shape[-1]]).swapaxes(0, 1)
    if image.dtype == np.uint8:
        image = image.astype(np.uint16) ** 2
    if return_pos:
        return image, x, y
    return image


class FovPrefetcher:
    """FOVs read ahead of use, in the role of the reference's ``ImageQueue``
    worker thread (io.py:405-463, which decodes one FOV at a time on one
    thread).  A background thread walks ``paths``; each FOV's chunks are
    decompressed by a pool of ``workers`` threads (bz2 / zlib release the GIL)
    straight into their place in a host buffer -- pinned when CUDA is up, so
    that ``pipeline.FovRunner.submit`` copies it asynchronously -- and squared
    to uint16 there (``uint16(u8) ** 2``).  At most ``prefetch`` decoded FOVs
    wait in the queue.  Iterating yields ``(path, image)`` with ``image`` the
    ``(ncol, Z, X, Y)`` uint16 tensor of ``read_im``; a FOV that fails to
    read is reported with ``image`` the exception (the reference prints a
    warning and skips it).  ``decode_seconds`` and ``decoded_bytes`` total the
    time and the uncompressed chunk bytes of the decode work."""

    def __init__(self, paths, prefetch=2, workers=None, pin=None):
        import torch
        self.paths = list(paths)
        self.pin = torch.cuda.is_available() if pin is None else bool(pin)
        self.pool = cf.ThreadPoolExecutor(max_workers=workers or os.cpu_count() or 1)
        self.queue = queue.Queue(maxsize=max(1, int(prefetch)))
        self.stop_event = threading.Event()
        self.decode_seconds = 0.0
        self.decoded_bytes = 0
        self.thread = threading.Thread(target=self._worker, daemon=True)
        self.thread.start()

    def _read(self, path):
        import time

        import torch
        t0 = time.perf_counter()
        folder, nch, _, _ = _fov_layout(path)
        meta = _zarr_meta(folder)
        dtype = np.dtype(meta["dtype"])
        n, X, Y = meta["shape"][0] - 1, meta["shape"][-2], meta["shape"][-1]
        if len(meta["shape"]) != 3:
            raise NotImplementedError("FOV arrays are (frames, X, Y)")
        split = nch is not None
        nch = nch or 1
        nz = n // nch
        wide = dtype == np.uint8
        tdt = torch.uint16 if wide or dtype == np.uint16 else torch.from_numpy(np.zeros(0, dtype)).dtype
        buf = torch.empty((nch, nz, X, Y), dtype=tdt, pin_memory=self.pin)
        view = buf.numpy() if tdt != torch.uint16 else buf.view(torch.int16).numpy().view(np.uint16)
        fill = meta.get("fill_value") or 0
        nbytes = [0]

        def one(job):
            f, dst, src = job
            block = _read_chunk(f, meta, dtype)
            lo = dst[0].start
            frames = range(max(lo, 1), min(dst[0].stop, 1 + nz * nch))
            for fr in frames:  # frame fr (after frame 0) is plane (fr-1)//nch of channel (fr-1)%nch
                c, z = (fr - 1) % nch, (fr - 1) // nch
                tgt = view[c, z, dst[1], dst[2]]
                if block is None:
                    tgt[...] = np.uint16(fill) ** 2 if wide else fill
                    continue
                v = block[fr - lo][src[1], src[2]]
                if wide:
                    np.multiply(v, v, out=tgt, dtype=np.uint16)
                else:
                    tgt[...] = v
            if block is not None:
                nbytes[0] += block.nbytes

        list(self.pool.map(one, list(_zarr_chunks(folder, meta))))
        self.decode_seconds += time.perf_counter() - t0
        self.decoded_bytes += nbytes[0]
        return buf if split else buf[0]

    def _worker(self):
        for path in self.paths:
            if self.stop_event.is_set():
                break
            try:
                item = (path, self._read(path))
            except Exception as e:  # reported to the consumer, as the reference's warning
                item = (path, e)
            while not self.stop_event.is_set():
                try:
                    self.queue.put(item, timeout=0.1)
                    break
                except queue.Full:
                    continue
        self.queue.put(None)

    def __iter__(self):
        return self

    def __next__(self):
        item = self.queue.get()
        if item is None:
            self.queue.put(None)
            raise StopIteration
        return item

    def close(self):
        self.stop_event.set()
        try:
            while True:
                self.queue.get_nowait()
        except queue.Empty:
            pass
        self.thread.join(timeout=5.0)
        self.pool.shutdown(wait=True)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


# ---------------------------------------------------------------------------
# settings and output names
# ---------------------------------------------------------------------------
def dict_to_namespace(d):
    """io.py:599-607: nested dicts (the parsed TOML) as SimpleNamespaces."""
    out = {}
    for key, value in d.items():
        if isinstance(value, dict):
            value = dict_to_namespace(value)
        elif isinstance(value, list):
            value = [dict_to_namespace(i) if isinstance(i, dict) else i for i in value]
        out[key] = value
    return types.SimpleNamespace(**out)


def namespace_to_array(obj, prefix=""):
    """io.py:619-637: the settings as (block, key, str(value)) rows, the
    ``args`` table of every output file."""
    rows = []
    if isinstance(obj, types.SimpleNamespace) or hasattr(obj, "__dict__") and not isinstance(obj, dict):
        obj = vars(obj)
    if isinstance(obj, dict):
        for k, v in obj.items():
            full_key = "%s.%s" % (prefix, k) if prefix else k
            if isinstance(v, dict) or isinstance(v, types.SimpleNamespace):
                rows.extend(namespace_to_array(v, prefix=full_key))
            else:
                rows.append((prefix, k, str(v)))
    else:
        rows.append((prefix, "", str(obj)))
    return rows


def get_ifov(file_path):
    """io.py:156-162: the digits before ``.zarr`` in the file name."""
    m = re.search(r"([0-9]+)[^0-9]*\.zarr", Path(file_path).name)
    if m:
        return int(m.group(1))
    raise ValueError("No digits found before .zarr in filename: %s" % Path(file_path).name)


def get_iset(file_path):
    """io.py:164-181: the digits after ``_set`` in the name or a parent's."""
    path = Path(file_path)
    m = re.search(r"_set([0-9]+)", path.name)
    if m:
        return int(m.group(1))
    if path.parent == path:
        raise ValueError("No digits found after the word _set in %s" % file_path)
    return get_iset(path.parent)


def output_name(path, icol=None, hyb_save="{fov}--{tag}--col{icol}__Xhfits.npz",
                dapi_save="{fov}--{tag}--dapiFeatures.npz", drift_save="drift_{ifov}--_set{iset}.pkl"):
    """ImageQueue.get_name (io.py:535-546): the drift file (icol None), the
    DAPI file (icol -1) or colour icol's file of a FOV path."""
    p = Path(path)
    fov, tag = p.stem, p.parent.name
    if icol is None:
        return drift_save.format(ifov=get_ifov(path), fov=fov, iset=get_iset(path))
    if icol == -1:
        return dapi_save.format(fov=fov, tag=tag)
    return hyb_save.format(fov=fov, tag=tag, icol=icol)


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
