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

from . import _lib, tune
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


def _capacity(dec, key, default):
    """Output rows to allocate: the largest count seen for ``key`` on this
    Deconvolver plus a quarter, at least ``default``."""
    seen = getattr(dec, "_rows_seen", {}).get(key, 0)
    return max(default, seen + seen // 4)


def _seen(dec, key, n):
    d = dec.__dict__.setdefault("_rows_seen", {})
    if n > d.get(key, 0):
        d[key] = n


def hyb_spots(dec, image, flat_field=None, *, threshold=None, delta=1, delta_fit=0, sigmaZ=1, sigmaXY=1.5,
              blur_radius=None, batch=0, capacity=None, stream=None, **kwargs):
    """Rows ``[zc, xc, yc, bg, a, habs, hn, h]`` of one colour, in FOV coordinates
    (mermake/__main__.py:253-265).  ``dec`` is a ``Deconvolver``.  ``batch``:
    tiles per batch; 0 picks it (``tune.batch_for``), negative means all.
    ``capacity``: rows allocated for the output; None sizes it from the
    largest count this Deconvolver has returned for the shape (a call that
    overflows is run again with the exact count)."""
    _check_delta(delta)
    img = _u16_channel(image)
    if batch == 0:
        batch = tune.batch_for(dec, img.shape)
    fl = _flat(flat_field, img.shape)
    Z, X, Y = img.shape
    L = _lib.lib()
    th = float("nan") if threshold is None else float(threshold)
    br = -1 if blur_radius is None else int(blur_radius)
    key = ("hyb", Z, X, Y)
    cap = _capacity(dec, key, 1 << 18) if capacity is None else int(capacity)
    for _ in range(2):
        out = torch.empty((cap, 8), dtype=torch.float32, device=img.device)
        n = C.c_uint32(0)
        rc = L.mm_hyb_spots(_lib.ctx(img.device.index), _lib.ptr(img), Z, X, Y, img.stride(0), img.stride(1),
                            _lib.ptr(fl), fl.stride(0) if fl is not None else 0, _lib.ptr(dec.psf_fft),
                            dec.psf_fft.shape[0], _lib.ptr(dec.z_operator), dec.tile_size, dec.zpad, dec.overlap,
                            br, th, int(delta), int(delta_fit), float(sigmaZ), float(sigmaXY), max(int(batch), 0),
                            _lib.ptr(out), cap, C.byref(n), _lib.stream_ptr(stream))
        _seen(dec, key, int(n.value))
        if rc == _lib.MM_EOVERFLOW:
            cap = int(n.value)
            continue
        _lib.check(rc)
        return out[: n.value]
    raise _lib.MermakeError("spot rows did not fit after resizing")


def dapi_spots(dec, image, flat_field=None, *, threshold=None, delta=1, delta_fit=0, sigmaZ=1, sigmaXY=1.5,
               blur_radius=None, batch=0, buffer=None, capacity=None, stream=None, **kwargs):
    """``(Xh_plus, Xh_minus, buffer, rms)`` of the DAPI block
    (mermake/__main__.py:215-225); ``buffer`` holds the stitched deconvolution
    before normalisation.  ``batch`` as in ``hyb_spots``."""
    _check_delta(delta)
    img = _u16_channel(image)
    if batch == 0:
        batch = tune.batch_for(dec, img.shape, dapi=True)
    fl = _flat(flat_field, img.shape)
    Z, X, Y = img.shape
    if buffer is None:
        buffer = torch.empty((Z, X, Y), dtype=torch.float32, device=img.device)
    L = _lib.lib()
    th = float("nan") if threshold is None else float(threshold)
    br = -1 if blur_radius is None else int(blur_radius)
    kp, km = ("dapi+", Z, X, Y), ("dapi-", Z, X, Y)
    if capacity is None:
        cp, cm = _capacity(dec, kp, 1 << 16), _capacity(dec, km, 1 << 16)
    else:
        cp, cm = int(capacity), int(capacity)
    for _ in range(2):
        op = torch.empty((cp, 8), dtype=torch.float32, device=img.device)
        om = torch.empty((cm, 8), dtype=torch.float32, device=img.device)
        n_p, n_m, rms = C.c_uint32(0), C.c_uint32(0), C.c_float(0)
        rc = L.mm_dapi_spots(_lib.ctx(img.device.index), _lib.ptr(img), Z, X, Y, img.stride(0), img.stride(1),
                             _lib.ptr(fl), fl.stride(0) if fl is not None else 0, _lib.ptr(dec.psf_fft),
                             dec.psf_fft.shape[0], _lib.ptr(dec.z_operator), dec.tile_size, dec.zpad,
                             dec.overlap, br, th, int(delta), int(delta_fit), float(sigmaZ), float(sigmaXY),
                             max(int(batch), 0), _lib.ptr(buffer), _lib.ptr(op), cp, C.byref(n_p), _lib.ptr(om), cm, C.byref(n_m), C.byref(rms),
                             _lib.stream_ptr(stream))
        _seen(dec, kp, int(n_p.value))
        _seen(dec, km, int(n_m.value))
        if rc == _lib.MM_EOVERFLOW:
            cp, cm = max(cp, int(n_p.value)), max(cm, int(n_m.value))
            continue
        _lib.check(rc)
        return op[: n_p.value], om[: n_m.value], buffer, float(rms.value)
    raise _lib.MermakeError("spot rows did not fit after resizing")


class FovRunner:
    """Whole FOVs from pinned host memory, with the next FOV's channels copied
    to the device on a side stream while the current FOV computes: the role of
    the reference's prefetching ``ImageQueue`` (mermake/io.py:405-463) for the
    host-to-device step of ``__main__.py:211-283``.

    ``submit(dapi, colours)`` enqueues the copies of one FOV (uint16 host
    arrays, pinned for overlap) into the next of two device slots and returns
    a ticket; ``run(ticket, flats)`` waits for that FOV's copies channel by
    channel and returns ``(Xh_plus, Xh_minus, [Xh per colour])`` as host
    arrays.  Submit FOV k+1 before running FOV k to overlap them.
    """

    def __init__(self, dec_hyb, dec_dapi=None, hyb_args=None, dapi_args=None, batch=0):
        self.dec_hyb, self.dec_dapi = dec_hyb, dec_dapi
        self.hyb_args = dict(hyb_args or {})
        self.dapi_args = dict(dapi_args or {})
        self.batch = batch
        self.copy_stream = torch.cuda.Stream()
        self._slots = [dict(), dict()]
        self._next = 0
        self._buffer = None
        self.h2d_bytes = 0

    def _dev(self, slot, key, host):
        buf = self._slots[slot].get(key)
        if buf is None or buf.shape != host.shape or buf.dtype != host.dtype:
            buf = torch.empty(host.shape, dtype=host.dtype, device="cuda")
            self._slots[slot][key] = buf
        return buf

    def submit(self, dapi, colours):
        slot = self._next
        self._next ^= 1
        ticket = {"slot": slot, "events": [], "dev": [], "free": self._slots[slot].get("free")}
        cs = self.copy_stream
        if ticket["free"] is not None:
            cs.wait_event(ticket["free"])  # the slot's previous FOV is done with its buffers
        nbytes = 0
        with torch.cuda.stream(cs):
            for k, h in enumerate(([dapi] if dapi is not None else []) + list(colours)):
                d = self._dev(slot, k, h)
                d.copy_(h, non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(cs)
                ticket["events"].append(ev)
                ticket["dev"].append(d)
                nbytes += h.numel() * h.element_size()
        ticket["has_dapi"] = dapi is not None
        self.h2d_bytes = nbytes
        return ticket

    def run(self, ticket, flats=None, dapi_flat=None):
        cur = torch.cuda.current_stream()
        evs, devs = list(ticket["events"]), list(ticket["dev"])
        out_plus = out_minus = None
        if ticket["has_dapi"]:
            cur.wait_event(evs.pop(0))
            p, m, self._buffer, _ = dapi_spots(self.dec_dapi, devs.pop(0), dapi_flat, buffer=self._buffer,
                                               batch=self.batch, **self.dapi_args)
            out_plus, out_minus = p.cpu().numpy(), m.cpu().numpy()
        flats = list(flats) if flats is not None else [None] * len(devs)
        rows = []
        for ev, d, f in zip(evs, devs, flats):
            cur.wait_event(ev)
            rows.append(hyb_spots(self.dec_hyb, d, f, batch=self.batch, **self.hyb_args).cpu().numpy())
        done = torch.cuda.Event()
        done.record(cur)
        self._slots[ticket["slot"]]["free"] = done
        return out_plus, out_minus, rows
