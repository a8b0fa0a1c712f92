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
              blur_radius=None, batch=0, capacity=None, stream=None, ctx=None, tuned=True, **kwargs):
    """Rows ``[zc, xc, yc, bg, a, habs, hn, h]`` of one colour, in FOV coordinates
    (mermake/__main__.py:253-265).  ``dec`` is a ``Deconvolver``.  ``batch``:
    tiles per batch; 0 picks it (``tune.batch_for``), negative means all.
    ``capacity``: rows allocated for the output; None sizes it from the
    largest count this Deconvolver has returned for the shape (a call that
    overflows is run again with the exact count).  ``ctx``: a library context
    to run on (default: the calling thread's).  ``tuned``: run the z form
    ``tune.autotune`` chose for the geometry, if any."""
    _check_delta(delta)
    img = _u16_channel(image)
    if batch == 0:
        batch = tune.batch_for(dec, img.shape)
    form = tune.zform_for(dec, img.shape) if tuned else _lib.MM_ZFORM_AUTO
    if form != _lib.MM_ZFORM_AUTO and ctx is None:
        with _lib.zform(form, img.device.index):
            return hyb_spots(dec, img, flat_field, threshold=threshold, delta=delta, delta_fit=delta_fit,
                             sigmaZ=sigmaZ, sigmaXY=sigmaXY, blur_radius=blur_radius, batch=batch,
                             capacity=capacity, stream=stream, tuned=False)
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
        rc = L.mm_hyb_spots(ctx or _lib.ctx(img.device.index), _lib.ptr(img), Z, X, Y, img.stride(0), img.stride(1),
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
               blur_radius=None, batch=0, buffer=None, capacity=None, stream=None, ctx=None, tuned=True, **kwargs):
    """``(Xh_plus, Xh_minus, buffer, rms)`` of the DAPI block
    (mermake/__main__.py:215-225); ``buffer`` holds the stitched deconvolution
    before normalisation.  ``batch``, ``ctx`` and ``tuned`` as in ``hyb_spots``."""
    _check_delta(delta)
    img = _u16_channel(image)
    if batch == 0:
        batch = tune.batch_for(dec, img.shape, dapi=True)
    form = tune.zform_for(dec, img.shape, dapi=True) if tuned else _lib.MM_ZFORM_AUTO
    if form != _lib.MM_ZFORM_AUTO and ctx is None:
        with _lib.zform(form, img.device.index):
            return dapi_spots(dec, img, flat_field, threshold=threshold, delta=delta, delta_fit=delta_fit,
                              sigmaZ=sigmaZ, sigmaXY=sigmaXY, blur_radius=blur_radius, batch=batch,
                              buffer=buffer, capacity=capacity, stream=stream, tuned=False)
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
        rc = L.mm_dapi_spots(ctx or _lib.ctx(img.device.index), _lib.ptr(img), Z, X, Y, img.stride(0), img.stride(1),
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

    ``run`` is ``collect(launch(ticket, flats))``: ``launch`` enqueues the FOV
    without waiting for anything, ``collect`` makes its one synchronisation
    and reads the rows back.  Launching FOV k before collecting FOV k - 1
    keeps the GPU busy while the host reads results; a slot is free for the
    next ``submit`` once its FOV has been collected.
    """

    def __init__(self, dec_hyb, dec_dapi=None, hyb_args=None, dapi_args=None, batch=0):
        self.dec_hyb, self.dec_dapi = dec_hyb, dec_dapi
        self.hyb_args = dict(hyb_args or {})
        self.dapi_args = dict(dapi_args or {})
        self.batch = batch
        self.copy_stream = torch.cuda.Stream()
        self.read_stream = torch.cuda.Stream()  # collect's reads, behind only the FOV read
        self._slots = [dict(), dict()]
        self._next = 0
        self._buffer = None
        self._out = {}
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
        """The FOV of ``ticket``: the DAPI block and every colour enqueued on the
        current stream by the asynchronous drivers (their counts on the
        device), then one read of all counts and the rows.  An output that did
        not fit its rows (or candidate list) is run again by the synchronous
        driver, which resizes; later FOVs get rows sized from its count."""
        return self.collect(self.launch(ticket, flats, dapi_flat))

    def launch(self, ticket, flats=None, dapi_flat=None):
        """Enqueues the FOV of ``ticket`` on the current stream (no host
        synchronisation) and returns the handle ``collect`` takes."""
        cur = torch.cuda.current_stream()
        slot = ticket["slot"]
        evs, devs = list(ticket["events"]), list(ticket["dev"])
        n = len(devs) - (1 if ticket["has_dapi"] else 0)
        flats = list(flats) if flats is not None else [None] * n
        Z, X, Y = shape = tuple(int(v) for v in devs[0].shape)
        dev = devs[0].device
        L = _lib.lib()
        ctx = _lib.ctx(dev.index)
        sp = _lib.stream_ptr(cur)
        counts = torch.zeros(3 + 2 * n, dtype=torch.int32, device=dev)
        cbase = counts.data_ptr()
        dapi_img = dflat = None
        if ticket["has_dapi"]:
            d, a = self.dec_dapi, _settings(self.dapi_args)
            cur.wait_event(evs.pop(0))
            dapi_img = devs.pop(0)
            dflat = _flat(dapi_flat, shape)
            if self._buffer is None or tuple(self._buffer.shape) != shape:
                self._buffer = torch.empty(shape, dtype=torch.float32, device=dev)
            cap_p = _capacity(d, ("dapi+", Z, X, Y), 1 << 16)
            cap_m = _capacity(d, ("dapi-", Z, X, Y), 1 << 16)
            plus = self._rows(("plus", slot), cap_p, dev)
            minus = self._rows(("minus", slot), cap_m, dev)
            rms = self._rows(("rms", slot), 1, dev)
            bd = tune.batch_for(d, shape, dapi=True) if self.batch == 0 else self.batch
            _lib.check(L.mm_dapi_spots_async(
                ctx, _lib.ptr(dapi_img), Z, X, Y, dapi_img.stride(0), dapi_img.stride(1), _lib.ptr(dflat),
                dflat.stride(0) if dflat is not None else 0, _lib.ptr(d.psf_fft), d.psf_fft.shape[0],
                _lib.ptr(d.z_operator), d.tile_size, d.zpad, d.overlap, a["br"], a["th"], a["delta"], a["dfit"],
                a["sz"], a["sxy"], max(int(bd), 0), _lib.ptr(self._buffer), _lib.ptr(plus), cap_p, _lib.ptr(minus),
                cap_m, _lib._vp(cbase), _lib.ptr(rms), sp))
        d, a = self.dec_hyb, _settings(self.hyb_args)
        cap = _capacity(d, ("hyb", Z, X, Y), 1 << 18)
        bh = tune.batch_for(d, shape) if self.batch == 0 else self.batch
        rows, fls = [], []
        for c, (ev, img, f) in enumerate(zip(evs, devs, flats)):
            cur.wait_event(ev)
            fl = _flat(f, shape)
            fls.append(fl)
            r = self._rows(("hyb", c, slot), cap, dev)
            rows.append(r)
            _lib.check(L.mm_hyb_spots_async(
                ctx, _lib.ptr(img), Z, X, Y, img.stride(0), img.stride(1), _lib.ptr(fl),
                fl.stride(0) if fl is not None else 0, _lib.ptr(d.psf_fft), d.psf_fft.shape[0],
                _lib.ptr(d.z_operator), d.tile_size, d.zpad, d.overlap, a["br"], a["th"], a["delta"], a["dfit"],
                a["sz"], a["sxy"], max(int(bh), 0), _lib.ptr(r), cap, _lib._vp(cbase + 4 * (3 + 2 * c)),
                _lib._vp(cbase + 4 * (4 + 2 * c)), sp))
        # the slot's images are free for the next submit once these kernels
        # have run (collect moves the mark past any rerun that reads them)
        used = torch.cuda.Event()
        used.record(cur)
        self._slots[slot]["free"] = used
        return dict(ticket=ticket, counts=counts, shape=shape, n=n, devs=devs, fls=fls, rows=rows, used=used,
                    dapi=(dapi_img, dapi_flat, plus, minus, cap_p, cap_m) if ticket["has_dapi"] else None, cap=cap)

    def collect(self, h):
        """The rows of a launched FOV as host arrays, after its one
        synchronisation (and the reruns of outputs that did not fit)."""
        cur = torch.cuda.current_stream()
        ticket, n, devs, fls, rows, cap = h["ticket"], h["n"], h["devs"], h["fls"], h["rows"], h["cap"]
        Z, X, Y = h["shape"]
        d = self.dec_hyb
        out_plus = out_minus = None
        reran = False
        # the reads go on a stream of their own, behind this FOV's kernels only,
        # so a FOV launched after it keeps the GPU busy meanwhile
        rs = self.read_stream
        rs.wait_event(h["used"])
        with torch.cuda.stream(rs):
            cnt = h["counts"].cpu().tolist()  # the FOV's one synchronisation
        if ticket["has_dapi"]:
            dapi_img, dapi_flat, plus, minus, cap_p, cap_m = h["dapi"]
            dd = self.dec_dapi
            _seen(dd, ("dapi+", Z, X, Y), cnt[0])
            _seen(dd, ("dapi-", Z, X, Y), cnt[1])
            if cnt[2] or cnt[0] > cap_p or cnt[1] > cap_m:
                reran = True
                p, m, self._buffer, _ = dapi_spots(dd, dapi_img, dapi_flat, buffer=self._buffer, batch=self.batch,
                                                   **self.dapi_args)
                out_plus, out_minus = p.cpu().numpy(), m.cpu().numpy()
            else:
                with torch.cuda.stream(rs):
                    out_plus, out_minus = plus[:cnt[0]].cpu().numpy(), minus[:cnt[1]].cpu().numpy()
        out = []
        for c in range(n):
            nc = cnt[3 + 2 * c]
            _seen(d, ("hyb", Z, X, Y), nc)
            if cnt[4 + 2 * c] or nc > cap:
                reran = True
                out.append(hyb_spots(d, devs[c], fls[c], batch=self.batch, **self.hyb_args).cpu().numpy())
            else:
                with torch.cuda.stream(rs):
                    out.append(rows[c][:nc].cpu().numpy())
        if reran:
            done = torch.cuda.Event()
            done.record(cur)
            self._slots[ticket["slot"]]["free"] = done
        return out_plus, out_minus, out

    def _rows(self, key, cap, dev):
        """A persistent device buffer of at least ``cap`` rows of 8 floats."""
        buf = self._out.get(key)
        if buf is None or buf.shape[0] < cap or buf.device != dev:
            buf = torch.empty((cap, 8), dtype=torch.float32, device=dev)
            self._out[key] = buf
        return buf


def _settings(args):
    """The driver settings of a TOML section (defaults as hyb_spots')."""
    a = dict(args or {})
    th = a.get("threshold")
    br = a.get("blur_radius")
    delta = int(a.get("delta", 1))
    _check_delta(delta)
    return dict(th=float("nan") if th is None else float(th), br=-1 if br is None else int(br), delta=delta,
                dfit=int(a.get("delta_fit", 0)), sz=float(a.get("sigmaZ", 1)), sxy=float(a.get("sigmaXY", 1.5)))


class FovGraph:
    """One whole FOV -- the DAPI block and every colour -- captured once as a
    CUDA graph and replayed for each FOV of the same shape (no counterpart in
    the reference, whose loop launches every kernel from Python;
    mermake/__main__.py:211-283).

    The graph runs ``mm_dapi_spots_async`` and ``mm_hyb_spots_async`` on a
    library context of its own (nothing else grows its scratch, whose addresses
    the graph holds) into static buffers: inputs ``dapi`` (Z, X, Y) and
    ``colours`` (n, Z, X, Y) uint16 -- the caller's device tensors when given
    as ``inputs=(dapi, [colours])``, else buffers of the graph's own that
    ``run`` fills -- and per-output row buffers sized from the counts the
    Deconvolvers have seen (``hyb_spots``' rule).  One eager pass sizes the
    context's scratch before capture.  ``run`` replays and reads every count
    in one transfer; a FOV whose rows or candidates did not fit falls back to
    the synchronous drivers (``fallbacks`` counts them), after which the row
    buffers and candidate lists are grown to that FOV's counts and the graph is
    captured again (``recaptures``).  Flat fields are fixed at construction.
    """

    def __init__(self, dec_hyb, dec_dapi, shape, n_colours, hyb_args=None, dapi_args=None, flats=None,
                 dapi_flat=None, batch=0, inputs=None):
        self.shape = tuple(int(v) for v in shape)
        Z, X, Y = self.shape
        self.dec_hyb, self.dec_dapi = dec_hyb, dec_dapi
        self.hyb_args, self.dapi_args = dict(hyb_args or {}), dict(dapi_args or {})
        self._h, self._d = _settings(self.hyb_args), _settings(self.dapi_args)
        self.n = int(n_colours)
        self.fallbacks = 0
        self.dev = torch.cuda.current_device()
        dev = torch.device("cuda", self.dev)
        self._ctx = _lib._vp()
        _lib.check(_lib.lib().mm_ctx_create(C.byref(self._ctx)))
        if inputs is not None:
            self.dapi = _u16_channel(inputs[0]) if dec_dapi is not None else None
            self.colours = [_u16_channel(t) for t in inputs[1]]
        else:
            self.dapi = torch.zeros(self.shape, dtype=torch.uint16, device=dev) if dec_dapi is not None else None
            self.colours = [torch.zeros(self.shape, dtype=torch.uint16, device=dev) for _ in range(self.n)]
        if len(self.colours) != self.n or any(tuple(t.shape) != self.shape for t in self.colours):
            raise ValueError("colour inputs must be n_colours tensors of the FOV shape")
        self.flats = [_flat(f, self.shape) for f in (flats if flats is not None else [None] * self.n)]
        self.dapi_flat = _flat(dapi_flat, self.shape)
        self.batch_h = max(int(tune.batch_for(dec_hyb, self.shape) if batch == 0 else batch), 0)
        # counts: [rows (+), rows (-), DAPI candidate overflow] + [rows, overflow] per colour
        self.counts = torch.zeros(3 + 2 * self.n, dtype=torch.int32, device=dev)
        self.rms = torch.zeros(1, dtype=torch.float32, device=dev)
        if dec_dapi is not None:
            self.batch_d = max(int(tune.batch_for(dec_dapi, self.shape, dapi=True) if batch == 0 else batch), 0)
            self.buffer = torch.empty(self.shape, dtype=torch.float32, device=dev)
        self._stream = torch.cuda.Stream(device=dev)
        self.graph = None
        self.recaptures = 0
        self._capture()

    def _alloc_rows(self):
        """Row buffers from the largest counts the Deconvolvers have seen
        (hyb_spots' rule)."""
        Z, X, Y = self.shape
        dev = torch.device("cuda", self.dev)
        self.cap = _capacity(self.dec_hyb, ("hyb", Z, X, Y), 1 << 18)
        self.rows = [torch.empty((self.cap, 8), dtype=torch.float32, device=dev) for _ in range(self.n)]
        if self.dec_dapi is not None:
            self.cap_p = _capacity(self.dec_dapi, ("dapi+", Z, X, Y), 1 << 16)
            self.cap_m = _capacity(self.dec_dapi, ("dapi-", Z, X, Y), 1 << 16)
            self.plus = torch.empty((self.cap_p, 8), dtype=torch.float32, device=dev)
            self.minus = torch.empty((self.cap_m, 8), dtype=torch.float32, device=dev)

    def _capture(self, grow=False):
        """Row buffers, one eager pass (sizes the context's scratch and the
        transform plans), then the capture.  grow: first run the synchronous
        drivers on the graph's own context, which grow its candidate lists and
        record the counts the row buffers are sized from."""
        self.graph = None
        with torch.cuda.stream(self._stream):
            if grow:
                if self.dec_dapi is not None:
                    dapi_spots(self.dec_dapi, self.dapi, self.dapi_flat, buffer=self.buffer, batch=self.batch_d,
                               ctx=self._ctx, **self.dapi_args)
                for c in range(self.n):
                    hyb_spots(self.dec_hyb, self.colours[c], self.flats[c], batch=self.batch_h, ctx=self._ctx,
                              **self.hyb_args)
            self._alloc_rows()
            self._issue()
        self._stream.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        n0 = _lib.launch_count()
        with torch.cuda.graph(self.graph, stream=self._stream, capture_error_mode="thread_local"):
            self._issue()
        self._stream.synchronize()
        self.launches = _lib.launch_count() - n0  # library kernels one replay runs

    def _issue(self):
        L = _lib.lib()
        Z, X, Y = self.shape
        sp = _lib.stream_ptr(torch.cuda.current_stream())
        cbase = self.counts.data_ptr()
        if self.dec_dapi is not None:
            d, a, img, fl = self.dec_dapi, self._d, self.dapi, self.dapi_flat
            _lib.check(L.mm_dapi_spots_async(
                self._ctx, _lib.ptr(img), Z, X, Y, img.stride(0), img.stride(1), _lib.ptr(fl),
                fl.stride(0) if fl is not None else 0, _lib.ptr(d.psf_fft), d.psf_fft.shape[0],
                _lib.ptr(d.z_operator), d.tile_size, d.zpad, d.overlap, a["br"], a["th"], a["delta"], a["dfit"],
                a["sz"], a["sxy"], self.batch_d, _lib.ptr(self.buffer), _lib.ptr(self.plus), self.cap_p,
                _lib.ptr(self.minus), self.cap_m, _lib._vp(cbase), _lib.ptr(self.rms), sp))
        d, a = self.dec_hyb, self._h
        for c in range(self.n):
            img, fl = self.colours[c], self.flats[c]
            _lib.check(L.mm_hyb_spots_async(
                self._ctx, _lib.ptr(img), Z, X, Y, img.stride(0), img.stride(1), _lib.ptr(fl),
                fl.stride(0) if fl is not None else 0, _lib.ptr(d.psf_fft), d.psf_fft.shape[0],
                _lib.ptr(d.z_operator), d.tile_size, d.zpad, d.overlap, a["br"], a["th"], a["delta"], a["dfit"],
                a["sz"], a["sxy"], self.batch_h, _lib.ptr(self.rows[c]), self.cap, _lib._vp(cbase + 4 * (3 + 2 * c)),
                _lib._vp(cbase + 4 * (4 + 2 * c)), sp))

    def replay(self):
        """Replays the graph on the current stream (inputs already in place)."""
        self.graph.replay()

    def results(self):
        """Device views of the last replay: (Xh_plus, Xh_minus, [Xh per colour]),
        or None when an output or a candidate list overflowed."""
        cnt = self.counts.cpu().tolist()
        if self.dec_dapi is not None and (cnt[2] or cnt[0] > self.cap_p or cnt[1] > self.cap_m):
            return None
        if any(cnt[4 + 2 * c] or cnt[3 + 2 * c] > self.cap for c in range(self.n)):
            return None
        plus = self.plus[:cnt[0]] if self.dec_dapi is not None else None
        minus = self.minus[:cnt[1]] if self.dec_dapi is not None else None
        return plus, minus, [self.rows[c][:cnt[3 + 2 * c]] for c in range(self.n)]

    def run(self, dapi=None, colours=None):
        """(Xh_plus, Xh_minus, [Xh per colour]) host arrays of one FOV: copies
        the channels given (host or device) into the graph's inputs, replays,
        and falls back to the synchronous drivers when a result overflowed."""
        if dapi is not None and self.dapi is not None:
            self.dapi.copy_(torch.as_tensor(dapi), non_blocking=True)
        for c, h in enumerate(colours or []):
            self.colours[c].copy_(torch.as_tensor(h), non_blocking=True)
        self.replay()
        got = self.results()
        if got is None:
            # a result did not fit: this FOV through the synchronous drivers,
            # then the row buffers and candidate lists grown to its counts and
            # the graph captured again, so that later FOVs like it replay
            self.fallbacks += 1
            plus = minus = None
            if self.dec_dapi is not None:
                plus, minus, _, _ = dapi_spots(self.dec_dapi, self.dapi, self.dapi_flat, **self.dapi_args)
            got = (plus, minus, [hyb_spots(self.dec_hyb, self.colours[c], self.flats[c], **self.hyb_args)
                                 for c in range(self.n)])
            torch.cuda.current_stream().synchronize()
            self._capture(grow=True)
            self.recaptures += 1
        plus, minus, xh = got
        return (plus.cpu().numpy() if plus is not None else None, minus.cpu().numpy() if minus is not None else None,
                [r.cpu().numpy() for r in xh])

    def close(self):
        """Frees the graph and the context's scratch."""
        if self._ctx:
            torch.cuda.synchronize(self.dev)
            self.graph = None
            _lib.check(_lib.lib().mm_ctx_destroy(self._ctx))
            self._ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
