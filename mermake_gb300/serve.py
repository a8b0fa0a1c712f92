"""Serving form of the per-FOV path: a request loop for FOV stacks of uneven
Z/XY that arrive over time (the streaming service of the reference's
acquisition loop, mermake/__main__.py:211-330, with the ImageQueue of
mermake/io.py:405-463 as the source).

* Admission: first in, first out, against the device memory actually held:
  torch's reserved memory (resident spectra, the workers' buffers, cached
  outputs) plus every worker's library scratch (``mm_ctx_scratch_bytes``),
  plus the growth reserved for the requests in flight.  A worker keeps its
  buffers (channel copies, the DAPI buffer) and its scratch between requests,
  growing them only, so a request is charged only what it adds to the worker
  that takes it.  When a request does not fit, idle workers give back what
  they hold; a request larger than the whole budget runs alone.
* Continuous batching: ``workers`` host threads each take the next admitted
  request as soon as they are free and run it on their own CUDA stream with
  their own library context, so the kernels of several FOVs overlap on the
  device while new ones keep arriving.
* Residency: the Wiener spectra (and z kernels) of every (Z, X, Y) shape are
  built once and kept; the DAPI maxima of round 0 of every FOV stay on the
  device as a DualAligner, and later rounds of that FOV are drift-aligned
  against them (mermake/align.py:131-176 with round 0 as the reference).

``submit`` returns a ``concurrent.futures.Future`` resolving to a
``FovResult`` (host arrays).  A request's result does not depend on what else
is in flight: every kernel reads only that request's buffers.
"""
from __future__ import annotations

import collections
import concurrent.futures as cf
import dataclasses
import threading
import time
import types

import numpy as np
import torch

from . import _lib, align, deconvolver, pipeline


@dataclasses.dataclass
class FovRequest:
    fov: int                  # FOV id: key of the drift reference
    round: int                # hyb round; round 0 holds the FOV's DAPI reference
    dapi: object              # (Z, X, Y) uint16 host array (pinned for overlap) or device tensor
    colours: list             # (Z, X, Y) uint16 arrays, one per colour
    flats: list = None        # per colour: (X, Y) float32 or None
    arrival: float = None     # time.perf_counter() of arrival (set by submit when None)


@dataclasses.dataclass
class FovResult:
    request: FovRequest
    xh_plus: np.ndarray
    xh_minus: np.ndarray
    xh: list                  # one (N, 8) array per colour
    drift: tuple              # (tzxyf, t+, t-, N+, N-) against round 0; None for round 0
    admitted: float
    done: float

    @property
    def latency(self):
        return self.done - self.request.arrival


def _shape_of(a):
    return tuple(int(v) for v in a.shape)


class FovServer:
    """Continuous-batching server for per-FOV requests (see the module doc)."""

    def __init__(self, psf, hyb_args, dapi_args, hbm_budget=120e9, workers=2, device=None, batch=0,
                 reference_timeout=60.0):
        self.psf = psf
        self.hyb_args = dict(hyb_args)
        self.dapi_args = dict(dapi_args)
        self.budget = float(hbm_budget)
        self.batch = int(batch)
        self.device = torch.cuda.current_device() if device is None else int(device)
        self.reference_timeout = reference_timeout
        self._cv = threading.Condition()
        self._pending = collections.deque()
        self._grow = 0.0          # growth reserved for admitted, unfinished requests
        self._resident = 0.0      # bytes of spectra not built yet for admitted shapes
        self._in_flight = 0
        self.max_in_flight = 0
        self._held = {}           # worker -> [buffer bytes, scratch bytes] it keeps
        self._busy = set()        # workers running a request
        self._release_wanted = False
        self.peak_bytes = 0.0     # largest measured total seen at admissions and completions
        self.releases = 0
        self._closed = False
        self._decs = {}           # shape -> (hyb, dapi) Deconvolvers
        self._reserved = set()    # shapes whose spectra are counted in _resident
        self._dec_lock = threading.Lock()
        self._refs = {}           # fov -> (DualAligner, lock)
        self._ref_cv = threading.Condition()
        self.results = []
        self._state = {}
        self._threads = [threading.Thread(target=self._worker, args=(i,), name="mm-serve-%d" % i, daemon=True)
                         for i in range(int(workers))]
        for t in self._threads:
            t.start()

    # -- client side ---------------------------------------------------------
    def submit(self, req):
        if req.arrival is None:
            req.arrival = time.perf_counter()
        fut = cf.Future()
        with self._cv:
            if self._closed:
                raise RuntimeError("server is closed")
            self._pending.append((req, fut))
            self._cv.notify_all()
        return fut

    def close(self):
        with self._cv:
            self._closed = True
            self._cv.notify_all()
        for t in self._threads:
            t.join()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- memory model --------------------------------------------------------
    def _est(self, req):
        """(buffer bytes, scratch bytes) a worker holds to run req: the channel
        copies and the DAPI buffer; the library scratch of the largest tile
        batch (spectrum, result and blur copy, with the 1/8 headroom the
        library allocates) and a candidate list."""
        Z, X, Y = _shape_of(req.dapi)
        nch = 1 + len(req.colours)
        buffers = nch * Z * X * Y * 2 + Z * X * Y * 4
        scratch = 0
        for args in (self.hyb_args, self.dapi_args):
            ts, ov = int(args.get("tile_size", 500)), int(args.get("overlap", 89))
            P = ts + 2 * ov
            ntiles = -(-X // ts) * -(-Y // ts)
            nb = ntiles if self.batch <= 0 else min(self.batch, ntiles)
            scratch = max(scratch, nb * Z * P * ((P // 2 + 1) * 8 + 2 * P * 4))
        return buffers, scratch * 9 // 8 + (64 << 20)

    def _spectra_bytes(self, shape):
        Z = shape[0]
        out = 0
        for args, zpad in ((self.hyb_args, Z - 1), (self.dapi_args, (Z - 1) // 2)):
            P = int(args.get("tile_size", 500)) + 2 * int(args.get("overlap", 89))
            out += 2 * (Z + 2 * zpad) * P * (P // 2 + 1) * 8
        return out

    def _measured(self):
        """Device bytes held now: torch's reserved memory and the workers'
        library scratch."""
        held = sum(h[1] for h in self._held.values())
        return float(torch.cuda.memory_reserved(self.device)) + held

    def _admit(self, worker):
        """Blocks until the head request fits; returns it (or None when closed
        and empty).  Idle workers asked to give memory back do so here."""
        with self._cv:
            while True:
                if self._release_wanted and worker not in self._busy and sum(self._held.get(worker, (0, 0))) > 0:
                    self._give_back(worker)
                if self._pending:
                    req, fut = self._pending[0]
                    need_b, need_s = self._est(req)
                    held_b, held_s = self._held.get(worker, (0, 0))
                    grow = max(0, need_b - held_b) + max(0, need_s - held_s)
                    shape = _shape_of(req.dapi)
                    extra = 0 if shape in self._reserved else self._spectra_bytes(shape)
                    total = self._measured() + self._grow + self._resident + grow + extra
                    idle = [w for w, h in self._held.items() if w not in self._busy and w != worker and sum(h) > 0]
                    # over the budget, a request runs only alone: nothing in
                    # flight and no idle worker holding memory
                    if total <= self.budget or (self._in_flight == 0 and not idle):
                        self._pending.popleft()
                        self._grow += grow
                        self._resident += extra
                        self._reserved.add(shape)
                        self._in_flight += 1
                        self._busy.add(worker)
                        self._release_wanted = False
                        self.max_in_flight = max(self.max_in_flight, self._in_flight)
                        self.peak_bytes = max(self.peak_bytes, self._measured())
                        return req, fut, (grow, extra)
                    # over budget: idle workers holding memory give it back
                    if idle:
                        self._release_wanted = True
                        self._cv.notify_all()
                elif self._closed:
                    return None
                self._cv.wait(0.05)

    def _give_back(self, worker):
        """Drops this (idle) worker's buffers and library context and returns
        torch's unused cache to the device."""
        self._state[worker].clear()
        torch.cuda.synchronize(self.device)
        _lib.release_thread_ctx()
        torch.cuda.empty_cache()
        self._held[worker] = [0, 0]
        self.releases += 1
        self._cv.notify_all()

    def _release(self, worker, reserved):
        grow, extra = reserved
        with self._cv:
            self._grow -= grow
            self._resident -= extra  # the spectra now sit in torch's reserved memory
            self._in_flight -= 1
            self._busy.discard(worker)
            st = self._state[worker]
            self._held[worker] = [sum(t.numel() * t.element_size() for t in st.values()
                                      if isinstance(t, torch.Tensor)),
                                  _lib.scratch_bytes(self.device)]
            self.peak_bytes = max(self.peak_bytes, self._measured())
            self._cv.notify_all()

    # -- work ----------------------------------------------------------------
    def _deconvolvers(self, shape):
        with self._dec_lock:
            d = self._decs.get(shape)
            if d is None:
                Z = shape[0]
                hyb = deconvolver.Deconvolver(self.psf, shape, zpad=Z - 1, **self.hyb_args)
                dap = deconvolver.Deconvolver(self.psf, shape, zpad=(Z - 1) // 2, **self.dapi_args)
                torch.cuda.current_stream().synchronize()  # built before another stream reads them
                d = self._decs[shape] = (hyb, dap)
            return d

    def _reference(self, fov, plus, minus):
        dual = align.DualAligner(types.SimpleNamespace(Xh_plus=plus, Xh_minus=minus), th=4)
        torch.cuda.current_stream().synchronize()  # resident before another stream reads it
        with self._ref_cv:
            self._refs[fov] = (dual, threading.Lock())
            self._ref_cv.notify_all()

    def _drift(self, fov, plus, minus):
        deadline = time.perf_counter() + self.reference_timeout
        with self._ref_cv:
            while fov not in self._refs:
                left = deadline - time.perf_counter()
                if left <= 0:
                    return None
                self._ref_cv.wait(left)
            dual, lock = self._refs[fov]
        with lock:
            return dual.get_best_translation_pointsV2(types.SimpleNamespace(Xh_plus=plus, Xh_minus=minus))

    @staticmethod
    def _grown(state, key, numel, dtype):
        """A flat device buffer of the worker's, grown to at least numel."""
        t = state.get(key)
        if t is None or t.numel() < numel or t.dtype != dtype:
            state.pop(key, None)
            t = state[key] = torch.empty(numel, dtype=dtype, device="cuda")
        return t[:numel]

    def _run(self, req, stream, state):
        dev = []
        for k, h in enumerate([req.dapi] + list(req.colours)):
            t = h if isinstance(h, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(h))
            d = self._grown(state, ("chan", k), t.numel(), t.dtype).view(t.shape)
            d.copy_(t, non_blocking=True)
            dev.append(d)
        hyb, dap = self._deconvolvers(_shape_of(req.dapi))
        buf = self._grown(state, "buffer", dev[0].numel(), torch.float32).view(dev[0].shape)
        plus, minus, _, _ = pipeline.dapi_spots(dap, dev[0], None, buffer=buf, batch=self.batch, **self.dapi_args)
        if req.round == 0:
            self._reference(req.fov, plus, minus)
            drift = None
        else:
            drift = self._drift(req.fov, plus, minus)
        flats = list(req.flats) if req.flats is not None else [None] * len(req.colours)
        xh = [pipeline.hyb_spots(hyb, d, f, batch=self.batch, **self.hyb_args).cpu().numpy()
              for d, f in zip(dev[1:], flats)]
        return plus.cpu().numpy(), minus.cpu().numpy(), xh, drift

    def _worker(self, wid):
        torch.cuda.set_device(self.device)
        stream = torch.cuda.Stream()
        state = self._state[wid] = {}
        with self._cv:
            self._held[wid] = [0, 0]
        try:
            while True:
                got = self._admit(wid)
                if got is None:
                    return
                req, fut, need = got
                admitted = time.perf_counter()
                try:
                    with torch.cuda.stream(stream):
                        p, m, xh, drift = self._run(req, stream, state)
                    res = FovResult(req, p, m, xh, drift, admitted, time.perf_counter())
                    with self._cv:
                        self.results.append(res)
                    fut.set_result(res)
                except BaseException as e:  # the request fails, the server keeps running
                    fut.set_exception(e)
                finally:
                    stream.synchronize()
                    self._release(wid, need)
        finally:
            state.clear()
            torch.cuda.synchronize()
            _lib.release_thread_ctx()
