"""ctypes binding of ``libmermake_gb300.so`` (the C ABI in include/mermake_gb300.h).

The library is the only compute path: if it is missing, or no CUDA device is
present, every entry point raises instead of falling back to another
implementation.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import torch

from . import _build

MM_OK, MM_EINVAL, MM_ENOMEM, MM_EOVERFLOW, MM_ETIMEOUT, MM_EDEVICE = range(6)
MM_OPT_BLUR_MODE, MM_OPT_ZFORM = 1, 2
MM_BLUR_AUTO, MM_BLUR_EXACT, MM_BLUR_SPECTRAL = range(3)
MM_ZFORM_AUTO, MM_ZFORM_REGISTERS, MM_ZFORM_SHARED, MM_ZFORM_DIRECT, MM_ZFORM_TRANSFORMS, MM_ZFORM_TENSOR = range(6)

_lock = threading.Lock()
_lib = None
_tls = threading.local()  # per-thread mm_ctx handles (ctx())


class MermakeError(RuntimeError):
    """A CUDA-side failure reported by the library (MM_EDEVICE / MM_ETIMEOUT)."""


class Overflow(Exception):
    def __init__(self, count):
        super().__init__(count)
        self.count = count


_vp = C.c_void_p
_i32 = C.c_int
_i64 = C.c_int64
_u32 = C.c_uint32
_f32 = C.c_float
_pi64 = C.POINTER(C.c_int64)
_pu32 = C.POINTER(C.c_uint32)
_pf32 = C.POINTER(C.c_float)

_SIGS = {
    "mm_abi_version": ([], _i32),
    "mm_last_error": ([], C.c_char_p),
    "mm_ctx_create": ([C.POINTER(_vp)], _i32),
    "mm_ctx_destroy": ([_vp], _i32),
    "mm_ctx_scratch_bytes": ([_vp, C.POINTER(C.c_uint64)], _i32),
    "mm_ctx_set_option": ([_vp, _i32, _i32], _i32),
    "mm_reflect_f32": ([_vp, _i32, _pi64, _pi64, _i32, _i32, _i32, _vp], _i32),
    "mm_box_1d_f32": ([_vp, _pi64, _vp, _pi64, _i32, _i32, _i32, _i32, _i32, _vp], _i32),
    "mm_subtract_u16": ([_vp, _pi64, _vp, _pi64, _vp, _pi64, _i32, _pi64, _i32, _vp], _i32),
    "mm_wiener_spectrum": ([_vp, _vp, _i32, _i32, _i32, _i32, _i32, _i32, _i32, _f32, _vp, _vp], _i32),
    "mm_wiener_zop": ([_vp, _vp, _i32, _i32, _i32, _i32, _vp, _vp], _i32),
    "mm_zkernel_supported": ([_i32, _i32], _i32),
    "mm_deconv_tiles": ([_vp, _vp, _i32, _i32, _i32, _i32, _i64, _i64, _vp, _i64, _vp, _i32, _vp] + [_i32] * 6
                        + [_vp, _vp, _vp, _i64, _i64, _vp], _i32),
    "mm_find_local_maxima": ([_vp, _vp, _i32, _i32, _i32, _i64, _i64, _vp, _i32, _i64, _i64, _f32, _i32, _i32,
                              _f32, _f32, _f32, _i32, _vp, _u32, _pu32, _vp], _i32),
    "mm_find_local_maxima_noalloc": ([_vp, _i32, _i32, _i32, _i64, _i64, _vp, _i32, _i64, _i64, _f32, _i32, _i32,
                                      _f32, _f32, _f32, _i32, _vp, _u32, _pu32, _vp], _i32),
    "mm_hyb_spots": ([_vp, _vp, _i32, _i32, _i32, _i64, _i64, _vp, _i64, _vp, _i32, _vp, _i32, _i32, _i32, _i32, _f32,
                      _i32, _i32, _f32, _f32, _i32, _vp, _u32, _pu32, _vp], _i32),
    "mm_dapi_spots": ([_vp, _vp, _i32, _i32, _i32, _i64, _i64, _vp, _i64, _vp, _i32, _vp, _i32, _i32, _i32, _i32,
                       _f32, _i32, _i32, _f32, _f32, _i32, _vp, _vp, _u32, _pu32, _vp, _u32, _pu32, _pf32, _vp], _i32),
    "mm_hyb_spots_async": ([_vp, _vp, _i32, _i32, _i32, _i64, _i64, _vp, _i64, _vp, _i32, _vp, _i32, _i32, _i32,
                            _i32, _f32, _i32, _i32, _f32, _f32, _i32, _vp, _u32, _vp, _vp, _vp], _i32),
    "mm_dapi_spots_async": ([_vp, _vp, _i32, _i32, _i32, _i64, _i64, _vp, _i64, _vp, _i32, _vp, _i32, _i32, _i32,
                             _i32, _f32, _i32, _i32, _f32, _f32, _i32, _vp, _vp, _u32, _vp, _u32, _vp, _vp, _vp],
                            _i32),
    "mm_tile_geometry": ([_i32] * 8 + [_vp] * 4, _i32),
    "mm_fft_c2c": ([_vp, _i32, _i32, _i32, _vp], _i32),
    "mm_median_f32": ([_vp, _vp, _i64, _pf32, _vp, _vp], _i32),
    "mm_aligner_create": ([_vp, _i32, _i32, _i64, _f32, _i32, _i32, C.POINTER(_vp), _vp], _i32),
    "mm_aligner_translation": ([_vp, _vp, _i32, _i32, _i64, _f32, _pf32, C.POINTER(_i32), _vp], _i32),
    "mm_aligner_info": ([_vp, C.POINTER(_i32), C.POINTER(_i32), C.POINTER(_i32)], _i32),
    "mm_aligner_destroy": ([_vp], _i32),
    "mm_profile_enable": ([_vp, _i32], _i32),
    "mm_profile_read": ([_vp, _i32, C.POINTER(C.c_double), C.POINTER(C.c_double), _pi64], _i32),
    "mm_stage_name": ([_i32], C.c_char_p),
    "mm_launch_count": ([], C.c_uint64),
}


def declared_symbols():
    """Names of the entry points bound here (checked against include/*.h by tests)."""
    return sorted(_SIGS)


def load(require_gpu=True):
    """Loads (building first if needed) the shared library."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.LIB
            if not os.path.exists(path):
                path = _build.build()
            lib = C.CDLL(path)
            for name, (args, res) in _SIGS.items():
                fn = getattr(lib, name)
                fn.argtypes = args
                fn.restype = res
            _lib = lib
    if require_gpu and not torch.cuda.is_available():
        raise MermakeError("mermake_gb300 needs a CUDA device; none is visible")
    return _lib


def lib():
    return load(True)


def ctx(device=None):
    """The calling thread's mm_ctx on a device (scratch owner).  The C ABI wants
    one context per host thread, so threads that call in concurrently (the
    serving workers) each get their own and run without waiting on a shared
    one."""
    L = lib()
    dev = torch.cuda.current_device() if device is None else int(device)
    per = getattr(_tls, "ctx", None)
    if per is None:
        per = _tls.ctx = {}
    c = per.get(dev)
    if c is None:
        with torch.cuda.device(dev):
            p = _vp()
            check(L.mm_ctx_create(C.byref(p)))
        c = per[dev] = p
    return c


def release_thread_ctx():
    """Frees the calling thread's contexts (their scratch); a later call makes new ones."""
    per = getattr(_tls, "ctx", None) or {}
    for dev, c in list(per.items()):
        with torch.cuda.device(dev):
            check(lib().mm_ctx_destroy(c))
    per.clear()


def scratch_bytes(device=None):
    """Device bytes of library scratch the calling thread's context holds."""
    v = C.c_uint64(0)
    check(lib().mm_ctx_scratch_bytes(ctx(device), C.byref(v)))
    return int(v.value)


def last_error():
    return (_lib.mm_last_error() or b"").decode(errors="replace") if _lib else ""


def check(rc, exc=ValueError):
    if rc == MM_OK:
        return
    msg = last_error()
    if rc == MM_EINVAL:
        raise exc(msg)
    if rc == MM_ENOMEM:
        raise MemoryError(msg)
    if rc == MM_ETIMEOUT:
        raise MermakeError("device wait timed out: " + msg)
    raise MermakeError(msg or "mermake_gb300 error %d" % rc)


def stream_ptr(stream=None):
    s = torch.cuda.current_stream() if stream is None else stream
    return _vp(s.cuda_stream)


def i64arr(vals):
    a = (C.c_int64 * len(vals))(*[int(v) for v in vals])
    return a


def ptr(t):
    return _vp(t.data_ptr()) if t is not None else _vp(0)


def profile_enable(on=True, device=None):
    check(lib().mm_profile_enable(ctx(device), int(bool(on))))


def profile_read(device=None):
    """{stage: (ms, algorithmic bytes, launches)} accumulated since profile_enable."""
    L = lib()
    n = 32
    ms = (C.c_double * n)()
    by = (C.c_double * n)()
    la = (C.c_int64 * n)()
    k = L.mm_profile_read(ctx(device), n, ms, by, la)
    if k < 0:
        check(k)
    return {L.mm_stage_name(i).decode(): (ms[i], by[i], int(la[i])) for i in range(k)}


def launch_count():
    return int(lib().mm_launch_count())


class blur_mode:
    """Context manager: the calling thread's library context runs with the
    given blur mode (MM_BLUR_AUTO / MM_BLUR_EXACT / MM_BLUR_SPECTRAL, see
    mm_ctx_set_option) inside the block and with MM_BLUR_AUTO after it."""

    def __init__(self, mode, device=None):
        self.mode, self.device = int(mode), device

    def __enter__(self):
        check(lib().mm_ctx_set_option(ctx(self.device), MM_OPT_BLUR_MODE, self.mode))
        return self

    def __exit__(self, *exc):
        check(lib().mm_ctx_set_option(ctx(self.device), MM_OPT_BLUR_MODE, MM_BLUR_AUTO))


class zform:
    """Context manager: the calling thread's library context runs the z step
    in the given form (MM_ZFORM_*, see mm_ctx_set_option) inside the block and
    with MM_ZFORM_AUTO after it."""

    def __init__(self, form, device=None):
        self.form, self.device = int(form), device

    def __enter__(self):
        check(lib().mm_ctx_set_option(ctx(self.device), MM_OPT_ZFORM, self.form))
        return self

    def __exit__(self, *exc):
        check(lib().mm_ctx_set_option(ctx(self.device), MM_OPT_ZFORM, MM_ZFORM_AUTO))
