"""ctypes wrappers for the oracle's C restatement (``kernels.c``) and, where it
was built, the reference kernels compiled as C++ (``_ref/libref.so``).

Test infrastructure only.  Function names and argument meaning follow the
reference's Python wrappers: ``find_local_maxima`` (mermake/maxima.py:17-98),
``box_1d`` (mermake/blur.py:157-188), ``reflect`` (mermake/fill.py:54-111).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_P = np.ctypeslib.ndpointer
_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        L.orc_box_1d.argtypes = [_P(np.float32, flags="C"), _P(np.float32, flags="C"),
                                 C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_box_mean_f64.argtypes = [_P(np.float64, flags="C"), _P(np.float64, flags="C"),
                                       C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_mirror.argtypes = [C.c_void_p, C.c_int, _P(np.int64), _P(np.int64), C.c_int, C.c_int, C.c_int]
        L.orc_local_maxima.restype = C.c_uint32
        L.orc_local_maxima.argtypes = [_P(np.float32, flags="C"), C.c_float, C.c_int, C.c_int, C.c_int,
                                       C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32]
        L.orc_delta_fit.argtypes = [_P(np.float32, flags="C"), _P(np.float32, flags="C"),
                                    _P(np.uint16), _P(np.uint16), _P(np.uint16), _P(np.float32, flags="C"),
                                    C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float]
        _lib = L
    return _lib


def ref():
    """The reference kernels compiled as C++, or None if the reference tree was
    not available to build them."""
    global _ref
    if _ref is None:
        path = _build.build_ref()
        if path is None or not os.path.exists(path):
            return None
        L = C.CDLL(path)
        L.ref_local_maxima.restype = C.c_uint
        L.ref_local_maxima.argtypes = [_P(np.float32, flags="C"), C.c_float, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint]
        L.ref_delta_fit.argtypes = [_P(np.float32, flags="C"), _P(np.float32, flags="C"),
                                    _P(np.uint16), _P(np.uint16), _P(np.uint16), _P(np.float32, flags="C"),
                                    C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float]
        L.ref_box_1d.argtypes = [_P(np.float32, flags="C"), _P(np.float32, flags="C"),
                                 C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        _ref = L
    return _ref


def box_1d(image, size, axis=0):
    """blur.py:157-188 semantics (2-D arrays are treated as (1, X, Y))."""
    a = np.ascontiguousarray(image, dtype=np.float32)
    if axis < 0:
        axis = a.ndim - 1
    if a.ndim == 2:
        sz, (sx, sy) = 1, a.shape
        axis += 1
    else:
        sz, sx, sy = a.shape
    out = np.empty_like(a)
    lib().orc_box_1d(a, out, sz, sx, sy, size // 2, axis)
    return out


def box_mean_f64(image, delta, axis):
    a = np.ascontiguousarray(image, dtype=np.float64)
    sz, sx, sy = a.shape
    out = np.empty_like(a)
    lib().orc_box_mean_f64(a, out, sz, sx, sy, delta, axis)
    return out


def reflect(arr, i, axis=0, mode="out"):
    """fill.py:54-111 (returns a reflected copy)."""
    res = np.array(arr, dtype=np.float32, copy=True)
    if axis < 0:
        axis += res.ndim
    n = res.shape[axis]
    if i < 0:
        i += n
    shape = np.array(res.shape, np.int64)
    strides = np.array([s // 4 for s in res.strides], np.int64)
    lib().orc_mirror(res.ctypes.data, res.ndim, shape, strides, axis, i, 0 if mode == "out" else 1)
    return res


def local_maxima(image, threshold, delta):
    """maxima.cu:1-145: (z, x, y) uint16 arrays of the maxima in raster order."""
    im = np.ascontiguousarray(image, dtype=np.float32)
    d, h, w = im.shape
    n = lib().orc_local_maxima(im, np.float32(threshold), delta, d, h, w, None, None, None, 0)
    z = np.zeros(n, np.uint16)
    x = np.zeros(n, np.uint16)
    y = np.zeros(n, np.uint16)
    if n:
        lib().orc_local_maxima(im, np.float32(threshold), delta, d, h, w,
                               z.ctypes.data, x.ctypes.data, y.ctypes.data, n)
    return z, x, y


def delta_fit(image, raw, z, x, y, delta_fit, sigmaZ=1.0, sigmaXY=1.5):
    im = np.ascontiguousarray(image, dtype=np.float32)
    rw = np.ascontiguousarray(raw, dtype=np.float32)
    n = len(z)
    out = np.zeros((n, 8), np.float32)
    if n:
        Z, X, Y = im.shape
        lib().orc_delta_fit(im, rw, np.ascontiguousarray(z, np.uint16), np.ascontiguousarray(x, np.uint16),
                            np.ascontiguousarray(y, np.uint16), out, n, Z, X, Y, delta_fit,
                            np.float32(sigmaZ), np.float32(sigmaXY))
    return out


def find_local_maxima(image, threshold=None, delta=1, delta_fit=0, raw=None, sigmaZ=1, sigmaXY=1.5, **kwargs):
    """maxima.py:17-98 restated: (N, 8) float32 rows [zc, xc, yc, bg, a, habs, hn, h]."""
    if delta > 5:
        raise TypeError("Delta must be an less than or equal to 5 due to MAX_KERNEL_POINTS")
    z, x, y = local_maxima(image, threshold, delta)
    if len(z) == 0:
        return np.zeros((0, 8), np.float32)
    return globals()["delta_fit"](image, raw, z, x, y, delta_fit, sigmaZ, sigmaXY)


def ref_find_local_maxima(image, threshold, delta, delta_fit, raw, sigmaZ=1.0, sigmaXY=1.5):
    """The reference kernels themselves (compiled as C++), same return value."""
    R = ref()
    im = np.ascontiguousarray(image, dtype=np.float32)
    d, h, w = im.shape
    cap = im.size
    z = np.zeros(cap, np.uint16)
    x = np.zeros(cap, np.uint16)
    y = np.zeros(cap, np.uint16)
    n = R.ref_local_maxima(im, np.float32(threshold), delta, d, h, w, z.ctypes.data, x.ctypes.data,
                           y.ctypes.data, cap)
    z, x, y = z[:n].copy(), x[:n].copy(), y[:n].copy()
    out = np.zeros((n, 8), np.float32)
    if n:
        rw = np.ascontiguousarray(raw, dtype=np.float32)
        R.ref_delta_fit(im, rw, z, x, y, out, n, d, h, w, delta_fit, np.float32(sigmaZ), np.float32(sigmaXY))
    return out


def ref_box_1d(image, size, axis):
    R = ref()
    a = np.ascontiguousarray(image, dtype=np.float32)
    if a.ndim == 2:
        sz, (sx, sy) = 1, a.shape
        axis += 1
    else:
        sz, sx, sy = a.shape
    out = np.empty_like(a)
    R.ref_box_1d(a, out, sz, sx, sy, size // 2, axis)
    return out


def sort_rows(Xh):
    """Row order of the reference output is set by atomics; compare after a
    lexsort on (z, x, y) as scripts/compare_xh.py:11-17 does."""
    Xh = np.asarray(Xh)
    if len(Xh) == 0:
        return Xh
    return Xh[np.lexsort((Xh[:, 2], Xh[:, 1], Xh[:, 0]))]


def match_rows(got, want, tol=1e-2):
    """Pairs the rows of two Xh arrays one to one by nearest centroid (the
    row order of either side is arbitrary, and sorting by float centroids
    misaligns rows whose coordinates differ in the last bits).  Returns the
    paired (got, want); raises AssertionError if the sets differ."""
    from scipy.spatial import cKDTree
    got = np.asarray(got)
    want = np.asarray(want)
    assert got.shape == want.shape, (got.shape, want.shape)
    if len(got) == 0:
        return got, want
    d, idx = cKDTree(want[:, :3].astype(np.float64)).query(got[:, :3].astype(np.float64))
    assert np.all(d <= tol), float(d.max())
    assert len(np.unique(idx)) == len(idx), "rows do not pair one to one"
    return got, want[idx]
