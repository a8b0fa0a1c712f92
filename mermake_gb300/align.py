"""Drift alignment with the reference's call surface (mermake/align.py:12-176),
computed by the kernels of ``csrc/drift.cu``.

``Aligner`` keeps the reference set's points and splat image resident on the
device; ``get_best_translation_points`` runs threshold, splat, the exact
correlation peak and the nearest-neighbour refinement there and returns the
shift on the host (a float32 NumPy array, like the reference's after its
``.tolist()``/``float()`` syncs).
"""
from __future__ import annotations

import ctypes as C
import os
import pickle

import numpy as np
import torch

from . import _lib
from ._arrays import as_device


def _rows(X):
    t = as_device(X, torch.float32)
    if t.dim() != 2 or t.shape[1] < 3:
        raise ValueError("point sets are (N, >=3) arrays")
    if t.stride(1) != 1:
        t = t.contiguous()
    return t


class Aligner:
    """align.py:12-129."""

    def __init__(self, X_ref, resc=5, trim=10, th=None):
        self.resc = int(resc)
        self.trim = int(trim)
        self.th = th
        X = _rows(X_ref)
        thv = float("nan") if not th else float(th)
        h = C.c_void_p()
        L = _lib.lib()
        _lib.check(L.mm_aligner_create(_lib.ptr(X) if X.numel() else None, X.shape[0], X.shape[1],
                                       X.stride(0) if X.numel() else X.shape[1], thv, self.resc, self.trim,
                                       C.byref(h), _lib.stream_ptr()))
        self._h = h
        n, nv, shp = C.c_int(), C.c_int(), (C.c_int * 3)()
        _lib.check(L.mm_aligner_info(h, C.byref(n), C.byref(nv), shp))
        self.n_ref = n.value
        self.n_ref_voxels = nv.value
        self.ref_shape = tuple(shp)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.mm_aligner_destroy(h)
            self._h = None

    def get_best_translation_points(self, X, target=3, return_counts=False):
        """align.py:94-118: shift (z, x, y) of X against the reference, in pixels."""
        Xd = _rows(X)
        t = (C.c_float * 3)()
        n = C.c_int()
        _lib.check(_lib.lib().mm_aligner_translation(self._h, _lib.ptr(Xd) if Xd.numel() else None, Xd.shape[0],
                                                     Xd.shape[1], Xd.stride(0) if Xd.numel() else Xd.shape[1],
                                                     float(target), t, C.byref(n), _lib.stream_ptr()))
        tzxy = np.array(list(t), dtype=np.float32)
        if return_counts:
            return tzxy, n.value
        return tzxy

    def get_shifted_slices(self, X, shape):
        """align.py:79-92: overlapping slices of signal and background for the
        rounded shift."""
        tzxy = np.round(self.get_best_translation_points(X)).astype(int).tolist()
        sig, bk = [], []
        for t, sh in zip(tzxy, shape):
            if t > 0:
                sig.append(slice(t, sh))
                bk.append(slice(0, sh - t))
            else:
                sig.append(slice(0, sh + t))
                bk.append(slice(-t, sh))
        return tuple(bk), tuple(sig)

    def threshold(self, X):
        """align.py:121-129: rows whose last column exceeds th."""
        X = as_device(X)
        dim = X.shape[1]
        if X.numel():
            X = X[X[:, -1] > self.th]
            if X.numel():
                return X
        return torch.zeros((0, dim), device=X.device)


class DualAligner:
    """align.py:131-156: aligners on the + and - DAPI maxima."""

    def __init__(self, ref, th=None):
        self.plus = Aligner(_rows(ref.Xh_plus)[:, :3], th=th)
        self.minus = Aligner(_rows(ref.Xh_minus)[:, :3], th=th)
        self.th = th

    def get_best_translation_pointsV2(self, obj):
        tp, Np = self.plus.get_best_translation_points(obj.Xh_plus, return_counts=True)
        tm, Nm = self.minus.get_best_translation_points(obj.Xh_minus, return_counts=True)
        if Np + Nm == 0:
            tzxyf = np.zeros(3)
        elif np.max(np.abs(tm - tp)) <= 2:
            tzxyf = -(tp * Np + tm * Nm) / (Np + Nm)
        else:
            tzxyf = -tp if Np >= Nm else -tm
        return tzxyf, tp, tm, Np, Nm


def drift_save(data, filepath):
    """align.py:158-161."""
    with open(filepath, "wb") as f:
        pickle.dump(data, f)


def drift(block):
    """align.py:163-176: every round of a FOV block against the block's middle
    round.  Returns ``([drifts, files, ifov, ref_path], filepath)``, or None when
    the block's drift file already exists."""
    filepath = block.drift_file() if hasattr(block, "drift_file") else None
    if filepath is not None and os.path.exists(filepath):
        return None
    ifov = block.ifov() if hasattr(block, "ifov") else None
    ref = block[len(block) // 2]
    dual = DualAligner(ref, th=4)
    drifts, files = [], []
    for image in block:
        drifts.append(dual.get_best_translation_pointsV2(image))
        files.append(os.path.dirname(getattr(image, "path", "") or ""))
    return [drifts, files, ifov, getattr(ref, "path", None)], filepath
