"""NumPy/SciPy restatement of ``mermake/align.py`` and ``mermake/utils.py:10-36``
(test oracle only).

The correlation of the two splat images is computed with a float64 FFT and
rounded to the nearest integer: both images are 0/1, so the full linear
correlation is an integer count per shift and the rounding recovers it
exactly.  The argmax then takes the first maximal index, as ``argmax`` does.
Nearest neighbours come from ``scipy.spatial.cKDTree`` (the reference uses
``cupyx.scipy.spatial.KDTree``, align.py:32).
"""
from __future__ import annotations

import numpy as np
import scipy.fft as sfft
from scipy.spatial import cKDTree


def fftconvolve_full(a, b):
    """utils.py:10-36 (mode='full') in float64."""
    shape = [sa + sb - 1 for sa, sb in zip(a.shape, b.shape)]
    fa = sfft.rfftn(a.astype(np.float64), shape)
    fb = sfft.rfftn(b.astype(np.float64), shape)
    return sfft.irfftn(fa * fb, shape)


class Aligner:
    """align.py:12-129."""

    def __init__(self, X_ref, resc=5, trim=10, th=None):
        self.resc = resc
        self.trim = trim
        self.th = th
        X_ref = np.asarray(X_ref)
        if th:
            X_ref = self.threshold(X_ref)
        if X_ref.size == 0:
            raise ValueError("No points left after thresholding; cannot build KDTree. "
                             "Check your data and/or threshold value.")
        self.X_ref = X_ref[:, :3]
        self.tree = cKDTree(self.X_ref)
        self.im_ref, self.Xm_ref = self.get_im_from_Xh(self.X_ref)

    def get_im_from_Xh(self, Xh):
        """align.py:37-59: round(X/resc), trim x/y by ``trim`` from the extremes,
        splat ones into an image anchored at the origin."""
        X = np.round(Xh / self.resc).astype(np.int32)
        Xm = X.min(axis=0)
        XM = X.max(axis=0)
        n = np.asarray([0, self.trim, self.trim], dtype=np.int32)
        keep = np.all((X <= (XM - n)) & (X >= (Xm + n)), axis=-1)
        X = X[keep]
        if X.shape[0] == 0:
            return np.zeros((1, 1, 1), np.float32), np.array([0, 0, 0], np.int32)
        Xm = np.array([0, 0, 0], np.int32)
        sz = X.max(axis=0) + 1
        imf = np.zeros(sz.tolist(), np.float32)
        imf[tuple(X.T)] = 1
        return imf, Xm

    def get_Xtzxy(self, X, tzxy0, target=3):
        """align.py:61-77: five nearest-neighbour refinements with radii
        linspace(resc, target, 5)."""
        tzxy = tzxy0
        keep = np.zeros(len(X), bool)
        for dist_th in np.linspace(self.resc, target, 5):
            XT = X - tzxy
            ds, inds = self.tree.query(XT)
            keep = ds < dist_th
            X_ref_ = self.X_ref[inds[keep]]
            X_ = X[keep]
            if X_.shape[0] == 0:
                continue
            tzxy = np.mean((X_ - X_ref_).astype(np.float64), axis=0).astype(np.float32)
        return tzxy, int(np.sum(keep))

    def coarse_shift(self, X):
        """align.py:103-111: argmax of the full correlation, in voxels * resc."""
        im, Xm = self.get_im_from_Xh(X)
        cor = np.rint(fftconvolve_full(im, self.im_ref[::-1, ::-1, ::-1]))
        idx = np.array(np.unravel_index(np.argmax(cor), cor.shape))
        tzxy = idx - np.asarray(self.im_ref.shape) + 1 + Xm - self.Xm_ref
        return tzxy * self.resc

    def get_best_translation_points(self, X, target=3, return_counts=False):
        """align.py:94-118."""
        X = np.asarray(X)
        if self.th:
            X = self.threshold(X)
        X = X[:, :3]
        tzxy = self.coarse_shift(X)
        tzxy, npts = self.get_Xtzxy(X, tzxy, target=target)
        if return_counts:
            return tzxy, npts
        return tzxy

    def get_shifted_slices(self, X, shape):
        """align.py:79-92."""
        tzxy = self.get_best_translation_points(X)
        tzxy = np.round(tzxy).astype(int).tolist()
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
        """align.py:121-129: rows whose LAST column exceeds th."""
        dim = X.shape[1]
        if X.size:
            X = X[X[:, -1] > self.th]
            if X.size:
                return X
        return np.zeros([0, dim])


class DualAligner:
    """align.py:131-156."""

    def __init__(self, ref, th=None):
        self.plus = Aligner(np.asarray(ref.Xh_plus)[:, :3], th=th)
        self.minus = Aligner(np.asarray(ref.Xh_minus)[:, :3], th=th)
        self.th = th

    def get_best_translation_pointsV2(self, obj):
        tp, Np = self.plus.get_best_translation_points(obj.Xh_plus, return_counts=True)
        tm, Nm = self.minus.get_best_translation_points(obj.Xh_minus, return_counts=True)
        return combine(tp, tm, Np, Nm) + (tp, tm, Np, Nm)


def combine(tp, tm, Np, Nm):
    """align.py:147-154: weighted mean when the two estimates agree within 2,
    else the estimate with more matches; the sign is flipped."""
    if Np + Nm == 0:
        return (np.zeros(3),)
    if np.max(np.abs(tm - tp)) <= 2:
        return (-(tp * Np + tm * Nm) / (Np + Nm),)
    return (-tp if Np >= Nm else -tm,)


def drift(block, th=4):
    """align.py:163-176 without the file checks: the middle round is the
    reference; returns the list of per-round tuples."""
    ref = block[len(block) // 2]
    dual = DualAligner(ref, th=th)
    return [dual.get_best_translation_pointsV2(im) for im in block]
