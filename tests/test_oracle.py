"""The oracle is pinned before it is trusted: against the reference's golden
deconvolution slices, the reference's own unit-test known answers, the
reference kernels compiled as C++ (where the reference tree is present) and
the reference's drift pickle."""
import json
import os
import types

import numpy as np
import pytest

from oracle import align as oalign
from oracle import ckernels as ck
from oracle import deconv as od


def f16_tolerance(gold):
    """One float16 spacing of the golden value plus 1e-5 of the range: the
    goldens are float16 roundings of float32 results."""
    g = np.abs(gold.astype(np.float64))
    return np.spacing(np.abs(gold)).astype(np.float64) + 1e-5 * g.max()


def load_tile(golden_dir, k):
    g = np.load(os.path.join(golden_dir, "deconv_tiles.npz"))
    ts, x, y, x0, x1, y0, y1, X, Y, Z, ov, zs = [int(v) for v in g[f"t{k}_meta"]]
    crop = g[f"t{k}_crop_u8"].astype(np.uint16) ** 2
    img = np.zeros((Z, X, Y), np.uint16)
    img[:, x0:x1, y0:y1] = crop
    return dict(ts=ts, x=x, y=y, box=(x, y, x0, x1, y0, y1), img=img, Z=Z, ov=ov, zs=zs,
                gold=g[f"t{k}_golden_f16"])


@pytest.mark.parametrize("k", [0, 1, 2])
def test_oracle_deconv_matches_reference_golden(golden_dir, k):
    """test_deconvolver.py:422-434 (full_deconv, tile 300/500, overlap 89,
    zpad = Z = 35, beta 1e-3) on the tiles stored in tests/golden."""
    t = load_tile(golden_dir, k)
    psf = np.load(os.path.join(golden_dir, "psf_750.npz"))["psf"]
    W = od.wiener_half(psf, t["Z"], t["ts"], t["Z"], t["ov"], 1e-3)
    res, _ = od.deconv_tile(t["img"], None, t["box"], W, t["ts"], t["Z"], t["ov"])
    ov = t["ov"]
    out = res[:, ov:-ov, ov:-ov][:: t["zs"]]
    gold = t["gold"]
    out = out[:, : gold.shape[1], : gold.shape[2]]
    err = np.abs(out - gold.astype(np.float64))
    assert np.all(err <= f16_tolerance(gold)), err.max()


def test_box_1d_known_answers():
    """test_blur.py:62-100."""
    arr = np.zeros((3, 3, 3), np.float32)
    arr[0, 0, 0] = 1
    want0 = np.zeros((3, 3, 3), np.float32)
    want0[0, 0, 0], want0[1, 0, 0] = 0.5, 0.33333334
    np.testing.assert_allclose(ck.box_1d(arr, 2, axis=0), want0, rtol=1e-6)
    want1 = np.zeros((3, 3, 3), np.float32)
    want1[0, 0, 0], want1[0, 1, 0] = 0.5, 0.33333334
    np.testing.assert_allclose(ck.box_1d(arr, 2, axis=1), want1, rtol=1e-6)
    want2 = np.zeros((3, 3, 3), np.float32)
    want2[0, 0, 0], want2[0, 0, 1] = 0.5, 0.33333334
    np.testing.assert_allclose(ck.box_1d(arr, 2, axis=2), want2, rtol=1e-6)


def numpy_box_1d(arr, size, axis=0):
    """The reference's NumPy spec of the truncated window (test_blur.py:9-23)."""
    arr = np.asarray(arr, dtype=np.float32)
    out = np.empty_like(arr)
    delta = size // 2
    for idx in np.ndindex(arr.shape):
        s = max(0, idx[axis] - delta)
        e = min(arr.shape[axis], idx[axis] + delta + 1)
        sl = [slice(i, i + 1) if ax != axis else slice(s, e) for ax, i in enumerate(idx)]
        out[idx] = arr[tuple(sl)].mean()
    return out


@pytest.mark.parametrize("shape,axis,size", [((5, 5), 0, 3), ((5, 5), 1, 3), ((4, 4, 4), 0, 3),
                                             ((4, 4, 4), 1, 5), ((4, 4, 4), 2, 3)])
def test_box_1d_matches_numpy_spec(shape, axis, size):
    """test_blur.py:26-37."""
    arr = np.arange(np.prod(shape), dtype=np.float32).reshape(shape)
    np.testing.assert_allclose(ck.box_1d(arr, size, axis=axis), numpy_box_1d(arr, size, axis), rtol=1e-6)


D2 = np.array([[1, 2, 3, 4, 5], [6, 7, 8, 9, 10], [11, 12, 13, 14, 15]], np.float32)

REFLECT_CASES = [  # test_fill.py:19-160
    (np.array([1, 2, 3, 4, 5], np.float32), 2, 0, "out", [1, 2, 3, 2, 1]),
    (np.array([1, 2, 3, 4, 5], np.float32), 2, 0, "in", [5, 4, 3, 4, 5]),
    (D2, 2, 0, "in", D2),
    (D2, 1, 0, "in", [[11, 12, 13, 14, 15], [6, 7, 8, 9, 10], [11, 12, 13, 14, 15]]),
    (D2, 2, 1, "in", [[5, 4, 3, 4, 5], [10, 9, 8, 9, 10], [15, 14, 13, 14, 15]]),
    (D2, 3, 1, "in", [[1, 2, 5, 4, 5], [6, 7, 10, 9, 10], [11, 12, 15, 14, 15]]),
    (D2, 0, 0, "out", D2),
    (D2, 1, 0, "out", [[1, 2, 3, 4, 5], [6, 7, 8, 9, 10], [1, 2, 3, 4, 5]]),
    (D2, 2, 1, "out", [[1, 2, 3, 2, 1], [6, 7, 8, 7, 6], [11, 12, 13, 12, 11]]),
]


@pytest.mark.parametrize("arr,i,axis,mode,want", REFLECT_CASES)
def test_reflect_known_answers(arr, i, axis, mode, want):
    np.testing.assert_array_equal(ck.reflect(arr, i, axis, mode), np.asarray(want, np.float32))


def test_maxima_known_answers():
    """test_maxima.py:26-100."""
    im = np.zeros((5, 5, 5), np.float32)
    im[1:4, 1:4, 1:4] = 0.5
    im[2, 2, 2] = 1.0
    r = ck.find_local_maxima(im, 0.8, 1, 1, im)
    assert r.shape == (1, 8) and np.all(np.abs(r[0, :3] - 2) < 0.5)
    im = np.zeros((5, 5, 5), np.float32)
    im[1, 1, 1], im[3, 3, 3] = 0.9, 0.6
    assert len(ck.find_local_maxima(im, 0.5, 1, 1, im)) == 2
    assert len(ck.find_local_maxima(im, 0.8, 1, 1, im)) == 1
    assert ck.find_local_maxima(im, 1.5, 1, 1, im).shape == (0, 8)
    im = np.zeros((7, 7, 7), np.float32)
    im[3, 3, 3], im[3, 3, 5] = 1.0, 0.9
    assert len(ck.find_local_maxima(im, 0.5, 3, 1, im)) <= len(ck.find_local_maxima(im, 0.5, 1, 1, im))
    with pytest.raises(TypeError, match="Delta must be an less than or equal to 5"):
        ck.find_local_maxima(im, 0.5, 6, 1, im)


def test_ckernels_match_reference_kernels_compiled():
    """kernels.c against the reference's maxima.cu / blur.cu compiled as C++."""
    if ck.ref() is None:
        pytest.skip("reference tree not available to build oracle/_ref")
    rng = np.random.default_rng(7)
    for shape, delta, dfit in [((10, 30, 40), 1, 3), ((8, 20, 25), 5, 5), ((5, 7, 9), 2, 1), ((6, 6, 6), 3, 0),
                               ((3, 9, 4), 1, 2)]:
        im = rng.random(shape).astype(np.float32)
        raw = (rng.random(shape) * 1000).astype(np.float32)
        a = ck.sort_rows(ck.find_local_maxima(im, 0.5, delta, dfit, raw))
        b = ck.sort_rows(ck.ref_find_local_maxima(im, 0.5, delta, dfit, raw))
        assert a.shape == b.shape
        np.testing.assert_array_equal(a, b)
    for ax in range(3):
        im = rng.random((5, 6, 7)).astype(np.float32) * 100
        np.testing.assert_array_equal(ck.box_1d(im, 7, ax), ck.ref_box_1d(im, 7, ax))


def test_drift_matches_reference_pickle(golden_dir):
    """drift_Conv_zscan__020--_set1.pkl: self-alignment of the dapiFeatures
    fixture through DualAligner(th=4) (align.py:131-176)."""
    d = np.load(os.path.join(golden_dir, "dapi_features.npz"))
    kat = json.load(open(os.path.join(golden_dir, "drift_kat.json")))
    im = types.SimpleNamespace(Xh_plus=d["Xh_plus"], Xh_minus=d["Xh_minus"])
    (tf, tp, tm, Np, Nm), = oalign.drift([im])
    want = kat["drifts"][0]
    np.testing.assert_array_equal(tf, want[0])
    np.testing.assert_array_equal(tp, want[1])
    np.testing.assert_array_equal(tm, want[2])
    assert (Np, Nm) == (want[3], want[4]) == (621, 261)


def test_dual_aligner_rules():
    """test_align.py:199-233: weighted mean when within 2, else the stronger set."""
    assert np.allclose(oalign.combine(np.array([1, 2, 3.]), np.array([1, 2, 3.]), 10, 5)[0], [-1, -2, -3])
    assert np.allclose(oalign.combine(np.array([1, 2, 3.]), np.array([10, 20, 30.]), 10, 5)[0], [-1, -2, -3])
    assert np.allclose(oalign.combine(np.array([1, 2, 3.]), np.array([1, 2, 3.]), 0, 0)[0], [0, 0, 0])
