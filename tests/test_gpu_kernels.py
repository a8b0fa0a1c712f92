"""GPU parity of the FFT engine, maxima + fit, box blur, reflect and uint16
subtraction against the CPU oracle and the reference's known answers."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import ckernels as ck

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mm():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mermake_gb300 import _lib, blur, fill, maxima
    from mermake_gb300 import math as mmath
    _lib.lib()
    return dict(lib=_lib, blur=blur, fill=fill, maxima=maxima, math=mmath)


# every padded length the benchmark configurations and the reference fixture use,
# plus primes and composites around them
FFT_LENGTHS = [1, 2, 3, 4, 5, 7, 8, 11, 13, 16, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 58, 59, 61, 67, 71, 73, 78,
               79, 83, 88, 89, 97, 98, 101, 103, 105, 107, 109, 113, 118, 121, 127, 131, 143, 148, 158, 178, 226,
               238, 239, 256, 437, 478, 678, 717, 956, 1000, 1024, 1073, 2048, 2053]


@pytest.mark.parametrize("n", FFT_LENGTHS)
@pytest.mark.parametrize("inverse", [False, True])
def test_fft_engine_matches_float64(mm, n, inverse):
    rng = np.random.default_rng(n)
    nl = 5
    x = (rng.standard_normal((n, nl)) + 1j * rng.standard_normal((n, nl))).astype(np.complex64)
    d = torch.from_numpy(x.view(np.float32).reshape(n, nl, 2)).cuda().contiguous()
    L = mm["lib"].lib()
    mm["lib"].check(L.mm_fft_c2c(mm["lib"].ptr(d), n, nl, int(inverse), mm["lib"].stream_ptr()))
    got = d.cpu().numpy().view(np.complex64)[..., 0]
    ref = np.fft.ifft(x.astype(np.complex128), axis=0) * n if inverse else np.fft.fft(x.astype(np.complex128), axis=0)
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 2e-6, err


def _maxima_case(mm, im, raw, th, delta, dfit, sz=1.0, sxy=1.5):
    got = mm["maxima"].find_local_maxima(torch.from_numpy(im).cuda(), th, delta, dfit,
                                         torch.from_numpy(raw).cuda(), sz, sxy).cpu().numpy()
    want = ck.find_local_maxima(im, th, delta, dfit, raw, sz, sxy)
    return ck.sort_rows(got), ck.sort_rows(want)


def assert_rows_close(got, want):
    """Same maxima; centroids within 1e-3 px (plus the float32 oracle's own
    rounding, ~2e-6 of the coordinate); background, habs and h (copies of
    volume values) within 1e-4 relative; the correlation columns a and hn
    (dimensionless, |.| <= 1) within 1e-4 absolute."""
    got, want = ck.match_rows(got, want)
    if len(got) == 0:
        return
    tol = 1e-3 + 2e-6 * np.abs(want[:, :3])
    assert np.all(np.abs(got[:, :3] - want[:, :3]) <= tol)
    for c in (3, 5, 7):
        np.testing.assert_allclose(got[:, c], want[:, c], rtol=1e-4, atol=1e-30)
    for c in (4, 6):
        w, g = want[:, c], got[:, c]
        assert np.array_equal(np.isnan(w), np.isnan(g))
        ok = ~np.isnan(w)
        assert np.all(np.abs(g[ok] - w[ok]) <= 1e-4), c


def test_maxima_known_answers(mm):
    """test_maxima.py:26-166."""
    fm = mm["maxima"].find_local_maxima
    im = torch.zeros((5, 5, 5), device="cuda")
    im[1:4, 1:4, 1:4] = 0.5
    im[2, 2, 2] = 1.0
    r = fm(im, threshold=0.8, delta=1, delta_fit=1, raw=im.clone())
    assert r.shape == (1, 8) and torch.all(torch.abs(r[0, :3] - 2) < 0.5)
    im = torch.zeros((5, 5, 5), device="cuda")
    im[1, 1, 1], im[3, 3, 3] = 0.9, 0.6
    assert fm(im, threshold=0.5, delta=1, delta_fit=1, raw=im).shape[0] == 2
    assert fm(im, threshold=0.8, delta=1, delta_fit=1, raw=im).shape[0] == 1
    assert tuple(fm(im, threshold=1.5, delta=1, delta_fit=1, raw=im).shape) == (0, 8)
    im = torch.zeros((7, 7, 7), device="cuda")
    im[3, 3, 3], im[3, 3, 5] = 1.0, 0.9
    assert fm(im, threshold=0.5, delta=3, delta_fit=1, raw=im).shape[0] <= fm(im, 0.5, 1, 1, im).shape[0]
    with pytest.raises(TypeError, match="Delta must be an less than or equal to 5"):
        fm(torch.ones((3, 3, 3), device="cuda"), threshold=0.5, delta=6, delta_fit=1)
    r = fm(torch.ones((3, 3, 3), device="cuda"), threshold=0.5, delta=5, delta_fit=1)
    assert r.dtype == torch.float32 and r.dim() == 2
    for shape in [(2, 2, 2), (10, 5, 3), (1, 1, 1)]:
        x = torch.rand(shape, device="cuda")
        r = fm(x, threshold=0.9, delta=1, delta_fit=1, raw=x)
        assert r.shape[1] == 8
    raw16 = (torch.ones((3, 3, 3)) * 65535).to(torch.int32).to(torch.uint16).cuda()
    assert fm(torch.ones((3, 3, 3), device="cuda"), 0.5, 1, 1, raw16).shape[1] == 8


@pytest.mark.parametrize("shape,delta,dfit", [((12, 40, 50), 1, 3), ((9, 30, 33), 5, 5), ((6, 17, 9), 2, 1),
                                              ((5, 8, 8), 3, 0), ((3, 9, 4), 1, 2), ((1, 1, 1), 1, 1),
                                              ((2, 7, 1), 2, 2), ((20, 64, 64), 1, 3)])
def test_maxima_fit_match_oracle(mm, shape, delta, dfit):
    rng = np.random.default_rng(sum(shape) + delta)
    im = rng.random(shape).astype(np.float32)
    im[rng.random(shape) < 0.05] = 0.75  # plateaus: ties keep both
    raw = (rng.random(shape) * 1000).astype(np.float32)
    got, want = _maxima_case(mm, im, raw, 0.5, delta, dfit)
    assert_rows_close(got, want)


def test_maxima_strided_and_uint16_raw(mm):
    rng = np.random.default_rng(3)
    big = rng.random((10, 40, 60)).astype(np.float32)
    raw = rng.integers(0, 65535, (10, 40, 60)).astype(np.uint16)
    view = torch.from_numpy(big).cuda()[:, 3:33, 5:50]
    rview = torch.from_numpy(raw.astype(np.int32)).to(torch.uint16).cuda()[:, 3:33, 5:50]
    got = ck.sort_rows(mm["maxima"].find_local_maxima(view, 0.6, 1, 3, rview).cpu().numpy())
    want = ck.sort_rows(ck.find_local_maxima(big[:, 3:33, 5:50], 0.6, 1, 3, raw[:, 3:33, 5:50].astype(np.float32)))
    assert_rows_close(got, want)


def test_maxima_normalised_ties_of_distinct_raw_values(mm):
    """The maxima test compares normalised values: a neighbour whose raw value
    is larger but whose quotient by the divisor rounds to the same float32
    (3.9916298 and the next float, divided by 0.99041766) does not make the
    centre a non-maximum, while the raw comparison alone would; the negated
    volume mirrors it."""
    a = np.float32(3.9916298)
    b = np.nextafter(a, np.float32(10))
    div = np.float32(0.99041766)
    assert a < b and a / div == b / div
    im = np.full((5, 9, 9), 0.25, np.float32)
    im[2, 4, 4], im[2, 4, 5] = a, b
    raw = np.ones((5, 9, 9), np.float32)
    for neg in (False, True):
        src = -im if neg else im
        v = src / div
        if neg:
            v = -v
        got = mm["maxima"].find_local_maxima(torch.from_numpy(src).cuda(), 1.0, 2, 1, torch.from_numpy(raw).cuda(),
                                             norm_div=float(div), negate=neg).cpu().numpy()
        want = ck.find_local_maxima(v.astype(np.float32), 1.0, 2, 1, raw)
        # both voxels are maxima (their fits coincide, so the rows are equal)
        assert len(want) == 2 and got.shape == want.shape
        np.testing.assert_allclose(ck.sort_rows(got), ck.sort_rows(want), rtol=1e-5, atol=1e-4)


def test_maxima_normalise_and_negate_on_read(mm):
    """DAPI: v / rms then -v (__main__.py:221-225), applied on read, bit-identical
    to dividing the volume first."""
    rng = np.random.default_rng(11)
    im = (rng.standard_normal((8, 30, 30)) * 3).astype(np.float32)
    raw = rng.integers(0, 4000, (8, 30, 30)).astype(np.uint16)
    div = np.float32(1.7371)
    for neg in (False, True):
        v = im / div
        if neg:
            v = -v
        got = mm["maxima"].find_local_maxima(torch.from_numpy(im).cuda(), 1.0, 2, 2,
                                             torch.from_numpy(raw.astype(np.int32)).to(torch.uint16).cuda(),
                                             norm_div=float(div), negate=neg).cpu().numpy()
        want = ck.find_local_maxima(v.astype(np.float32), 1.0, 2, 2, raw.astype(np.float32))
        assert_rows_close(ck.sort_rows(got), ck.sort_rows(want))


def test_box_1d_known_answers(mm):
    """test_blur.py:62-116."""
    b = mm["blur"]
    arr = torch.zeros((3, 3, 3), device="cuda")
    arr[0, 0, 0] = 1
    for ax in range(3):
        want = np.zeros((3, 3, 3), np.float32)
        idx = [0, 0, 0]
        want[0, 0, 0] = 0.5
        idx[ax] = 1
        want[tuple(idx)] = 0.33333334
        np.testing.assert_allclose(b.box_1d(arr, 2, axis=ax).cpu().numpy(), want, rtol=1e-6)
    with pytest.raises(ValueError):
        b.box_1d(arr, 2, axis=0, out=arr)
    with pytest.raises(ValueError):
        b.box(torch.ones((3, 3, 3), device="cuda"), 3, axes=(0, 1, 2, 3))
    with pytest.raises(TypeError):
        b.box(torch.ones((3, 3, 3), device="cuda"), 3, axes="bad")
    with pytest.raises(ValueError):
        b.box(torch.ones((3, 3, 3), device="cuda"), (3, 3), axes=(0, 1, 2))


@pytest.mark.parametrize("shape,axes,size", [((5, 5), (0,), 3), ((4, 4, 4), (0, 1), 3), ((4, 4, 4), (1, 2), (3, 5)),
                                             ((13, 70, 90), (1, 2), (31, 31)), ((1, 300, 280), (1, 2), 21)])
def test_box_matches_oracle(mm, shape, axes, size):
    rng = np.random.default_rng(5)
    arr = (rng.random(shape) * 100).astype(np.float32)
    got = mm["blur"].box(torch.from_numpy(arr).cuda(), size, axes=axes).cpu().numpy()
    sizes = [size] * len(axes) if isinstance(size, int) else size
    want = arr
    for ax, s in zip(axes, sizes):
        want = ck.box_1d(want, s, axis=ax)
    np.testing.assert_allclose(got, want, rtol=1e-6, atol=1e-5)


D2 = np.array([[1, 2, 3, 4, 5], [6, 7, 8, 9, 10], [11, 12, 13, 14, 15]], np.float32)


@pytest.mark.parametrize("arr,i,axis,mode", [(np.arange(1, 6, dtype=np.float32), 2, 0, "out"),
                                             (np.arange(1, 6, dtype=np.float32), 2, 0, "in"),
                                             (D2, 1, 0, "in"), (D2, 3, 1, "in"), (D2, 1, 0, "out"),
                                             (D2, 2, 1, "out"), (D2, 2, 0, "in")])
def test_reflect_matches_reference_answers(mm, arr, i, axis, mode):
    got = mm["fill"].reflect(torch.from_numpy(arr).cuda(), i, axis=axis, mode=mode).cpu().numpy()
    np.testing.assert_array_equal(got, ck.reflect(arr, i, axis, mode))


def test_reflect_errors(mm):
    r = mm["fill"].reflect
    a = torch.tensor([1.0, 2.0, 3.0], device="cuda")
    with pytest.raises(IndexError):
        r(a, i=5, axis=0)
    with pytest.raises(ValueError):
        r(a, i=1, mode="invalid")
    with pytest.raises(IndexError):
        r(a, i=1, axis=1)
    with pytest.raises(ValueError, match="output array shape"):
        r(a, i=1, out=torch.zeros(4, device="cuda"))
    out = torch.zeros(3, device="cuda")
    assert r(a, i=1, out=out) is out


def test_subtract_u16(mm):
    rng = np.random.default_rng(2)
    x = rng.integers(0, 65536, (4, 7, 9)).astype(np.uint16)
    y = rng.integers(0, 65536, (4, 7, 9)).astype(np.uint16)
    tx = torch.from_numpy(x.astype(np.int32)).to(torch.uint16).cuda()
    ty = torch.from_numpy(y.astype(np.int32)).to(torch.uint16).cuda()
    r = mm["math"].subtract_reflect(tx, ty).to(torch.int32).cpu().numpy()
    np.testing.assert_array_equal(r, np.abs(x.astype(np.int64) - y.astype(np.int64)))
    c = mm["math"].subtract_clamp(tx, ty).to(torch.int32).cpu().numpy()
    np.testing.assert_array_equal(c, np.maximum(x.astype(np.int64) - y.astype(np.int64), 0))
    # strided views as __main__.py:250 uses them
    out = tx.clone()
    mm["math"].subtract_reflect(tx[:, 1:, :-2], ty[:, :-1, 2:], out=out[:, 1:, :-2])
    want = x.astype(np.int64).copy()
    want[:, 1:, :-2] = np.abs(x[:, 1:, :-2].astype(np.int64) - y[:, :-1, 2:])
    np.testing.assert_array_equal(out.to(torch.int32).cpu().numpy(), want)
