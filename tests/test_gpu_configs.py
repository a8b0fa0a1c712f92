"""GPU parity at the geometries the benchmark runs, against the FP64 oracle.

Each case runs the production instantiation of the kernels -- the kernel
variant, transform lengths, padding and batch form that the named workload
uses -- on a channel small enough for the oracle to finish in seconds:

* hyb colour of the 3-colour + DAPI FOV: Z = 50, tile 500, overlap 89,
  zpad 49 (Zp 148, P 678), uint16 with the quadratic flat field, 10 tiles in
  one batch, so the z step is the Z = 50 matrix form of the z operator; the
  tile extents in y are those of a 2048-wide FOV (589, 678, 678, 637, 137);
* DAPI block of that FOV: zpad 24 (Zp 98), delta 5 / fit 5, stitched,
  normalised by the RMS, both signs (mermake/__main__.py:215-225);
* the multi-PSF workload: tiles of 300 (P 478, the 239-point Rader stage),
  Z = 40, a PSF per tile, so the z step is the direct sum per tile;
* the single smFISH tile: 40 x 500 x 500, no flat field, the x = y = 0 tile
  whose far pad stays zero (mermake/deconvolver.py:132-144).

Voxels are compared with the FP64 oracle (|gpu - oracle| <= 1e-4 max|oracle|,
the maximum printed): the truncated box blur of tile_wise over the whole
yielded view, and the drivers' form -- the blur subtraction folded into the z
step -- over the voxels at least the box half-width from the tile edges,
which are all the drivers read.  The maxima sets are compared bit-exact the
way the parity contract states them: the oracle's C maxima + fit run on the
drivers' own deconvolved tiles and raw views, and must give the same spots
(centroids within 1e-3 px, heights within 1e-4 relative) as the batched
driver.
"""
import numpy as np
import pytest
import torch

from oracle import ckernels as ck
from oracle import deconv as od
from tests.test_gpu_kernels import assert_rows_close

pytestmark = pytest.mark.gpu

REL = 1e-4

HYB = dict(tile_size=500, overlap=89, beta=1e-4, threshold=3600, blur_radius=30, delta=1, delta_fit=3,
           sigmaZ=1, sigmaXY=1.5)
DAPI = dict(tile_size=500, overlap=89, beta=0.01, threshold=3.0, blur_radius=50, delta=5, delta_fit=5,
            sigmaZ=1, sigmaXY=1.5)


@pytest.fixture(scope="module")
def mm():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mermake_gb300 import deconvolver, pipeline, synth
    return dict(dc=deconvolver, pl=pipeline, synth=synth)


def tile_volumes(mm, dec, img, flat, blur_radius, mode):
    """Every tile's result and raw view from one batch of all tiles (the batch
    form the drivers use), as host float32 (nt, Z, P, P).  mode
    MM_BLUR_EXACT: the truncated box blur of tile_wise; MM_BLUR_SPECTRAL: the
    blur folded into the z step, the volumes the drivers compute."""
    from mermake_gb300 import _lib
    nt = dec.n_tiles(img.shape)
    shape = (nt, dec.tile_height, dec.P, dec.P)
    res = torch.empty(shape, dtype=torch.float32, device="cuda")
    raw = torch.empty(shape, dtype=torch.float32, device="cuda")
    with _lib.blur_mode(mode):
        dec._call(img, mm["dc"].MM_DTYPE_U16, flat, 0, nt, blur_radius, res_out=res, raw_out=raw)
    torch.cuda.synchronize()
    out = res.cpu().numpy(), raw.cpu().numpy()
    del res, raw
    torch.cuda.empty_cache()
    return out


def both_volumes(mm, dec, img, flat, blur_radius):
    from mermake_gb300 import _lib
    return (tile_volumes(mm, dec, img, flat, blur_radius, _lib.MM_BLUR_EXACT),
            tile_volumes(mm, dec, img, flat, blur_radius, _lib.MM_BLUR_SPECTRAL))


# A row's keep decision (overlap <= xc < extent - overlap on the fitted
# centroid, mermake/__main__.py:254-256) is a comparison of a float centroid,
# which both sides know to 1e-3 px.  On tiles at the field edge the padded
# data is a mirror image about the overlap line, so a maximum on that line has
# its centroid exactly on the keep boundary, and the comparison falls to the
# rounding of each side's sums.  Rows whose centroid lies within this margin of
# a boundary may be kept by either side; every other row must agree.
KEEP_MARGIN = 2e-3


def oracle_rows_on_gpu_tiles(dec, boxes, res, raw, a):
    """mermake/__main__.py:253-265 with the oracle's C maxima + fit run on the
    GPU's deconvolved tiles: keep ov <= xc, yc < extent - ov, shift by the
    tile origin, concatenate.  Returns (sure, edge): the kept rows farther
    than KEEP_MARGIN from a keep boundary, and the rows within it (either
    side of it)."""
    ov = a["overlap"]
    sure, edge = [], []
    for t, box in enumerate(boxes):
        xe, ye = dec._extent(box)
        Xh = ck.find_local_maxima(np.ascontiguousarray(res[t, :, :xe, :ye]), a["threshold"], a["delta"],
                                  a["delta_fit"], np.ascontiguousarray(raw[t, :, :xe, :ye]), a["sigmaZ"],
                                  a["sigmaXY"])
        c = Xh[:, 1:3].astype(np.float64)
        hi = np.array([xe - ov, ye - ov], np.float64)
        inside = np.all((c >= ov + KEEP_MARGIN) & (c < hi - KEEP_MARGIN), axis=-1)
        near = np.all((c >= ov - KEEP_MARGIN) & (c < hi + KEEP_MARGIN), axis=-1) & ~inside
        for rows, m in ((sure, inside), (edge, near)):
            R = Xh[m].copy()
            R[:, 1] += box[0] - ov
            R[:, 2] += box[1] - ov
            rows.append(R)
    cat = lambda L: np.concatenate(L) if L else np.zeros((0, 8), np.float32)
    return cat(sure), cat(edge)


def assert_kept_rows_match(got, sure, edge):
    """Every oracle row clear of a keep boundary is among the GPU's rows, each
    GPU row pairs one to one with an oracle row (clear or at a boundary), and
    the paired rows agree within the fit tolerances."""
    from scipy.spatial import cKDTree
    allw = np.concatenate([sure, edge])
    d, idx = cKDTree(allw[:, :3].astype(np.float64)).query(got[:, :3].astype(np.float64))
    assert np.all(d <= 1e-2), float(d.max())
    assert len(np.unique(idx)) == len(idx), "rows do not pair one to one"
    assert np.isin(np.arange(len(sure)), idx).all(), "a row clear of the keep boundaries is missing"
    n_edge = int((idx >= len(sure)).sum())
    print("kept rows: %d clear of the boundaries, %d of %d boundary rows kept" % (len(sure), n_edge, len(edge)))
    assert_rows_close(got, allw[idx])


def check_tiles_against_oracle(dec, img_np, flat_np, boxes, which, exact, folded, W, a, zpad):
    """Voxels of the chosen tiles against the FP64 oracle, within REL of its
    maximum: the truncated blur over the whole yielded view, the folded blur
    (the drivers' volumes) over the voxels at least the box half-width d from
    the padded tile's edges; raw views bit-exact.  Returns the largest
    relative errors (truncated, folded)."""
    worst = [0.0, 0.0]
    d = a["blur_radius"] // 2
    for t in which:
        W_t = W[0] if len(W) == 1 else W[t]
        want, want_raw = od.deconv_tile(img_np, flat_np, boxes[t], W_t, a["tile_size"], zpad, a["overlap"],
                                        a["blur_radius"])
        xe, ye = dec._extent(boxes[t])
        assert want.shape[1:] == (xe, ye)
        scale = np.abs(want).max()
        got = exact[0][t, :, :xe, :ye].astype(np.float64)
        e0 = np.abs(got - want).max() / scale
        inner = (slice(None), slice(d, min(xe, dec.P - d)), slice(d, min(ye, dec.P - d)))
        e1 = np.abs(folded[0][t][inner].astype(np.float64) - want[inner]).max() / scale
        print("tile", t, boxes[t], "max |gpu - oracle| / max|oracle| = %.3g (truncated), %.3g (folded, inner)"
              % (e0, e1))
        assert e0 < REL and e1 < REL, (t, e0, e1)
        np.testing.assert_array_equal(exact[1][t, :, :xe, :ye], want_raw)
        np.testing.assert_array_equal(folded[1][t, :, :xe, :ye], want_raw)
        worst = [max(worst[0], e0), max(worst[1], e1)]
    return worst


def test_hyb_colour_at_fov_geometry(mm):
    """A colour of the 3-colour FOV (Z 50, tile 500, zpad 49, flat field),
    10 tiles: the Z = 50 z operator, the compile-time 678-point engine and
    the uint16 + flat gather, against the oracle."""
    synth = mm["synth"]
    Z, X, Y = 50, 1000, 2048
    gain = synth.flat_gain(X, Y)
    img = synth.hyb_stack(Z, X, Y, 40000 * X * Y // 2048 ** 2, 1017, gain=gain)
    psf = synth.gaussian_psf((40, 40, 40), 2.0, 1.3)
    dec = mm["dc"].Deconvolver(psf, (Z, X, Y), zpad=Z - 1, **HYB)
    dimg, dflat = img.cuda(), torch.from_numpy(gain).cuda()
    boxes = dec.tile_boxes(img.shape)
    assert len(boxes) == 10 and dec.z_operator is not None
    assert sorted({b[5] - b[4] for b in boxes}) == [137, 589, 637, 678]
    rows = mm["pl"].hyb_spots(dec, dimg, dflat, batch=-1, **HYB).cpu().numpy()
    exact, folded = both_volumes(mm, dec, dimg, dflat, HYB["blur_radius"])
    W = [od.wiener_half(psf, Z, 500, Z - 1, 89, HYB["beta"])]
    # reflect-in corner, the clipped 637 extent, the thin 137 edge, and an x reflect-out interior-y tile
    err = check_tiles_against_oracle(dec, img.numpy(), gain, boxes, (0, 3, 4, 6), exact, folded, W, HYB, Z - 1)
    print("hyb fov geometry: worst voxel error %.3g / %.3g of max" % tuple(err))
    del exact
    sure, edge = oracle_rows_on_gpu_tiles(dec, boxes, folded[0], folded[1], HYB)
    assert len(sure) > 1000 and len(edge) < 0.01 * len(sure)
    assert_kept_rows_match(rows, sure, edge)


def test_dapi_block_at_fov_geometry(mm):
    """The DAPI block of the 3-colour FOV (zpad 24, blur 50, delta 5, fit 5) on
    10 tiles, so the z operator runs with Zp = 98: the stitched buffer against
    the oracle's Deconvolver.apply, the RMS divisor, and both signs' maxima on
    the GPU's buffer."""
    synth = mm["synth"]
    Z, X, Y = 50, 1000, 2048
    img = synth.dapi_stack(Z, X, Y, 1099, n_nuclei=300 * X * Y // 2048 ** 2)
    psf = synth.gaussian_psf((40, 40, 40), 2.0, 1.3)
    zpad = (Z - 1) // 2
    dec = mm["dc"].Deconvolver(psf, (Z, X, Y), zpad=zpad, **DAPI)
    assert dec.n_tiles(img.shape) == 10 and dec.z_operator is not None
    dimg = img.cuda()
    plus, minus, buf, rms = mm["pl"].dapi_spots(dec, dimg, None, batch=-1, **DAPI)
    got = buf.cpu().numpy()
    o = od.Deconvolver(psf, (Z, X, Y), tile_size=500, zpad=zpad, overlap=89, beta=DAPI["beta"])
    want = o.apply(img.numpy(), None, DAPI["blur_radius"])
    assert not np.isnan(want).any()
    err = np.abs(got - want).max() / np.abs(want).max()
    print("dapi fov geometry: max |gpu - oracle| / max|oracle| = %.3g" % err)
    assert err < REL
    v = got.astype(np.float64)
    rms_ref = np.float32(np.float32(np.sqrt((v * v).sum())) / np.sqrt(v.size))
    assert abs(rms - rms_ref) <= 2e-7 * rms_ref
    normed = (got / np.float32(rms)).astype(np.float32)
    raw = img.numpy().astype(np.float32)
    want_p = ck.find_local_maxima(normed, DAPI["threshold"], 5, 5, raw, 1, 1.5)
    want_m = ck.find_local_maxima(-normed, DAPI["threshold"], 5, 5, raw, 1, 1.5)
    assert len(want_p) > 50 and len(want_m) > 10
    assert_rows_close(ck.sort_rows(plus.cpu().numpy()), ck.sort_rows(want_p))
    assert_rows_close(ck.sort_rows(minus.cpu().numpy()), ck.sort_rows(want_m))


def test_psf_grid_tiles_of_300(mm):
    """The multi-PSF workload's kernels: tiles of 300 (P 478 = 2 x 239), Z 40,
    zpad 39, a PSF per tile (sigma growing across the grid), 3 x 3 tiles: the
    direct z sum with a z kernel per tile."""
    synth = mm["synth"]
    Z, X, Y, n = 40, 900, 900, 3
    psfs = {(i, j): synth.gaussian_psf((40, 40, 40), 1.8 + 0.6 * (i + j) / (2 * n - 2),
                                       1.1 + 0.5 * (i + j) / (2 * n - 2)) for i in range(n) for j in range(n)}
    a = dict(HYB, tile_size=300)
    img = synth.hyb_stack(Z, X, Y, 5400, 1002)
    dec = mm["dc"].Deconvolver(psfs, (Z, X, Y), zpad=Z - 1, **a)
    assert dec.P == 478 and dec.psf_fft.shape[0] == 9
    dimg = img.cuda()
    rows = mm["pl"].hyb_spots(dec, dimg, None, batch=-1, **a).cpu().numpy()
    exact, folded = both_volumes(mm, dec, dimg, None, a["blur_radius"])
    boxes = dec.tile_boxes(img.shape)
    W = [od.wiener_half(p, Z, 300, Z - 1, 89, a["beta"]) for p in psfs.values()]
    err = check_tiles_against_oracle(dec, img.numpy(), None, boxes, range(9), exact, folded, W, a, Z - 1)
    print("psf grid: worst voxel error %.3g / %.3g of max" % tuple(err))
    sure, edge = oracle_rows_on_gpu_tiles(dec, boxes, folded[0], folded[1], a)
    assert len(sure) > 100 and len(edge) < 0.01 * len(sure)
    assert_kept_rows_match(rows, sure, edge)


def test_single_smfish_tile(mm):
    """One 40 x 500 x 500 tile without a flat field: x = y = 0, so the near
    side reflects in at the overlap and the far side (columns 589..677) stays
    zero."""
    synth = mm["synth"]
    Z, X, Y = 40, 500, 500
    img = synth.hyb_stack(Z, X, Y, 2000, 1000)
    psf = synth.gaussian_psf((40, 40, 40), 2.0, 1.3)
    dec = mm["dc"].Deconvolver(psf, (Z, X, Y), zpad=Z - 1, **HYB)
    dimg = img.cuda()
    rows = mm["pl"].hyb_spots(dec, dimg, None, **HYB).cpu().numpy()
    exact, folded = both_volumes(mm, dec, dimg, None, HYB["blur_radius"])
    res, raw = exact
    boxes = dec.tile_boxes(img.shape)
    assert len(boxes) == 1 and dec._extent(boxes[0]) == (589, 589)
    W = [od.wiener_half(psf, Z, 500, Z - 1, 89, HYB["beta"])]
    check_tiles_against_oracle(dec, img.numpy(), None, boxes, (0,), exact, folded, W, HYB, Z - 1)
    sure, edge = oracle_rows_on_gpu_tiles(dec, boxes, folded[0], folded[1], HYB)
    assert len(sure) > 100 and len(edge) < 0.02 * len(sure)
    assert_kept_rows_match(rows, sure, edge)
    # the plain per-tile form of the same tile (Deconvolver.tile_wise + find_local_maxima)
    from mermake_gb300 import maxima
    (_, _, tile, rawv), = list(dec.tile_wise(dimg, None, **HYB))
    np.testing.assert_array_equal(tile.cpu().numpy(), res[0, :, :589, :589])
    plain = maxima.find_local_maxima(tile, raw=rawv, **HYB).cpu().numpy()
    full = ck.find_local_maxima(np.ascontiguousarray(res[0, :, :589, :589]), HYB["threshold"], 1, 3,
                                np.ascontiguousarray(raw[0, :, :589, :589]), 1, 1.5)
    assert_rows_close(ck.sort_rows(plain), ck.sort_rows(full))
