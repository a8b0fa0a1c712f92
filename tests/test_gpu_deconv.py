"""GPU parity of the Wiener spectrum and the tiled deconvolution against the
FP64 oracle and the reference's golden float16 slices."""
import os

import numpy as np
import pytest
import torch

from oracle import deconv as od
from tests.test_oracle import f16_tolerance, load_tile

pytestmark = pytest.mark.gpu

# voxels: |gpu - oracle| <= REL * max|oracle| (float32 FFTs against float64)
REL = 1e-4


@pytest.fixture(scope="module")
def dc():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mermake_gb300 import deconvolver
    return deconvolver


def u16(a):
    return torch.from_numpy(np.asarray(a).astype(np.int32)).to(torch.uint16).cuda()


def test_wiener_spectrum_matches_oracle(dc, golden_dir):
    psf = np.load(os.path.join(golden_dir, "psf_750.npz"))["psf"]
    Z, ts, zpad, ov, beta = 35, 300, 35, 89, 1e-3
    d = dc.Deconvolver(psf, (Z, 1200, 1200), tile_size=ts, zpad=zpad, overlap=ov, beta=beta)
    got = d.psf_fft[0].cpu().numpy().astype(np.complex128) * (d.Zp * d.P * d.P)
    want = od.wiener_half(psf, Z, ts, zpad, ov, beta)
    err = np.abs(got - want).max() / np.abs(want).max()
    assert err < 1e-5, err


@pytest.mark.parametrize("zop", [True, False])
@pytest.mark.parametrize("k", [0, 1, 2])
def test_deconv_tiles_match_golden_and_oracle(dc, golden_dir, k, zop):
    """test_deconvolver.py:422-434 on the stored tiles: Deconvolver.apply of the
    tile's input crop, against the reference's float16 goldens and the FP64 oracle."""
    t = load_tile(golden_dir, k)
    psf = np.load(os.path.join(golden_dir, "psf_750.npz"))["psf"]
    Z, ts, ov = t["Z"], t["ts"], t["ov"]
    x, y, x0, x1, y0, y1 = t["box"]
    img = u16(t["img"])
    d = dc.Deconvolver(psf, img.shape, tile_size=ts, zpad=Z, overlap=ov, beta=1e-3, z_operator=zop)
    assert (d.z_operator is not None) == zop
    tiles = d.tile_boxes(img.shape)
    ti = tiles.index(tuple(t["box"]))
    # the whole tile grid in one batch: the z operator runs on batches of >= 10
    # tiles (16 here for tile 300; tile 500 has 9 and keeps the transforms)
    res = torch.empty((len(tiles), Z, d.P, d.P), device="cuda")
    d._call(img, dc.MM_DTYPE_U16, None, 0, len(tiles), None, res_out=res)
    xend, yend = d._extent(t["box"])
    got = res[ti, :, :xend, :yend].cpu().numpy().astype(np.float64)
    W = od.wiener_half(psf, Z, ts, Z, ov, 1e-3)
    want, _ = od.deconv_tile(t["img"], None, t["box"], W, ts, Z, ov)
    err = np.abs(got - want).max() / np.abs(want).max()
    print("tile", k, "max |gpu - oracle| / max|oracle| =", err)
    assert err < REL
    cen = got[:, ov:-ov, ov:-ov][:: t["zs"]]
    gold = t["gold"]
    cen = cen[:, : gold.shape[1], : gold.shape[2]]
    diff = np.abs(cen - gold.astype(np.float64))
    # float16 goldens: one f16 spacing + 1e-5 of the range, as for the oracle
    assert np.mean(diff <= f16_tolerance(gold)) > 0.999
    assert diff.max() <= 2 * f16_tolerance(gold).max()


def small_case(seed=0, Z=10, X=50, Y=50, flat=True):
    rng = np.random.default_rng(seed)
    img = rng.integers(100, 5000, (Z, X, Y)).astype(np.uint16)
    psf = np.zeros((5, 5, 5), np.float32)
    psf[2, 2, 2] = 1.0
    psf[1:4, 1:4, 1:4] += 0.1 * rng.random((3, 3, 3)).astype(np.float32)
    fl = (0.8 + 0.2 * rng.random((X, Y))).astype(np.float32) if flat else None
    return img, psf, fl


@pytest.mark.parametrize("zop", [True, False])
@pytest.mark.parametrize("ts,zpad,ov,blur", [(30, 5, 5, None), (30, 5, 5, 8), (20, 3, 7, 5), (64, 9, 11, 30),
                                             (17, 4, 3, None), (15, 4, 3, 4)])
def test_tile_wise_matches_oracle(dc, ts, zpad, ov, blur, zop):
    """Every yielded tile and raw view of tile_wise (deconvolver.py:98-170)
    with a flat field and optional blur subtraction, with the z operator and
    with the padded-depth transforms (P = 21: an odd plane of 21 x 11)."""
    img, psf, fl = small_case(ts + zpad)
    d = dc.Deconvolver(psf, img.shape, tile_size=ts, zpad=zpad, overlap=ov, beta=0.01, z_operator=zop)
    o = od.Deconvolver(psf, img.shape, tile_size=ts, zpad=zpad, overlap=ov, beta=0.01)
    n = 0
    for (x, y, res, raw), (xo, yo, rres, rraw) in zip(d.tile_wise(u16(img), torch.from_numpy(fl).cuda(), blur),
                                                      o.tile_wise(img, fl, blur)):
        assert (x, y) == (xo, yo)
        assert tuple(res.shape) == rres.shape == rraw.shape
        g = res.cpu().numpy().astype(np.float64)
        assert np.abs(g - rres).max() <= REL * np.abs(rres).max()
        np.testing.assert_array_equal(raw.cpu().numpy(), rraw)
        n += 1
    assert n == len(od.tiles(img.shape, ts, ov))


def test_apply_float_image_and_multi_psf(dc):
    """float64 images (test_deconvolver.py uses cp.random.random) and a dict of
    PSFs paired with tiles in order, truncated by zip (deconvolver.py:110-116)."""
    rng = np.random.default_rng(4)
    img = rng.random((10, 50, 50))
    psf = np.zeros((5, 5, 5))
    psf[2, 2, 2] = 1.0
    psfs = {"a": psf, "b": psf * 0.9 + 0.01, "c": np.roll(psf, 1, axis=2)}
    for p in (psf, psfs):
        d = dc.Deconvolver(p, img.shape, tile_size=20, zpad=10, overlap=5, beta=0.001)
        o = od.Deconvolver(p, img.shape, tile_size=20, zpad=10, overlap=5, beta=0.001)
        got = d.apply(torch.from_numpy(img).cuda()).cpu().numpy()
        want = o.apply(img.astype(np.float32))
        ok = ~np.isnan(want)
        assert np.abs(got[ok] - want[ok]).max() <= REL * np.abs(want[ok]).max()


@pytest.mark.parametrize("ts", [500, 300])
def test_tile_wise_float_image_at_the_specialised_lengths(dc, ts):
    """float32 images through the FFT engine compiled for the benchmark tile
    lengths (P = 678 at tile 500, 478 at tile 300), with a flat field and blur,
    against the FP64 oracle: every yielded tile of a 2 x 2 grid (one thin edge)."""
    rng = np.random.default_rng(ts)
    Z, X = 4, ts + 100
    img = (1000 * rng.random((Z, X, X))).astype(np.float32)
    fl = (0.8 + 0.2 * rng.random((X, X))).astype(np.float32)
    psf = np.zeros((5, 5, 5), np.float32)
    psf[2, 2, 2] = 1.0
    psf[1:4, 1:4, 1:4] += 0.1 * rng.random((3, 3, 3)).astype(np.float32)
    args = dict(tile_size=ts, zpad=3, overlap=89, beta=0.01)
    d = dc.Deconvolver(psf, img.shape, **args)
    o = od.Deconvolver(psf, img.shape, **args)
    assert d.P == ts + 178
    n = 0
    for (x, y, res, raw), (xo, yo, rres, rraw) in zip(d.tile_wise(torch.from_numpy(img).cuda(),
                                                                   torch.from_numpy(fl).cuda(), 15),
                                                      o.tile_wise(img, fl, 15)):
        assert (x, y) == (xo, yo)
        g = res.cpu().numpy().astype(np.float64)
        assert np.abs(g - rres).max() <= REL * np.abs(rres).max()
        n += 1
    assert n == 4


def test_full_deconv_signature(dc):
    """test_deconvolver.py:436-470: shapes and intensity."""
    img = torch.zeros((10, 50, 50), dtype=torch.float64, device="cuda")
    img[5, 25, 25] = 100
    psf = np.zeros((5, 5, 5))
    psf[2, 2, 2] = 1.0
    out = dc.full_deconv(img, psf, tile_size=30, overlap=5)
    assert tuple(out.shape) == (10, 50, 50)
    assert torch.isfinite(out).all()
    assert abs(float(out.sum()) - 100) / 100 < 0.5


def test_zpad_zero_is_rejected(dc):
    img, psf, _ = small_case(flat=False)
    with pytest.raises(ValueError, match="zpad"):
        d = dc.Deconvolver(psf, img.shape, tile_size=30, zpad=0, overlap=5)
        list(d.tile_wise(u16(img)))


@pytest.mark.parametrize("npsf", [1, 2, 4, 9])
def test_apply_stitch_order_matches_reference(dc, npsf):
    """Deconvolver.apply writes tile centres in order and the truncated
    second-to-last tile reaches into the last tile's span, which the later
    tile overwrites (deconvolver.py:179-183).  Batched stitching must keep the
    surviving values, also when zip() drops tiles (npsf < tiles)."""
    rng = np.random.default_rng(8)
    img = rng.integers(100, 4000, (10, 130, 140)).astype(np.uint16)
    base = np.zeros((5, 5, 5), np.float32)
    base[2, 2, 2] = 1.0
    psfs = base if npsf == 1 else {i: np.roll(base, i % 3 - 1, axis=2) + 0.01 * i for i in range(npsf)}
    args = dict(tile_size=60, zpad=4, overlap=12, beta=0.01)
    d = dc.Deconvolver(psfs, img.shape, **args)
    o = od.Deconvolver(psfs, img.shape, **args)
    want = o.apply(img, None, 20)
    got_all = d.apply(u16(img), None, 20).cpu().numpy()
    got_one = d.apply(u16(img), None, 20, batch=1).cpu().numpy()
    ok = ~np.isnan(want)
    np.testing.assert_array_equal(got_all[ok], got_one[ok])
    assert np.abs(got_all[ok] - want[ok]).max() <= REL * np.abs(want[ok]).max()


@pytest.mark.parametrize("Z,zpad,ts,ov", [(13, 12, 10, 3), (64, 63, 10, 3), (50, 24, 30, 9), (7, 2, 15, 3),
                                          (5, 9, 10, 3), (50, 49, 10, 3), (30, 14, 12, 4), (80, 79, 10, 3),
                                          (60, 29, 10, 3), (100, 99, 8, 2), (50, 49, 11, 4)])
def test_z_operator_matches_padded_transforms(dc, Z, zpad, ts, ov):
    """The z operator (one Z x Z matrix per frequency, from the z kernel)
    against the FFT z pass over the padded depth, on whole batches: Z not a
    multiple of the 10-plane chunks, a batch of 25 tiles split into two tile
    chunks at Z = 64, an odd frequency plane (P = 21), and zpad > Z (four
    padded planes copy one real plane) take the form with the matrix in shared
    memory; Z a multiple of 5 with 1 <= zpad <= Z - 1 (the depths of both
    benchmark blocks, zpad = Z - 1 and (Z - 1) / 2) the form with the matrix
    in registers and TMA-staged operands (csrc/zop_tma.cu), whose 25 tiles
    are split into two chunks of 13 at Z = 80 and 100 (the second chunk's box
    reaching back one tile into the first; at Z = 60 the shared-memory form
    takes the batch instead), also on a plane of 190 frequencies (P = 19: the
    last group of four half outside the plane)."""
    rng = np.random.default_rng(Z)
    X = Y = 5 * ts
    img = rng.integers(100, 5000, (Z, X, Y)).astype(np.uint16)
    psf = np.zeros((5, 5, 5), np.float32)
    psf[2, 2, 2] = 1.0
    psf[1:4, 1:4, 1:4] += 0.1 * rng.random((3, 3, 3)).astype(np.float32)
    args = dict(tile_size=ts, zpad=zpad, overlap=ov, beta=0.01)
    a = dc.Deconvolver(psf, img.shape, z_operator=True, **args)
    b = dc.Deconvolver(psf, img.shape, z_operator=False, **args)
    nt = len(a.tile_boxes(img.shape))
    assert nt == 25
    ra = torch.empty((nt, Z, a.P, a.P), device="cuda")
    rb = torch.empty_like(ra)
    a._call(u16(img), dc.MM_DTYPE_U16, None, 0, nt, 6, res_out=ra)
    b._call(u16(img), dc.MM_DTYPE_U16, None, 0, nt, 6, res_out=rb)
    err = float((ra - rb).abs().max() / rb.abs().max())
    assert err < 2e-5, err


@pytest.mark.parametrize("Z,zpad,ts,ov,npsf,nx", [(13, 12, 10, 3, 1, 2), (40, 39, 12, 4, 4, 2), (7, 2, 15, 3, 9, 3),
                                                  (5, 9, 10, 3, 6, 3), (80, 79, 8, 3, 1, 3), (128, 1, 8, 2, 4, 2),
                                                  (50, 24, 30, 9, 25, 5)])
def test_z_convolution_matches_padded_transforms(dc, Z, zpad, ts, ov, npsf, nx):
    """The direct z convolution (each tile's own z kernel, summed over the
    padded planes; MM_ZFORM_DIRECT) against the FFT z pass over the padded
    depth: one PSF in batches below the matrix form's 10 tiles, a PSF per
    tile, Z = 80 and 128 (past the matrix form's 64), zpad > Z, and 25 tiles
    of 25 PSFs."""
    from mermake_gb300 import _lib
    rng = np.random.default_rng(Z + npsf)
    X = Y = nx * ts
    img = rng.integers(100, 5000, (Z, X, Y)).astype(np.uint16)
    psfs = {}
    for k in range(npsf):
        p = np.zeros((5, 5, 5), np.float32)
        p[2, 2, 2] = 1.0
        p[1:4, 1:4, 1:4] += 0.1 * rng.random((3, 3, 3)).astype(np.float32)
        psfs[k] = p
    psf = psfs if npsf > 1 else psfs[0]
    args = dict(tile_size=ts, zpad=zpad, overlap=ov, beta=0.01)
    a = dc.Deconvolver(psf, img.shape, z_operator=True, **args)
    b = dc.Deconvolver(psf, img.shape, z_operator=False, **args)
    assert a.z_operator.shape == a.psf_fft.shape
    nt = a.n_tiles(img.shape)
    assert npsf > 1 or nt < 10
    ra = torch.empty((nt, Z, a.P, a.P), device="cuda")
    rb = torch.empty_like(ra)
    with _lib.zform(_lib.MM_ZFORM_DIRECT):
        a._call(u16(img), dc.MM_DTYPE_U16, None, 0, nt, 6, res_out=ra)
    b._call(u16(img), dc.MM_DTYPE_U16, None, 0, nt, 6, res_out=rb)
    err = float((ra - rb).abs().max() / rb.abs().max())
    assert err < 2e-5, err


@pytest.mark.parametrize("Z,zpad,ts,ov,npsf,nx,batch", [(40, 39, 12, 4, 4, 2, 6), (40, 39, 10, 3, 9, 3, 6),
                                                        (50, 24, 30, 9, 25, 5, 25), (5, 1, 10, 3, 6, 3, 4),
                                                        (45, 10, 12, 4, 4, 2, 4), (80, 79, 8, 3, 1, 3, 9),
                                                        (60, 29, 11, 4, 16, 4, 16), (10, 9, 21, 5, 1, 2, 3),
                                                        (50, 49, 10, 3, 4, 2, 4), (20, 19, 10, 3, 9, 3, 9)])
def test_per_tile_register_z_operator_matches_padded_transforms(dc, Z, zpad, ts, ov, npsf, nx, batch):
    """The z operator with each tile's matrix formed in registers from its own
    z kernel (csrc/zop_pt.cu; the register form of a batch of several PSFs,
    or of one PSF in batches below the shared-spectrum forms' 10 tiles)
    against the FFT z pass over the padded depth: items of 16 frequencies
    (Z <= 55) and of 8 (Z = 60, 80), chunks of several tiles (Z = 5, 10, 20)
    with a last chunk of fewer, batches that start past tile 0 (the kernel
    index t0 + t), zpad 1 to Z - 1 (the column classes at compile time for
    zpad = Z - 1), and planes whose last group of frequencies lies partly
    outside them (P = 19, 20, 31)."""
    from mermake_gb300 import _lib
    rng = np.random.default_rng(200 + Z + npsf)
    X = Y = nx * ts
    img = rng.integers(100, 5000, (Z, X, Y)).astype(np.uint16)
    psfs = {}
    for k in range(npsf):
        p = np.zeros((5, 5, 5), np.float32)
        p[2, 2, 2] = 1.0
        p[1:4, 1:4, 1:4] += 0.1 * rng.random((3, 3, 3)).astype(np.float32)
        psfs[k] = p
    psf = psfs if npsf > 1 else psfs[0]
    args = dict(tile_size=ts, zpad=zpad, overlap=ov, beta=0.01)
    a = dc.Deconvolver(psf, img.shape, z_operator=True, **args)
    b = dc.Deconvolver(psf, img.shape, z_operator=False, **args)
    nt = a.n_tiles(img.shape)
    assert nt == (nx * nx if npsf == 1 else min(nx * nx, npsf))  # zip() drops the tiles past the PSFs
    ra = torch.full((nt, Z, a.P, a.P), float("nan"), device="cuda")
    rb = torch.empty_like(ra)
    with _lib.zform(_lib.MM_ZFORM_REGISTERS if npsf > 1 else _lib.MM_ZFORM_AUTO):
        for t0 in range(0, nt, batch):
            n = min(batch, nt - t0)
            a._call(u16(img), dc.MM_DTYPE_U16, None, t0, n, 6, res_out=ra[t0:t0 + n])
    b._call(u16(img), dc.MM_DTYPE_U16, None, 0, nt, 6, res_out=rb)
    torch.cuda.synchronize()
    assert bool(torch.isfinite(ra).all())
    err = float((ra - rb).abs().max() / rb.abs().max())
    assert err < 2e-5, err


@pytest.mark.parametrize("Z,zpad,ts,ov,nx", [(13, 12, 10, 3, 2), (50, 49, 10, 3, 5), (50, 24, 30, 9, 5),
                                             (30, 29, 12, 4, 5), (56, 55, 8, 2, 4), (2, 1, 10, 3, 3),
                                             (40, 7, 12, 4, 3)])
def test_tensor_z_operator_matches_padded_transforms(dc, Z, zpad, ts, ov, nx):
    """The z operator on the tensor cores (csrc/zop_mma.cu: tcgen05 MMAs of
    the real form of each frequency's matrix, TF32 operands split into two
    parts) against the FFT z pass over the padded depth: the benchmark
    depths (Z = 50 with zpad 49 and 24, 25 tiles in one 32-wide MMA), the
    largest depth the form takes (Z = 56, 16 tiles in a 16-wide MMA), a
    single plane pair (Z = 2) and reflections that do not overlap (zpad 7 of
    40)."""
    from mermake_gb300 import _lib
    rng = np.random.default_rng(100 + Z)
    X = Y = nx * ts
    img = rng.integers(100, 5000, (Z, X, Y)).astype(np.uint16)
    psf = np.zeros((5, 5, 5), np.float32)
    psf[2, 2, 2] = 1.0
    psf[1:4, 1:4, 1:4] += 0.1 * rng.random((3, 3, 3)).astype(np.float32)
    args = dict(tile_size=ts, zpad=zpad, overlap=ov, beta=0.01)
    a = dc.Deconvolver(psf, img.shape, z_operator=True, **args)
    b = dc.Deconvolver(psf, img.shape, z_operator=False, **args)
    nt = a.n_tiles(img.shape)
    assert nt == nx * nx
    ra = torch.full((nt, Z, a.P, a.P), float("nan"), device="cuda")
    rb = torch.empty_like(ra)
    with _lib.zform(_lib.MM_ZFORM_TENSOR):
        a._call(u16(img), dc.MM_DTYPE_U16, None, 0, nt, 6, res_out=ra)
    b._call(u16(img), dc.MM_DTYPE_U16, None, 0, nt, 6, res_out=rb)
    torch.cuda.synchronize()
    assert bool(torch.isfinite(ra).all())
    err = float((ra - rb).abs().max() / rb.abs().max())
    assert err < 2e-5, err
