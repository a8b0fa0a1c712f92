"""GPU parity of the per-FOV drivers: the batched hyb colour (mm_hyb_spots) and
the DAPI block (mm_dapi_spots) against the plain per-tile loop of the same
library (identical volumes, so identical maxima) and against the oracle."""
import numpy as np
import pytest
import torch

from oracle import ckernels as ck
from oracle import deconv as od
from tests.test_gpu_kernels import assert_rows_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mm():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mermake_gb300 import deconvolver, maxima, pipeline, synth
    from mermake_gb300 import _lib
    return dict(dc=deconvolver, mx=maxima, pl=pipeline, synth=synth, lib=_lib)


HYB = dict(tile_size=60, overlap=12, beta=1e-4, threshold=3600, blur_radius=10, delta=1, delta_fit=3,
           sigmaZ=1, sigmaXY=1.5)


def hyb_case(mm, seed=1, Z=12, X=170, Y=150):
    img = mm["synth"].hyb_stack(Z, X, Y, 300, seed, gain=mm["synth"].flat_gain(X, Y))
    flat = mm["synth"].flat_gain(X, Y)
    psf = mm["synth"].gaussian_psf((9, 9, 9), 2.0, 1.3)
    return img, flat, psf


def plain_loop(mm, dec, img, flat, a):
    """__main__.py:253-265 verbatim, on this library's tile_wise + find_local_maxima."""
    out = []
    ov = a["overlap"]
    for x, y, tile, raw in dec.tile_wise(img, flat, **a):
        Xh = mm["mx"].find_local_maxima(tile, raw=raw, **a)
        keep = torch.all((Xh[:, 1:3] >= ov) & (Xh[:, 1:3] < torch.tensor([tile.shape[1] - ov, tile.shape[2] - ov],
                                                                        device="cuda")), dim=-1)
        if torch.any(keep):
            Xh = Xh[keep]
            Xh[:, 1] += x - ov
            Xh[:, 2] += y - ov
            out.append(Xh)
    return torch.cat(out) if out else torch.zeros((0, 8), device="cuda")


@pytest.mark.parametrize("X,Y", [(170, 150), (130, 130)])
def test_hyb_batched_equals_plain_loop(mm, X, Y):
    """With the truncated box blur on both sides (MM_BLUR_EXACT) the batched
    driver gives the rows of the plain loop exactly.  Also at X = Y = 130,
    where the second tile has xd = 82 > P - overlap, so xd + overlap is
    clipped to the padded size P = 84 in the yielded view."""
    img, flat, psf = hyb_case(mm, X=X, Y=Y)
    Z = img.shape[0]
    dec = mm["dc"].Deconvolver(psf, img.shape, zpad=Z - 1, **HYB)
    dimg, dflat = img.cuda(), torch.from_numpy(flat).cuda()
    want = ck.sort_rows(plain_loop(mm, dec, dimg, dflat, HYB).cpu().numpy())
    with mm["lib"].blur_mode(mm["lib"].MM_BLUR_EXACT):
        for batch in (1, 4, 0):
            got = ck.sort_rows(mm["pl"].hyb_spots(dec, dimg, dflat, batch=batch, **HYB).cpu().numpy())
            assert len(want) > 20
            np.testing.assert_array_equal(got, want)


def test_folded_blur_volumes_and_rows(mm):
    """The drivers' default: the blur subtraction folded into the z step
    (1 - D(kx) D(ky) per frequency).  Its volumes (mm_deconv_tiles under
    MM_BLUR_SPECTRAL) equal the truncated blur's at every voxel at least the
    box half-width from a tile edge, within float32 rounding, and the
    driver's rows are the oracle's maxima + fit on those volumes."""
    from tests.test_gpu_configs import assert_kept_rows_match, oracle_rows_on_gpu_tiles
    img, flat, psf = hyb_case(mm, seed=4)
    Z = img.shape[0]
    dec = mm["dc"].Deconvolver(psf, img.shape, zpad=Z - 1, **HYB)
    dimg, dflat = img.cuda(), torch.from_numpy(flat).cuda()
    nt, P = dec.n_tiles(img.shape), dec.P
    vols = {}
    for mode in (mm["lib"].MM_BLUR_EXACT, mm["lib"].MM_BLUR_SPECTRAL):
        res = torch.empty((nt, Z, P, P), device="cuda")
        raw = torch.empty_like(res)
        with mm["lib"].blur_mode(mode):
            dec._call(dimg, mm["dc"].MM_DTYPE_U16, dflat, 0, nt, HYB["blur_radius"], res_out=res, raw_out=raw)
        vols[mode] = res.cpu().numpy(), raw.cpu().numpy()
    ex, sp = vols[mm["lib"].MM_BLUR_EXACT][0], vols[mm["lib"].MM_BLUR_SPECTRAL][0]
    d = HYB["blur_radius"] // 2
    inner = (slice(None), slice(None), slice(d, P - d), slice(d, P - d))
    err = np.abs(sp[inner] - ex[inner]).max() / np.abs(ex[inner]).max()
    print("folded vs truncated blur, voxels >= %d from the edges: %.3g of max" % (d, err))
    assert err < 1e-5
    rows = mm["pl"].hyb_spots(dec, dimg, dflat, **HYB).cpu().numpy()
    sure, edge = oracle_rows_on_gpu_tiles(dec, dec.tile_boxes(img.shape), sp, vols[mm["lib"].MM_BLUR_SPECTRAL][1],
                                          HYB)
    assert len(sure) > 20
    assert_kept_rows_match(rows, sure, edge)


def test_hyb_spots_match_oracle_on_same_volumes(mm):
    """The maxima set is bit-exact when both sides see the same deconvolved
    tile; the fit agrees within tolerance."""
    img, flat, psf = hyb_case(mm, seed=2)
    Z = img.shape[0]
    dec = mm["dc"].Deconvolver(psf, img.shape, zpad=Z - 1, **HYB)
    dimg, dflat = img.cuda(), torch.from_numpy(flat).cuda()
    for x, y, tile, raw in dec.tile_wise(dimg, dflat, **HYB):
        t = tile.cpu().numpy()
        r = raw.cpu().numpy()
        got = ck.sort_rows(mm["mx"].find_local_maxima(tile, raw=raw, **HYB).cpu().numpy())
        want = ck.sort_rows(ck.find_local_maxima(t, HYB["threshold"], 1, 3, r, 1, 1.5))
        assert_rows_close(got, want)


def test_hyb_end_to_end_against_oracle(mm):
    """Full oracle path (FP64 deconvolution, C maxima/fit, keep/offset): the
    maxima sets agree except at near-ties flipped by float32 FFT rounding."""
    img, flat, psf = hyb_case(mm, seed=3)
    Z = img.shape[0]
    dec = mm["dc"].Deconvolver(psf, img.shape, zpad=Z - 1, **HYB)
    got = ck.sort_rows(mm["pl"].hyb_spots(dec, img.cuda(), torch.from_numpy(flat).cuda(), **HYB).cpu().numpy())
    o = od.Deconvolver(psf, img.shape, zpad=Z - 1, **HYB)
    rows = []
    ov = HYB["overlap"]
    for x, y, res, raw in o.tile_wise(img.numpy(), flat, HYB["blur_radius"]):
        Xh = ck.find_local_maxima(res.astype(np.float32), HYB["threshold"], 1, 3, raw, 1, 1.5)
        k = np.all((Xh[:, 1:3] >= ov) & (Xh[:, 1:3] < [res.shape[1] - ov, res.shape[2] - ov]), axis=-1)
        Xh = Xh[k]
        Xh[:, 1] += x - ov
        Xh[:, 2] += y - ov
        rows.append(Xh)
    want = ck.sort_rows(np.concatenate(rows))
    gi = {tuple(np.round(r[:3], 2)) for r in got}
    wi = {tuple(np.round(r[:3], 2)) for r in want}
    assert len(want) > 20
    assert len(gi & wi) >= 0.98 * max(len(gi), len(wi))


DAPI = dict(tile_size=60, overlap=12, beta=0.01, threshold=3.0, blur_radius=20, delta=5, delta_fit=5,
            sigmaZ=1, sigmaXY=1.5)


def test_dapi_batched_equals_stepwise(mm):
    """__main__.py:215-225: apply -> RMS -> maxima(+) -> negate -> maxima(-),
    bit-identical with the truncated blur on both sides."""
    Z, X, Y = 10, 130, 140
    img = mm["synth"].dapi_stack(Z, X, Y, 5, n_nuclei=12, radii=(3.0, 12.0, 12.0))
    psf = mm["synth"].gaussian_psf((9, 9, 9), 2.0, 1.3)
    dec = mm["dc"].Deconvolver(psf, img.shape, zpad=(Z - 1) // 2, **DAPI)
    dimg = img.cuda()
    folded = mm["pl"].dapi_spots(dec, dimg, None, **DAPI)[2].cpu().numpy()
    with mm["lib"].blur_mode(mm["lib"].MM_BLUR_EXACT):
        plus, minus, buf, rms = mm["pl"].dapi_spots(dec, dimg, None, **DAPI)
    ref_buf = dec.apply(dimg, None, **DAPI)
    np.testing.assert_array_equal(buf.cpu().numpy(), ref_buf.cpu().numpy())
    # the default folds the blur into the z step: the stitched centres lie at
    # least the overlap inside their tiles, where the two blurs agree
    r = ref_buf.cpu().numpy()
    assert np.abs(folded - r).max() <= 1e-5 * np.abs(r).max()
    v = ref_buf.double()
    rms_ref = np.float32(np.float32(np.sqrt(float((v * v).sum()))) / np.sqrt(v.numel()))
    assert abs(rms - rms_ref) <= 2e-7 * rms_ref
    normed = (ref_buf / torch.tensor(rms, dtype=torch.float32, device="cuda"))
    p2 = mm["mx"].find_local_maxima(normed, raw=dimg, **DAPI)
    m2 = mm["mx"].find_local_maxima(-normed, raw=dimg, **DAPI)
    np.testing.assert_array_equal(ck.sort_rows(plus.cpu().numpy()), ck.sort_rows(p2.cpu().numpy()))
    np.testing.assert_array_equal(ck.sort_rows(minus.cpu().numpy()), ck.sort_rows(m2.cpu().numpy()))
    assert len(plus) > 0 and len(minus) > 0


def test_fov_runner_matches_direct_calls(mm):
    """FovRunner (pinned host channels, copies of FOV k+1 overlapping FOV k)
    gives the rows of the direct dapi_spots / hyb_spots calls, FOV after FOV,
    with both device slots reused."""
    Z, X, Y = 12, 170, 150
    dapi = mm["synth"].dapi_stack(Z, X, Y, 5, n_nuclei=12, radii=(3.0, 12.0, 12.0))
    cols, flats = [], []
    for seed in (1, 2):
        img, flat, psf = hyb_case(mm, seed=seed, Z=Z, X=X, Y=Y)
        cols.append(img.cpu().pin_memory())
        flats.append(torch.from_numpy(flat).cuda())
    dh = mm["dc"].Deconvolver(psf, (Z, X, Y), zpad=Z - 1, **HYB)
    dd = mm["dc"].Deconvolver(psf, (Z, X, Y), zpad=(Z - 1) // 2, **DAPI)
    hd = dapi.cpu().pin_memory()
    want_p, want_m, _, _ = mm["pl"].dapi_spots(dd, dapi.cuda(), None, **DAPI)
    want_rows = [mm["pl"].hyb_spots(dh, c.cuda(), f, **HYB) for c, f in zip(cols, flats)]
    runner = mm["pl"].FovRunner(dh, dd, HYB, DAPI)
    ticket = runner.submit(hd, cols)
    for _ in range(3):
        nxt = runner.submit(hd, cols)
        p, m, rows = runner.run(ticket, flats)
        ticket = nxt
        np.testing.assert_array_equal(ck.sort_rows(p), ck.sort_rows(want_p.cpu().numpy()))
        np.testing.assert_array_equal(ck.sort_rows(m), ck.sort_rows(want_m.cpu().numpy()))
        for got, want in zip(rows, want_rows):
            np.testing.assert_array_equal(ck.sort_rows(got), ck.sort_rows(want.cpu().numpy()))
    assert runner.h2d_bytes == 3 * Z * X * Y * 2


@pytest.mark.parametrize("small_rows", [False, True])
def test_fov_runner_launch_before_collect(mm, monkeypatch, small_rows):
    """FovRunner pipelined: FOV k is launched before FOV k - 1 is collected
    and FOV k + 1 submitted after it, the order the bench's e2e loop uses.
    Two different FOVs alternate over the two slots, so rows or images taken
    from the wrong slot would show; with row buffers of 8 every output is
    rerun by the synchronous driver while the next FOV is already queued."""
    Z, X, Y = 12, 170, 150
    fovs, want = [], []
    imgs = [hyb_case(mm, seed=s, Z=Z, X=X, Y=Y) for s in (4, 5)]
    psf = imgs[0][2]
    dh = mm["dc"].Deconvolver(psf, (Z, X, Y), zpad=Z - 1, **HYB)
    dd = mm["dc"].Deconvolver(psf, (Z, X, Y), zpad=(Z - 1) // 2, **DAPI)
    flats = [torch.from_numpy(f).cuda() for _, f, _ in imgs]
    for k in range(2):
        dapi = mm["synth"].dapi_stack(Z, X, Y, 6 + k, n_nuclei=10 + 3 * k, radii=(3.0, 12.0, 12.0))
        cols = [imgs[k][0], imgs[1 - k][0]]
        fl = [flats[k], flats[1 - k]]
        p, m, _, _ = mm["pl"].dapi_spots(dd, dapi.cuda(), None, **DAPI)
        rows = [mm["pl"].hyb_spots(dh, c.cuda(), f, **HYB) for c, f in zip(cols, fl)]
        want.append((p.cpu().numpy(), m.cpu().numpy(), [r.cpu().numpy() for r in rows]))
        fovs.append((dapi.cpu().pin_memory(), [c.cpu().pin_memory() for c in cols], fl))
    if small_rows:
        assert min(len(w[0]) for w in want) > 8 and min(len(r) for w in want for r in w[2]) > 8
        monkeypatch.setattr(mm["pl"], "_capacity", lambda dec, key, default: 8)
    runner = mm["pl"].FovRunner(dh, dd, HYB, DAPI)
    seq = [0, 1, 0, 1, 1, 0]
    nxt, pending, got = runner.submit(fovs[seq[0]][0], fovs[seq[0]][1]), None, []
    for k, f in enumerate(seq):
        h = (runner.launch(nxt, fovs[f][2]), f)
        if pending is not None:
            got.append((runner.collect(pending[0]), pending[1]))
        pending = h
        if k + 1 < len(seq):
            nxt = runner.submit(fovs[seq[k + 1]][0], fovs[seq[k + 1]][1])
    got.append((runner.collect(pending[0]), pending[1]))
    assert [f for _, f in got] == seq
    for (p, m, rows), f in got:
        wp, wm, wr = want[f]
        np.testing.assert_array_equal(ck.sort_rows(p), ck.sort_rows(wp))
        np.testing.assert_array_equal(ck.sort_rows(m), ck.sort_rows(wm))
        for g, w in zip(rows, wr):
            np.testing.assert_array_equal(ck.sort_rows(g), ck.sort_rows(w))


def test_fov_runner_reruns_outputs_that_overflow(mm, monkeypatch):
    """FovRunner enqueues a FOV with the asynchronous drivers and reads all
    counts once; an output whose rows did not fit (here every output, with
    row buffers of 8) is run again by the synchronous driver, and the rows
    are those of the direct calls."""
    Z, X, Y = 12, 170, 150
    dapi = mm["synth"].dapi_stack(Z, X, Y, 5, n_nuclei=12, radii=(3.0, 12.0, 12.0))
    img, flat, psf = hyb_case(mm, seed=3, Z=Z, X=X, Y=Y)
    flat_d = torch.from_numpy(flat).cuda()
    dh = mm["dc"].Deconvolver(psf, (Z, X, Y), zpad=Z - 1, **HYB)
    dd = mm["dc"].Deconvolver(psf, (Z, X, Y), zpad=(Z - 1) // 2, **DAPI)
    want_p, want_m, _, _ = mm["pl"].dapi_spots(dd, dapi.cuda(), None, **DAPI)
    want = mm["pl"].hyb_spots(dh, img.cuda(), flat_d, **HYB)
    assert len(want) > 8 and len(want_p) > 8
    monkeypatch.setattr(mm["pl"], "_capacity", lambda dec, key, default: 8)
    runner = mm["pl"].FovRunner(dh, dd, HYB, DAPI)
    p, m, rows = runner.run(runner.submit(dapi.cpu().pin_memory(), [img.cpu().pin_memory()]), [flat_d])
    np.testing.assert_array_equal(ck.sort_rows(p), ck.sort_rows(want_p.cpu().numpy()))
    np.testing.assert_array_equal(ck.sort_rows(m), ck.sort_rows(want_m.cpu().numpy()))
    np.testing.assert_array_equal(ck.sort_rows(rows[0]), ck.sort_rows(want.cpu().numpy()))


def test_autotune_picks_batch_and_z_form(mm):
    """tune.autotune times every candidate batch size with every z form the
    geometry qualifies for (25 tiles of one PSF, Z = 10: the matrix in
    registers, the matrix in shared memory, the direct sum, the transforms over
    the padded depth), keeps the fastest pair for the geometry, and
    hyb_spots(batch=0) then runs it: its rows are those of the same pair set
    explicitly, and every form's rows agree with the others' within float32
    rounding of the voxels (the same spots but for near-ties)."""
    from mermake_gb300 import _lib, tune
    Z, X, Y = 10, 300, 300
    img = mm["synth"].hyb_stack(Z, X, Y, 600, 9, gain=mm["synth"].flat_gain(X, Y))
    flat = mm["synth"].flat_gain(X, Y)
    psf = mm["synth"].gaussian_psf((9, 9, 9), 2.0, 1.3)
    dec = mm["dc"].Deconvolver(psf, img.shape, zpad=Z - 1, **HYB)
    dimg, dflat = img.cuda(), torch.from_numpy(flat).cuda()
    assert dec.n_tiles(img.shape) == 25
    forms = tune.zforms(dec)
    assert forms == [_lib.MM_ZFORM_REGISTERS, _lib.MM_ZFORM_TENSOR, _lib.MM_ZFORM_SHARED, _lib.MM_ZFORM_DIRECT,
                     _lib.MM_ZFORM_TRANSFORMS]
    times = tune.autotune(dec, dimg, dflat, HYB, candidates=(4, -1), reps=1)
    assert set(times) == {(b, f) for b in (4, -1) for f in forms} and all(t > 0 for t in times.values())
    best = min(times, key=times.get)
    assert tune.settings_for(dec, img.shape) == best
    got = ck.sort_rows(mm["pl"].hyb_spots(dec, dimg, dflat, **HYB).cpu().numpy())
    with _lib.zform(best[1]):
        want = ck.sort_rows(mm["pl"].hyb_spots(dec, dimg, dflat, batch=best[0], tuned=False, **HYB).cpu().numpy())
    np.testing.assert_array_equal(got, want)
    ref = {tuple(np.round(r[:3], 2)) for r in want}
    for f in forms:
        with _lib.zform(f):
            rows = mm["pl"].hyb_spots(dec, dimg, dflat, batch=-1, tuned=False, **HYB).cpu().numpy()
        keys = {tuple(np.round(r[:3], 2)) for r in rows}
        assert len(ref) > 50 and len(keys & ref) >= 0.99 * max(len(keys), len(ref)), f


def test_fov_graph_replays_match_direct_calls(mm):
    """FovGraph (the DAPI block and every colour captured once as a CUDA graph)
    gives the rows of the direct dapi_spots / hyb_spots calls, for two FOVs of
    different content replayed through the same graph, without falling back."""
    Z, X, Y = 12, 170, 150
    fovs = []
    for k in range(2):
        dapi = mm["synth"].dapi_stack(Z, X, Y, 5 + k, n_nuclei=12, radii=(3.0, 12.0, 12.0))
        cols, flats = [], []
        for seed in (1 + 10 * k, 2 + 10 * k):
            img, flat, psf = hyb_case(mm, seed=seed, Z=Z, X=X, Y=Y)
            cols.append(img)
            flats.append(torch.from_numpy(flat).cuda())
        fovs.append((dapi, cols, flats))
    dh = mm["dc"].Deconvolver(psf, (Z, X, Y), zpad=Z - 1, **HYB)
    dd = mm["dc"].Deconvolver(psf, (Z, X, Y), zpad=(Z - 1) // 2, **DAPI)
    flats = fovs[0][2]  # flat fields are fixed per graph
    with mm["pl"].FovGraph(dh, dd, (Z, X, Y), 2, HYB, DAPI, flats=flats) as g:
        for dapi, cols, _ in fovs:
            want_p, want_m, _, _ = mm["pl"].dapi_spots(dd, dapi.cuda(), None, **DAPI)
            want = [mm["pl"].hyb_spots(dh, c.cuda(), f, **HYB) for c, f in zip(cols, flats)]
            p, m, rows = g.run(dapi, cols)
            np.testing.assert_array_equal(ck.sort_rows(p), ck.sort_rows(want_p.cpu().numpy()))
            np.testing.assert_array_equal(ck.sort_rows(m), ck.sort_rows(want_m.cpu().numpy()))
            for got, w in zip(rows, want):
                np.testing.assert_array_equal(ck.sort_rows(got), ck.sort_rows(w.cpu().numpy()))
        assert g.fallbacks == 0


def test_fov_graph_grows_and_recaptures_after_an_overflow(mm):
    """A graph captured with row buffers too small for the FOV (8 rows) falls
    back to the synchronous drivers once, grows its buffers to that FOV's
    counts, captures again, and replays the next FOV without falling back; the
    rows equal the direct calls' both times."""
    Z, X, Y = 12, 170, 150
    dapi = mm["synth"].dapi_stack(Z, X, Y, 5, n_nuclei=12, radii=(3.0, 12.0, 12.0))
    img, flat, psf = hyb_case(mm, seed=1, Z=Z, X=X, Y=Y)
    flats = [torch.from_numpy(flat).cuda()]
    dh = mm["dc"].Deconvolver(psf, (Z, X, Y), zpad=Z - 1, **HYB)
    dd = mm["dc"].Deconvolver(psf, (Z, X, Y), zpad=(Z - 1) // 2, **DAPI)
    want_p, want_m, _, _ = mm["pl"].dapi_spots(dd, dapi.cuda(), None, **DAPI)
    want = mm["pl"].hyb_spots(dh, img.cuda(), flats[0], **HYB).cpu().numpy()
    real = mm["pl"]._capacity
    mm["pl"]._capacity = lambda dec, key, default: 8
    try:
        g = mm["pl"].FovGraph(dh, dd, (Z, X, Y), 1, HYB, DAPI, flats=flats)
    finally:
        mm["pl"]._capacity = real
    with g:
        assert g.cap == 8
        for k in range(2):
            p, m, rows = g.run(dapi, [img])
            np.testing.assert_array_equal(ck.sort_rows(p), ck.sort_rows(want_p.cpu().numpy()))
            np.testing.assert_array_equal(ck.sort_rows(m), ck.sort_rows(want_m.cpu().numpy()))
            np.testing.assert_array_equal(ck.sort_rows(rows[0]), ck.sort_rows(want))
            assert (g.fallbacks, g.recaptures) == (1, 1)
        assert g.cap >= len(want)
