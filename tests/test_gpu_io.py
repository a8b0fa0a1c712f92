"""GPU median / load_flats (io.py:42-54) and the background subtraction flow
(__main__.py:232-250: shifted slices from the DAPI maxima, reflecting uint16
subtraction on strided views)."""
import os
import types

import numpy as np
import pytest
import torch

from oracle import align as oalign
from oracle import ckernels as ck

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mm():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mermake_gb300 import align, io
    from mermake_gb300 import math as mmath
    return dict(io=io, align=align, math=mmath)


@pytest.mark.parametrize("n", [1, 2, 3, 1000, 1001, 4096 * 4096 + 3])
def test_median_matches_numpy(mm, n):
    rng = np.random.default_rng(n)
    x = (rng.standard_normal(n) * 10).astype(np.float32)
    if n > 10:
        x[::7] = x[3]  # duplicates
    got = mm["io"].median(torch.from_numpy(x).cuda())
    s = np.sort(x)
    want = s[n // 2] if n % 2 else np.float32((s[n // 2 - 1] + s[n // 2]) / np.float32(2))
    assert got == want


def test_flat_field_matches_reference_recipe(mm):
    """crop -> blur.box(size=(20, 20)) -> / median (io.py:46-53)."""
    rng = np.random.default_rng(3)
    im = (1000 + 200 * rng.random((300, 320))).astype(np.float32)
    got = mm["io"].flat_from_image(im, shape=(2, 3, 250, 260)).cpu().numpy()
    c = mm["io"].center_crop(im, (250, 260))
    b = ck.box_1d(ck.box_1d(c, 20, axis=0), 20, axis=1)
    s = np.sort(b.ravel())
    med = np.float32((s[len(s) // 2 - 1] + s[len(s) // 2]) / np.float32(2))
    np.testing.assert_allclose(got, b / med, rtol=1e-5)


def test_background_subtraction_flow(mm, golden_dir):
    """Aligner(background Xh_plus).get_shifted_slices(Xh_plus[:, :3], shape) then
    subtract_reflect(chan[sig], back[bk], out=chan[sig])."""
    d = np.load(os.path.join(golden_dir, "dapi_features.npz"))
    Xb = d["Xh_plus"]
    shift = np.array([1.2, 6.6, -4.3], np.float32)
    Xs = Xb.copy()
    Xs[:, :3] += shift
    shape = (35, 260, 270)
    g = mm["align"].Aligner(torch.from_numpy(Xb).cuda())
    o = oalign.Aligner(Xb)
    bk, sig = g.get_shifted_slices(torch.from_numpy(Xs[:, :3].copy()).cuda(), shape)
    assert (bk, sig) == o.get_shifted_slices(Xs[:, :3].copy(), shape)
    rng = np.random.default_rng(5)
    chan = rng.integers(0, 60000, shape).astype(np.uint16)
    back = rng.integers(0, 60000, shape).astype(np.uint16)
    tc = torch.from_numpy(chan.astype(np.int32)).to(torch.uint16).cuda()
    tb = torch.from_numpy(back.astype(np.int32)).to(torch.uint16).cuda()
    mm["math"].subtract_reflect(tc[sig], tb[bk], out=tc[sig])
    want = chan.astype(np.int64)
    want[sig] = np.abs(chan[sig].astype(np.int64) - back[bk].astype(np.int64))
    np.testing.assert_array_equal(tc.to(torch.int32).cpu().numpy(), want)
