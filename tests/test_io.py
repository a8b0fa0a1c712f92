"""Host-side I/O (no GPU): the zarr v2 reader on a written store, the FOV
reader and the prefetching loader on a written FOV (frames split into
channels by the xml's z_offsets), and -- where a MERMAKE checkout is named by
MERMAKE_REF -- the reader against the reference's own FOV fixture."""
import bz2
import json
import os

import numpy as np
import pytest

from tests.test_oracle import load_tile

REF = os.environ.get("MERMAKE_REF")
REF_FOV = os.path.join(REF, "tests/examples/single/H1_TEST_set1/Conv_zscan__020.zarr") if REF else ""


def test_zarr_round_trip(tmp_path):
    from mermake_gb300.io import read_zarr
    rng = np.random.default_rng(0)
    a = rng.integers(0, 255, (5, 7, 9)).astype(np.uint8)
    d = tmp_path / "arr"
    d.mkdir()
    json.dump({"chunks": [2, 7, 4], "compressor": {"id": "bz2", "level": 9}, "dtype": "|u1", "fill_value": 3,
               "filters": None, "order": "C", "shape": [5, 7, 9], "zarr_format": 2}, open(d / ".zarray", "w"))
    for i in range(3):
        for k in range(3):
            if (i, k) == (1, 1):
                continue  # missing chunk -> fill value
            blk = np.full((2, 7, 4), 0, np.uint8)
            src = a[2 * i:2 * i + 2, :, 4 * k:4 * k + 4]
            blk[:src.shape[0], :, :src.shape[2]] = src
            (d / f"{i}.0.{k}").write_bytes(bz2.compress(blk.tobytes()))
    got = read_zarr(str(d))
    want = a.copy()
    want[2:4, :, 4:8] = 3
    np.testing.assert_array_equal(got, want)


@pytest.mark.skipif(not REF_FOV or not os.path.exists(REF_FOV), reason="MERMAKE_REF does not name a checkout")
def test_read_im_matches_fixture_crops(golden_dir):
    """io.py:116-146 on the reference fixture: 3 channels x 35 z, uint16 = u8**2."""
    from mermake_gb300.io import read_im
    im = read_im(REF_FOV)
    assert im.shape == (3, 35, 1200, 1200) and im.dtype == np.uint16
    for k in range(3):
        t = load_tile(golden_dir, k)
        x0, x1, y0, y1 = t["box"][2:]
        np.testing.assert_array_equal(im[0][:, x0:x1, y0:y1], t["img"][:, x0:x1, y0:y1])


def write_fov(root, name, frames, nch, chunk=None, missing=()):
    """A FOV in the layout read_im reads (io.py:116-146): ``<name>.zarr`` beside
    ``<name>.xml`` (z_offsets ending in ':nch'), the frames in the zarr v2 store
    ``<fov>/data`` as uint8 bz2 chunks of ``chunk`` frames."""
    n, X, Y = frames.shape
    chunk = chunk or (1, X, Y)
    fov = name.split("_")[-1]
    d = root / fov / "data"
    d.mkdir(parents=True)
    json.dump({"chunks": list(chunk), "compressor": {"id": "bz2", "level": 9}, "dtype": "|u1", "fill_value": 0,
               "filters": None, "order": "C", "shape": [n, X, Y], "zarr_format": 2}, open(d / ".zarray", "w"))
    for i in range(-(-n // chunk[0])):
        for j in range(-(-X // chunk[1])):
            for k in range(-(-Y // chunk[2])):
                if (i, j, k) in missing:
                    continue
                blk = np.zeros(chunk, np.uint8)
                src = frames[i * chunk[0]:(i + 1) * chunk[0], j * chunk[1]:(j + 1) * chunk[1],
                             k * chunk[2]:(k + 1) * chunk[2]]
                blk[:src.shape[0], :src.shape[1], :src.shape[2]] = src
                (d / f"{i}.{j}.{k}").write_bytes(bz2.compress(blk.tobytes()))
    (root / (name + ".xml")).write_text('<settings><z_offsets type="string">-5:0.5:5:%d</z_offsets>'
                                        '<stage_position type="custom">[12.5, -3.25]</stage_position></settings>'
                                        % nch)
    (root / (name + ".zarr")).mkdir()
    return str(root / (name + ".zarr"))


def test_read_im_splits_channels(tmp_path):
    """Frame 0 dropped, frames 1.. dealt to nch channels in turn, uint8 widened
    to uint16 ** 2, trailing frames that do not fill a plane dropped."""
    from mermake_gb300.io import read_im
    rng = np.random.default_rng(1)
    frames = rng.integers(0, 256, (1 + 3 * 4 + 2, 10, 12)).astype(np.uint8)
    path = write_fov(tmp_path, "Conv_zscan__007", frames, 3)
    im, x, y = read_im(path, return_pos=True)
    assert im.shape == (3, 4, 10, 12) and im.dtype == np.uint16 and (x, y) == (12.5, -3.25)
    for c in range(3):
        for z in range(4):
            np.testing.assert_array_equal(im[c, z], frames[1 + 3 * z + c].astype(np.uint16) ** 2)


@pytest.mark.parametrize("chunk,missing", [(None, ()), ((4, 6, 5), ((1, 1, 2),))])
def test_prefetcher_matches_read_im(tmp_path, chunk, missing):
    """FovPrefetcher (the ImageQueue worker's role, io.py:405-463): FOVs in
    order, each equal to read_im's, with chunks of several frames and partial
    and missing chunks; a FOV that fails to read is reported, not raised."""
    from mermake_gb300 import io
    rng = np.random.default_rng(2)
    paths, want = [], []
    for f in range(3):
        frames = rng.integers(0, 256, (1 + 2 * 5, 13, 11)).astype(np.uint8)
        root = tmp_path / f"r{f}"
        root.mkdir()
        paths.append(write_fov(root, "Conv_zscan__%03d" % f, frames, 2, chunk, missing))
        want.append(io.read_im(paths[-1]))
    paths.append(str(tmp_path / "absent" / "Conv_zscan__009.zarr"))
    with io.FovPrefetcher(paths, prefetch=1, workers=3, pin=False) as pf:
        got = list(pf)
    assert [p for p, _ in got] == paths
    for (_, im), w in zip(got[:3], want):
        np.testing.assert_array_equal(im.numpy().view(np.uint16) if hasattr(im, "numpy") else im, w)
    assert isinstance(got[3][1], Exception)
    assert pf.decoded_bytes > 0 and pf.decode_seconds > 0
