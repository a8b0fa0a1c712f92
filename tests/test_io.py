"""Host-side I/O (no GPU): the zarr v2 reader against the reference's FOV
fixture (where the reference tree is present) and a written round trip."""
import bz2
import json
import os

import numpy as np
import pytest

from tests.test_oracle import load_tile

REF_FOV = "/root/reference/tests/examples/single/H1_TEST_set1/Conv_zscan__020.zarr"


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


@pytest.mark.skipif(not os.path.exists(REF_FOV), reason="reference FOV fixture not present")
def test_read_im_matches_fixture_crops(golden_dir):
    """io.py:116-146 on the reference fixture: 3 channels x 35 z, uint16 = u8**2."""
    from mermake_gb300.io import read_im
    im = read_im(REF_FOV)
    assert im.shape == (3, 35, 1200, 1200) and im.dtype == np.uint16
    for k in range(3):
        t = load_tile(golden_dir, k)
        x0, x1, y0, y1 = t["box"][2:]
        np.testing.assert_array_equal(im[0][:, x0:x1, y0:y1], t["img"][:, x0:x1, y0:y1])
