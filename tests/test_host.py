"""Host-side checks that need no GPU: the C ABI library loads and exports what
include/*.h declares, and the tile layout it computes reproduces the
reference's placement + reflect sequence exactly."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

from mermake_gb300 import _lib
from oracle import deconv as od

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names.update(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(mm_\w+)\s*\(", txt, flags=re.M))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = _lib.load(require_gpu=False)
    names = header_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(_lib.declared_symbols())
    assert L.mm_abi_version() == 1


GEOMS = [  # (Z, X, Y, tile_size, zpad, overlap, npsf)
    (35, 1200, 1200, 300, 35, 89, 1),    # the reference FOV fixture, tile 300
    (35, 1200, 1200, 500, 35, 89, 1),    # tile 500 (thin last tile, xd = 289)
    (50, 2048, 2048, 500, 49, 89, 1),    # hyb FOV
    (50, 2048, 2048, 500, 24, 89, 1),    # DAPI zpad
    (40, 500, 500, 500, 39, 89, 1),      # one tile, right pad left at zero
    (10, 50, 50, 30, 5, 5, 1),           # small geometry of test_deconvolver.py
    (7, 23, 41, 10, 3, 4, 1),
    (5, 9, 9, 4, 2, 6, 1),               # overlap wider than the tile
    (12, 100, 100, 30, 4, 7, 3),         # several spectra: zip truncates to 3 tiles
]


def geometry(geom, tile):
    Z, X, Y, ts, zpad, ov, npsf = geom
    L = _lib.load(require_gpu=False)
    desc = np.zeros(13, np.int32)
    rc = L.mm_tile_geometry(Z, X, Y, ts, zpad, ov, npsf, tile, desc.ctypes.data, None, None, None)
    assert rc == 0
    P, Zp = desc[11], desc[12]
    mz, mx, my = np.zeros(Zp, np.int32), np.zeros(P, np.int32), np.zeros(P, np.int32)
    rc = L.mm_tile_geometry(Z, X, Y, ts, zpad, ov, npsf, tile, None, mz.ctypes.data, mx.ctypes.data,
                            my.ctypes.data)
    assert rc == 0
    return desc, mz, mx, my


@pytest.mark.parametrize("geom", GEOMS)
def test_tile_layout_reproduces_reference_padding(geom):
    """The kernels gather the padded tile through per-axis maps; the oracle
    runs the reference's placement and fill.reflect calls literally.  Three
    axis-coded tiles (value = 1 + index along one axis) pin each map."""
    Z, X, Y, ts, zpad, ov, npsf = geom
    L = _lib.load(require_gpu=False)
    nt = L.mm_tile_geometry(Z, X, Y, ts, zpad, ov, npsf, -1, None, None, None, None)
    boxes = od.tiles((Z, X, Y), ts, ov)
    assert nt == (len(boxes) if npsf == 1 else min(npsf, len(boxes)))
    ny = -(-Y // ts)
    # first, last, middle, and the second-to-last along y and x (where xd + ov
    # can exceed the padded size and the yielded extent is clipped)
    pick = sorted({0, max(ny - 2, 0), ny - 1, nt // 2, max(nt - 2 * ny, 0), max(nt - ny, 0), nt - 1}
                  if nt > 8 else set(range(nt)))
    for t in pick:
        desc, mz, mx, my = geometry(geom, t)
        P = int(desc[11])
        x, y, x0, x1, y0, y1 = boxes[t]
        assert tuple(desc[:6]) == (x, y, x0, y0, x1 - x0, y1 - y0)
        zd, xd, yd = Z, x1 - x0, y1 - y0
        valid = (mz[:, None, None] >= 0) & (mx[None, :, None] >= 0) & (my[None, None, :] >= 0)
        grids = np.meshgrid(np.arange(zd), np.arange(xd), np.arange(yd), indexing="ij")
        for ax, m in enumerate((mz[:, None, None], mx[None, :, None], my[None, None, :])):
            tile = (1 + grids[ax]).astype(np.float32)
            pad, xs, ys, xend, yend = od.pad_tile(tile, None, x, y, ts, zpad, ov)
            # the reference yields tile_res[:, :xend, :yend], which slicing clips at P
            assert (xs, ys, min(xend, P), min(yend, P)) == tuple(desc[6:10])
            want = np.where(valid, m + 1, 0).astype(np.float32)
            np.testing.assert_array_equal(pad, want)


def test_tile_geometry_rejects_bad_arguments():
    L = _lib.load(require_gpu=False)
    assert L.mm_tile_geometry(10, 50, 50, 30, 0, 5, 1, 0, None, None, None, None) == _lib.MM_EINVAL
    assert b"zpad" in L.mm_last_error()
    assert L.mm_tile_geometry(10, 50, 50, 30, 5, 5, 1, 99, None, None, None, None) == _lib.MM_EINVAL


def test_find_local_maxima_rejects_large_delta_before_any_device_work():
    from mermake_gb300.maxima import find_local_maxima
    with pytest.raises(TypeError, match="Delta must be an less than or equal to 5"):
        find_local_maxima(np.ones((3, 3, 3), np.float32), threshold=0.5, delta=6, delta_fit=1)


def test_default_batch_takes_all_tiles_within_the_scratch_budget(monkeypatch):
    """tune.default_batch: one batch of all tiles (-1) while their scratch
    fits SCRATCH_BYTES, else as many tiles as fit; a tuned size wins."""
    import types
    from mermake_gb300 import tune

    def dec(Z, ts, ov, nt):
        P = ts + 2 * ov
        return types.SimpleNamespace(tile_height=Z, P=P, H=P // 2 + 1, n_tiles=lambda shape: nt)

    assert tune.default_batch(dec(40, 300, 89, 100), (40, 3000, 3000)) == -1    # 11 GB
    assert tune.default_batch(dec(50, 500, 89, 25), (50, 2048, 2048)) == -1    # 6.9 GB
    monkeypatch.setattr(tune, "SCRATCH_BYTES", 1 << 30)
    assert tune.default_batch(dec(40, 300, 89, 100), (40, 3000, 3000)) == 9     # 110 MB per tile
    assert tune.default_batch(dec(50, 500, 89, 25), (50, 2048, 2048)) == 3
    d = dec(40, 300, 89, 100)
    d._tuned_batch = {((40, 3000, 3000), False): 4}
    assert tune.batch_for(d, (40, 3000, 3000)) == 4
    assert tune.batch_for(d, (40, 3000, 3000), dapi=True) == 9


def test_spot_capacity_grows_from_counts_seen():
    """The drivers size the output rows from the largest count a Deconvolver
    has returned for the shape (plus a quarter), so a FOV with more spots than
    the default overflows (and reruns) once, not on every call."""
    import types
    from mermake_gb300 import pipeline
    dec = types.SimpleNamespace()
    key = ("hyb", 40, 3000, 3000)
    assert pipeline._capacity(dec, key, 1 << 18) == 1 << 18
    pipeline._seen(dec, key, 322214)
    assert pipeline._capacity(dec, key, 1 << 18) == 322214 + 322214 // 4
    pipeline._seen(dec, key, 1000)                       # a smaller count keeps the largest
    assert pipeline._capacity(dec, key, 1 << 18) == 322214 + 322214 // 4
    assert pipeline._capacity(dec, ("dapi+", 40, 3000, 3000), 1 << 16) == 1 << 16
