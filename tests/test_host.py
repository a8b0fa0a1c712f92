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
    d._tuned = {((40, 3000, 3000), False): (4, 3)}
    assert tune.batch_for(d, (40, 3000, 3000)) == 4
    assert tune.zform_for(d, (40, 3000, 3000)) == 3
    assert tune.settings_for(d, (40, 3000, 3000)) == (4, 3)
    assert tune.batch_for(d, (40, 3000, 3000), dapi=True) == 9
    assert tune.zform_for(d, (40, 3000, 3000), dapi=True) == 0  # MM_ZFORM_AUTO


def test_tuner_z_forms_per_deconvolver():
    """tune.zforms: with one PSF, the register, tensor, shared-memory, direct
    and transform forms; with a PSF per tile, the register form (each tile's
    matrix from its own z kernel), the direct sum and the transforms; without
    z kernels, the transforms only."""
    import types
    from mermake_gb300 import tune
    L = _lib
    one = types.SimpleNamespace(z_operator=object(), psf_fft=np.zeros((1, 2)))
    grid = types.SimpleNamespace(z_operator=object(), psf_fft=np.zeros((100, 2)))
    none = types.SimpleNamespace(z_operator=None, psf_fft=np.zeros((1, 2)))
    assert tune.zforms(one) == [L.MM_ZFORM_REGISTERS, L.MM_ZFORM_TENSOR, L.MM_ZFORM_SHARED, L.MM_ZFORM_DIRECT,
                                L.MM_ZFORM_TRANSFORMS]
    assert tune.zforms(grid) == [L.MM_ZFORM_REGISTERS, L.MM_ZFORM_DIRECT, L.MM_ZFORM_TRANSFORMS]
    assert tune.zforms(none) == [L.MM_ZFORM_TRANSFORMS]


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


def _map_z(z, Z, zpad, Zp):
    """mm_map_z (csrc/deconv.cuh): padded plane z -> real plane, or -1."""
    i2 = zpad + Z - 1
    q = z
    if z > i2 and 2 * i2 - z >= 0:
        q = 2 * i2 - z
    if q < zpad and 2 * zpad - q < Zp:
        q = 2 * zpad - q
    return q - zpad if zpad <= q < zpad + Z else -1


@pytest.mark.parametrize("Z,zpad", [(13, 12), (50, 49), (50, 24), (7, 2), (5, 9), (40, 39), (1, 1), (80, 79),
                                    (128, 1)])
def test_z_sum_index_algebra_matches_the_padded_transforms(Z, zpad):
    """The index arithmetic of k_zconv (csrc/zop.cu) restated in NumPy: the
    staged kernel run wx[u] = w[(u + zpad + 1 - Tpad) mod Zp] of
    ceil(Z/8)*8 + Tpad - 1 rows, the 15-value window at i0 - zb + Tpad - 8, the
    zero row for unmapped planes; against reflect padding, FFT over Zp, times
    W, inverse FFT and the crop.  Every window read stays inside the run."""
    kCI = 8
    Zp = Z + 2 * zpad
    rng = np.random.default_rng(Z * 1000 + zpad)
    X = rng.standard_normal(Z) + 1j * rng.standard_normal(Z)
    W = rng.standard_normal(Zp) + 1j * rng.standard_normal(Zp)
    w = np.fft.ifft(W)  # the z kernel: inverse DFT of W (W carries 1 / Zp here)
    Tpad = -(-Zp // kCI) * kCI
    G = -(-Z // kCI)
    Lw = G * kCI + Tpad - 1
    wx = np.array([w[(u + zpad + 1 - Tpad) % Zp] for u in range(Lw)])
    xs = np.concatenate([X, [0]])
    zm = [(_map_z(z, Z, zpad, Zp) if z < Zp else -1) for z in range(Tpad)]
    zm = [Z if m < 0 else m for m in zm]
    Y = np.zeros(Z, complex)
    for g in range(G):
        i0 = g * kCI
        acc = np.zeros(kCI, complex)
        for zb in range(0, Tpad, kCI):
            base = i0 - zb + Tpad - kCI
            assert 0 <= base and base + 2 * kCI - 2 < Lw
            wr = wx[base:base + 2 * kCI - 1]
            for s_ in range(kCI):
                acc += wr[kCI - 1 - s_:2 * kCI - 1 - s_] * xs[zm[zb + s_]]
        n = min(kCI, Z - i0)
        Y[i0:i0 + n] = acc[:n]
    xp = np.array([X[m] if (m := _map_z(z, Z, zpad, Zp)) >= 0 else 0 for z in range(Zp)])
    want = np.fft.ifft(np.fft.fft(xp) * W)[zpad:zpad + Z]
    assert np.abs(Y - want).max() <= 1e-12 * np.abs(want).max()


@pytest.mark.parametrize("R,N1,N2,g", [(113, 16, 7, 3), (239, 14, 17, 7)])
@pytest.mark.parametrize("inverse", [False, True])
def test_rader_split_matches_the_dft(R, N1, N2, g, inverse):
    """The three passes of stage_rader<R, N1, N2> (csrc/fft.cuh) with the tables
    of rader_tables (csrc/fft_plan.cu), restated in NumPy for one butterfly:
    gather u[q1 + N1 q2] = x[g^-(q1 + N1 q2)] and an N2-point DFT times
    wM^(q1 k2); per k2 an N1-point DFT, the product with H[k2 + N2 k1] and the
    inverse N1-point DFT times wM^-(q1 k2); an inverse N2-point DFT and the
    scatter to X[g^(q1 + N1 q2)], with X[0] = x0 + sum u."""
    M = R - 1
    ginv = pow(g, R - 2, R)
    gp = [pow(g, q, R) for q in range(M)]
    gi = [pow(ginv, q, R) for q in range(M)]
    assert len(set(gp)) == M  # g is a primitive root
    sgn = 1 if inverse else -1
    H = np.fft.fft(np.exp(sgn * 2j * np.pi * np.array(gp) / R)) / M
    wM = np.exp(-2j * np.pi * np.arange(M) / M)
    x = np.random.default_rng(R).standard_normal(R) + 1j * np.random.default_rng(R + 1).standard_normal(R)
    T = np.zeros(M, complex)
    for q1 in range(N1):
        v = np.fft.fft([x[gi[q1 + N1 * q2]] for q2 in range(N2)])
        T[q1 * N2:(q1 + 1) * N2] = v * np.array([wM[q1 * k2] if k2 else 1 for k2 in range(N2)])
    for k2 in range(N2):
        v = np.fft.fft(T[k2::N2][:N1])
        if k2 == 0:
            s0 = v[0]
        v = np.fft.ifft(v * H[k2 + N2 * np.arange(N1)]) * N1
        T[k2] = v[0]
        for q1 in range(1, N1):
            T[q1 * N2 + k2] = v[q1] * np.conj(wM[q1 * k2])
    X = np.zeros(R, complex)
    for q1 in range(N1):
        v = np.fft.ifft(T[q1 * N2:(q1 + 1) * N2]) * N2
        for q2 in range(N2):
            X[gp[q1 + N1 * q2]] = x[0] + v[q2]
    X[0] = x[0] + s0
    want = np.fft.ifft(x) * R if inverse else np.fft.fft(x)
    assert np.abs(X - want).max() <= 1e-12 * np.abs(want).max()


def test_fov_graph_settings_follow_the_driver_defaults():
    """FovGraph reads a TOML section as hyb_spots does: None threshold -> NaN
    (every voxel), None blur -> -1 (no blur), delta > 5 -> TypeError."""
    from mermake_gb300 import pipeline
    a = pipeline._settings({"threshold": None, "blur_radius": None})
    assert np.isnan(a["th"]) and a["br"] == -1 and a["delta"] == 1 and a["dfit"] == 0
    b = pipeline._settings(dict(threshold=3600, blur_radius=30, delta=1, delta_fit=3, sigmaZ=1, sigmaXY=1.5))
    assert (b["th"], b["br"], b["dfit"], b["sxy"]) == (3600.0, 30, 3, 1.5)
    with pytest.raises(TypeError, match="Delta must be"):
        pipeline._settings({"delta": 6})


def test_zpass_flop_model_follows_the_z_pass_form():
    """bench.zpass_flops: the matrix form (Z x Z complex FMAs per frequency and
    tile) for one spectrum and >= 10 tiles of height <= 64, or per tile for Z
    a multiple of 5 up to 80 with 1 <= zpad <= Z - 1, else (or with the direct
    form forced) the direct sum (outputs and padded planes in blocks of 8);
    8 flops a complex FMA."""
    import sys
    import types
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    def dec(Z, zpad, P, npsf, nt):
        return types.SimpleNamespace(tile_height=Z, zpad=zpad, Zp=Z + 2 * zpad, P=P, H=P // 2 + 1,
                                     z_operator=object(), psf_fft=np.zeros((npsf, 1)), n_tiles=lambda shape: nt)

    w = dict(Z=50, X=2048, Y=2048, colours=3)
    s = dict(dec_h=dec(50, 49, 678, 1, 25), dec_d=dec(50, 24, 678, 1, 25))
    assert bench.zpass_flops(w, s) == 4 * 25 * 678 * 340 * 2500 * 8.0
    w = dict(Z=40, X=3000, Y=3000, colours=1)
    s = dict(dec_h=dec(40, 39, 478, 100, 100), dec_d=None)
    assert bench.zpass_flops(w, s) == 100 * 478 * 240 * 1600 * 8.0
    assert bench.zpass_flops(w, s, "direct") == 100 * 478 * 240 * 40 * 120 * 8.0
    w = dict(Z=42, X=3000, Y=3000, colours=1)
    s = dict(dec_h=dec(42, 41, 478, 100, 100), dec_d=None)
    assert bench.zpass_flops(w, s) == 100 * 478 * 240 * 48 * 128 * 8.0


def test_z_operator_register_rings_restate_the_matrix():
    """The register z operator (csrc/zop_tma.cu) forms M[i][j] in registers from
    two rings of five values: the direct copy w[i - j], and the reflected copy
    of the column's class, read from the staged kernel rows (w[i + j] or
    w[i + j - 2Z + 2]), from hB[i + j] = w[i + j] + w[i + j - 2Z + 2] where
    both reflections copy plane j, or from zero rows where neither does.  The
    columns come in segments of one class; a column that starts a segment
    reloads the reflected ring.  Restated here with the kernel's slot
    arithmetic, segment table and staged rows (k + kA for w[k mod Zp], kA =
    2Z - 2 rounded up to a multiple of 4, the rows past the padded depth zero as
    the TMA fills them; hB after them), against M built from the padding map;
    every read stays inside the staged, hB or zero rows."""
    rng = np.random.default_rng(5)
    for Z, zpad in [(50, 49), (50, 24), (30, 29), (40, 20), (10, 3), (15, 14), (20, 9), (80, 79), (80, 39)]:
        Zp = Z + 2 * zpad
        w = rng.standard_normal(Zp) + 1j * rng.standard_normal(Zp)
        M = np.zeros((Z, Z), complex)
        for z in range(Zp):
            j = int(_map_z(z, Z, zpad, Zp))
            if j >= 0:
                for i in range(Z):
                    M[i, j] += w[(zpad + i - z) % Zp]
        kA = (2 * Z - 2 + 3) & ~3  # rows of box A: 2Z - 2 rounded up to a multiple of 4 (128-byte boxes)
        kb, ko = kA, kA - (2 * Z - 2)
        assert (kA * 4 * 8) % 128 == 0
        wrows = kA + 2 * Z - 1
        staged = np.zeros(wrows + 2 * Z - 1, complex)
        for row in range(kA):  # box A: kernel rows Zp - kA .. Zp - 1 (negative rows read as zero)
            src = Zp - kA + row
            staged[row] = w[src] if 0 <= src < Zp else 0
        for row in range(2 * Z - 1):  # box B: kernel rows 0 .. 2Z - 2 (rows >= Zp read as zero)
            staged[kA + row] = w[row] if row < Zp else 0
        for sr in range(2 * Z - 1):  # hB, written by the producer warp
            staged[wrows + sr] = staged[sr + kb] + staged[sr + ko]
        zeros = np.zeros(2 * Z + 3, complex)
        zrow = 1000  # the zero rows, elsewhere in shared memory
        # column segments of one reflection class (the host's table)
        segj, segc = [], []
        for j in range(Z):
            vin, vout = 1 <= j <= zpad, Z - 1 - zpad <= j <= Z - 2
            cls = (2 if vout else 0) if vin else (1 if vout else 3)
            if not segc or segc[-1] != cls:
                segj.append(j)
                segc.append(cls)
        assert len(segj) <= 6
        if zpad == Z - 1 and Z >= 2:
            # the fixed classes the per-tile kernel (csrc/zop_pt.cu) compiles
            # in for zpad = Z - 1: column 0, columns 1 .. Z - 2, column Z - 1
            assert (segj, segc) == (([0, 1, Z - 1], [1, 2, 0]) if Z > 2 else ([0, 1], [1, 0]))

        def at(i):
            if i >= zrow:
                assert i - zrow < len(zeros), i
                return zeros[i - zrow]
            assert 0 <= i < len(staged), i  # every read stays inside the staged rows
            return staged[i]

        def seg_row(k):
            return {0: kb, 1: ko, 2: wrows, 3: zrow}[segc[k]]

        got = np.zeros((Z, Z), complex)
        for i0 in range(0, Z, 5):
            sk, hrow = 0, seg_row(0)
            jnext = segj[1] if len(segj) > 1 else Z
            rT, rH = [0j] * 5, [0j] * 5
            for q in range(1, 5):
                rT[q] = at(i0 + q + kb)
            for q in range(4):
                rH[q] = at(i0 + q + hrow)
            for j0 in range(0, Z, 5):
                for u in range(5):
                    j = j0 + u
                    rT[(5 - u) % 5] = at(i0 - j + kb)
                    if j == jnext:
                        sk += 1
                        hrow = seg_row(sk)
                        jnext = segj[sk + 1] if sk + 1 < len(segj) else Z
                        for q in range(4):
                            rH[(q + u) % 5] = at(i0 + j + q + hrow)
                    rH[(u + 4) % 5] = at(i0 + j + 4 + hrow)
                    for q in range(5):
                        got[i0 + q, j] = rT[(q - u + 5) % 5] + rH[(q + u) % 5]
        np.testing.assert_allclose(got, M, rtol=0, atol=1e-12)


@pytest.mark.parametrize("Z", [10, 15, 40, 50, 80])
def test_per_tile_z_operator_full_variant_restates_the_matrix(Z):
    """The per-tile z operator's variant for zpad = Z - 1 (csrc/zop_pt.cu,
    k_zpt_apply<., true, .>): its producer stages the tile's kernel rows
    w[-kA .. 2Z - 2] by copying, in two linear runs, the rows
    [max(kA - Zp, 0), kA) from w[r - kA + Zp] and [kA, min(kA + Zp, wrows))
    from w[r - kA] (the rest are zero rows written once); column 0 takes the
    reflection w[i + j - 2Z + 2], columns 1 .. Z - 2 the sum
    w[i + j] + w[i + j - 2Z + 2] formed as the reflected ring is loaded (two
    staged rows per value), column Z - 1 the reflection w[i + j], the class
    changes at compile-time columns.  Restated with the kernel's ring slots
    and staged rows against M built from the padding map; every read stays
    inside the staged rows."""
    zpad = Z - 1
    Zp = Z + 2 * zpad
    rng = np.random.default_rng(Z)
    w = rng.standard_normal(Zp) + 1j * rng.standard_normal(Zp)
    M = np.zeros((Z, Z), complex)
    for z in range(Zp):
        j = int(_map_z(z, Z, zpad, Zp))
        if j >= 0:
            for i in range(Z):
                M[i, j] += w[(zpad + i - z) % Zp]
    kA = (2 * Z - 2 + 3) & ~3
    kb, ko = kA, kA - (2 * Z - 2)
    wrows = kA + 2 * Z - 1
    rlo, rhi = max(kb - Zp, 0), min(wrows, kb + Zp)
    staged = np.full(wrows, np.nan, complex)
    staged[:rlo] = 0
    staged[rhi:] = 0
    for r in range(rlo, kb):  # first run
        staged[r] = w[r - kb + Zp]
    for r in range(kb, rhi):  # second run
        staged[r] = w[r - kb]
    assert not np.isnan(staged).any()

    def at(i):
        assert 0 <= i < wrows, i
        return staged[i]

    got = np.zeros((Z, Z), complex)
    for i0 in range(0, Z, 5):
        rT, rH = [0j] * 5, [0j] * 5
        for q in range(1, 5):  # ring_start, column 0's class (hrow = ko)
            rT[q] = at(i0 + q + kb)
        for q in range(4):
            rH[q] = at(i0 + q + ko)

        def col(j, u, rh):
            rT[(5 - u) % 5] = at(i0 - j + kb)
            rH[(u + 4) % 5] = rh(i0 + j + 4)
            for q in range(5):
                got[i0 + q, j] = rT[(q - u + 5) % 5] + rH[(q + u) % 5]

        one = lambda h: at(h + ko)  # noqa: E731
        two = lambda h: at(h + kb) + at(h + ko)  # noqa: E731
        col(0, 0, one)
        for q in range(4):  # reload2<1>
            rH[(q + 1) % 5] = two(i0 + 1 + q)
        for j in range(1, Z - 1):
            col(j, j % 5, two)
        for q in range(4):  # reload<4> from w[i + j]
            rH[(q + 4) % 5] = at(i0 + Z - 1 + q + kb)
        col(Z - 1, (Z - 1) % 5, lambda h: at(h + kb))
    np.testing.assert_allclose(got, M, rtol=0, atol=1e-12)


def _unit_protocol_run(rng, nwarps, nunits, nitems):
    """One simulated run of the register z operator's warp-unit protocol
    (csrc/zop_tma.cu): nwarps compute warps take units in order from a shared
    counter (unit u of item it = sequence number it * nunits + u) and wait for
    their buffer (it & 1) with an mbarrier parity wait, (it >> 1) & 1; the
    producer fills item it once all units of item it - 2 have arrived on the
    buffer's "empty" barrier.  A parity wait passes once the number of
    completed phases P has P % 2 != parity.  Returns [] after a run whose
    every wait passed on its own item's phase, else [(item, completed
    phases)] of the first wait that did not."""
    import heapq
    full_done, empty_done, empty_cnt = [0, 0], [0, 0], [0, 0]
    counter, t_now, ev = 0, 0.0, []
    prod = {"it": 0, "busy": False}
    done = set()
    warps = ["grab"] * nwarps
    for _ in range(200000):
        if not prod["busy"] and prod["it"] < nitems:
            it = prod["it"]
            if it < 2 or empty_done[it & 1] % 2 != ((it - 2) >> 1) & 1:
                prod["busy"] = True
                heapq.heappush(ev, (t_now + float(rng.uniform(0.1, 3.0)), 0, it))
        progress = False
        for k in range(nwarps):
            if warps[k] == "grab":
                it, u = divmod(counter, nunits)
                counter += 1
                warps[k] = "done" if it >= nitems else ("wait", it, u)
                progress = True
            st = warps[k]
            if isinstance(st, tuple) and st[0] == "wait":
                _, it, u = st
                b = it & 1
                if full_done[b] % 2 != (it >> 1) & 1:
                    if full_done[b] != (it >> 1) + 1:
                        return [(it, full_done[b])]  # what follows runs on the wrong data
                    assert (it, u) not in done
                    warps[k] = ("run", it, u)
                    heapq.heappush(ev, (t_now + float(rng.uniform(0.5, 2.0)), 1, k))
                    progress = True
        if all(w == "done" for w in warps) and prod["it"] >= nitems and not ev:
            assert len(done) == nitems * nunits
            return []
        if not progress:
            assert ev, "deadlock"
            t_now, kind, pay = heapq.heappop(ev)
            if kind == 0:
                full_done[pay & 1] += 1
                prod["busy"] = False
                prod["it"] += 1
            else:
                _, it, u = warps[pay]
                done.add((it, u))
                empty_cnt[it & 1] += 1
                if empty_cnt[it & 1] == nunits:
                    empty_cnt[it & 1] = 0
                    empty_done[it & 1] += 1
                warps[pay] = "grab"
    raise AssertionError("no end")


def test_register_z_operator_warp_unit_protocol():
    """The register z operator's compute warps take an item's warp units from
    a shared counter and wait for their buffer with a parity wait only.  With
    as many units per item as compute warps (the kernel: ncw of each), every
    wait passes on its own item's phase, every unit runs once and nothing
    deadlocks (random unit times and copy latencies).  A warp could pass on
    an earlier phase only by reaching item it while item it - 2's buffer is
    unfilled; the producer fills in order, so then no unit of items it - 2 and
    it - 1 can have finished, and holding them takes 2 x units warps besides
    the taker: with 2 x units + 1 warps the simulation finds such a pass,
    with the kernel's units = warps it cannot happen."""
    rng = np.random.default_rng(11)
    for _ in range(300):
        n = int(rng.integers(1, 9))
        assert _unit_protocol_run(rng, n, n, int(rng.integers(1, 25))) == []
    found = 0
    for _ in range(100):
        u = int(rng.integers(1, 4))
        found += len(_unit_protocol_run(rng, 2 * u + 1, u, int(rng.integers(3, 25)))) > 0
    assert found > 0
