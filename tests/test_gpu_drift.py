"""GPU drift alignment (align.py:12-176) against the reference's drift pickle and
the CPU oracle."""
import json
import os
import types

import numpy as np
import pytest
import torch

from oracle import align as oalign

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def al():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mermake_gb300 import align
    return align


@pytest.fixture(scope="module")
def feats(golden_dir):
    d = np.load(os.path.join(golden_dir, "dapi_features.npz"))
    return d["Xh_plus"], d["Xh_minus"]


def test_drift_matches_reference_pickle(al, feats, golden_dir):
    """drift_Conv_zscan__020--_set1.pkl: DualAligner(th=4) self-alignment."""
    kat = json.load(open(os.path.join(golden_dir, "drift_kat.json")))["drifts"][0]
    im = types.SimpleNamespace(Xh_plus=torch.from_numpy(feats[0]).cuda(), Xh_minus=torch.from_numpy(feats[1]).cuda(),
                               path="x/y.zarr")
    (drifts, files, ifov, ref_path), _ = al.drift([im])
    tf, tp, tm, Np, Nm = drifts[0]
    assert (Np, Nm) == (kat[3], kat[4]) == (621, 261)
    np.testing.assert_array_equal(tp, kat[1])
    np.testing.assert_array_equal(tm, kat[2])
    np.testing.assert_array_equal(tf, kat[0])
    assert np.all(np.signbit(tf) == np.signbit(np.asarray(kat[0], np.float32)))


def shifted(X, shift, seed, drop=0.1, jitter=0.3):
    rng = np.random.default_rng(seed)
    Y = X.copy()
    Y[:, :3] += np.asarray(shift, np.float32)
    Y[:, :3] += rng.normal(0, jitter, (len(Y), 3)).astype(np.float32)
    keep = rng.random(len(Y)) > drop
    return np.ascontiguousarray(Y[keep])


@pytest.mark.parametrize("shift", [(0.0, 0.0, 0.0), (1.3, -7.6, 12.2), (-2.7, 19.4, -18.8), (3.0, 0.4, 6.6)])
def test_translation_matches_oracle(al, feats, shift):
    """Known shifts (cfg 3 range: +-3 z, +-20 px xy) with point loss and jitter:
    the GPU shift equals the oracle's within 0.01 px and the match counts agree."""
    for k, X in enumerate(feats):
        ref = X[:, :3].copy()
        mov = shifted(X, shift, seed=k + 7)
        g = al.Aligner(torch.from_numpy(ref).cuda(), th=4)
        o = oalign.Aligner(ref, th=4)
        tg, ng = g.get_best_translation_points(torch.from_numpy(mov).cuda(), return_counts=True)
        to, no = o.get_best_translation_points(mov, return_counts=True)
        assert ng == no
        np.testing.assert_allclose(tg, to, atol=0.01)
        np.testing.assert_allclose(tg, shift, atol=0.5)


def test_dual_aligner_and_no_points(al, feats):
    ref = types.SimpleNamespace(Xh_plus=feats[0], Xh_minus=feats[1])
    mov = types.SimpleNamespace(Xh_plus=shifted(feats[0], (0.5, 4.0, -3.0), 1),
                                Xh_minus=shifted(feats[1], (0.5, 4.0, -3.0), 2))
    got = al.DualAligner(ref, th=4).get_best_translation_pointsV2(mov)
    want = oalign.DualAligner(ref, th=4).get_best_translation_pointsV2(mov)
    np.testing.assert_allclose(got[0], want[0], atol=0.01)
    assert got[3:] == want[3:]
    with pytest.raises(ValueError, match="No points left"):
        al.Aligner(torch.zeros((5, 3), device="cuda"), th=4)


@pytest.mark.parametrize("npts,shift", [(6000, (2.0, -13.4, 7.7)), (20000, (-1.2, 4.9, -18.6))])
def test_translation_many_points_matches_oracle(al, npts, shift):
    """A field-sized point set (the DAPI maxima of a 50 x 2048 x 2048 FOV are
    thousands): the cell-grid nearest-neighbour refinement spread over many
    blocks gives the oracle's shift and match count."""
    rng = np.random.default_rng(npts)
    ref = np.stack([rng.uniform(0, 50, npts), rng.uniform(0, 2048, npts), rng.uniform(0, 2048, npts)],
                   axis=1).astype(np.float32)
    mov = shifted(np.concatenate([ref, np.full((npts, 1), 10, np.float32)], axis=1), shift, seed=3)[:, :3]
    g = al.Aligner(torch.from_numpy(ref).cuda(), th=None)
    o = oalign.Aligner(ref, th=None)
    tg, ng = g.get_best_translation_points(torch.from_numpy(np.ascontiguousarray(mov)).cuda(), return_counts=True)
    to, no = o.get_best_translation_points(np.ascontiguousarray(mov), return_counts=True)
    assert ng == no
    np.testing.assert_allclose(tg, to, atol=0.01)
    np.testing.assert_allclose(tg, shift, atol=0.5)


def test_drift_save_round_trip_matches_reference_pickle(al, feats, golden_dir, tmp_path):
    """drift() -> drift_save (align.py:158-176) -> a plain pickle load: the
    reference pickle's nesting and values (N+ = 621, N- = 261, zero shift),
    with NumPy arrays in place of CuPy ones."""
    import pickle
    kat = json.load(open(os.path.join(golden_dir, "drift_kat.json")))
    lay = json.load(open(os.path.join(golden_dir, "output_layout.json")))["drift"]
    im = types.SimpleNamespace(Xh_plus=torch.from_numpy(feats[0]).cuda(), Xh_minus=torch.from_numpy(feats[1]).cuda(),
                               path=kat["ref_path"])
    data, _ = al.drift([im])
    path = tmp_path / lay["file"]
    al.drift_save(data, str(path))

    class NoCupy(pickle.Unpickler):
        def find_class(self, module, name):
            assert not module.startswith("cupy")
            return super().find_class(module, name)

    with open(path, "rb") as f:
        drifts, files, ifov, ref_path = NoCupy(f).load()
    tf, tp, tm, Np, Nm = drifts[0]
    assert all(isinstance(a, np.ndarray) and a.shape == (3,) for a in (tf, tp, tm))
    assert isinstance(Np, int) and isinstance(Nm, int) and (Np, Nm) == (621, 261)
    np.testing.assert_array_equal(tf, kat["drifts"][0][0])
    assert files == kat["files"] and ref_path == kat["ref_path"]
