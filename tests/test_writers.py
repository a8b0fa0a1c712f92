"""Output formats (no GPU): the writers keep the layout of the reference's own
output files (mermake/io.py:561-586, mermake/align.py:158-176).

``tests/golden/output_layout.json`` records, from the reference's
``tests/examples/single/out`` files, each ``.npz``'s keys, dtypes and shapes,
its ``args`` table and the settings it was written from, and the nested
types of the drift ``.pkl`` (made by ``tests/golden/make_golden.py``).
"""
import json
import os
import pickle
import tomllib

import numpy as np
import pytest

from mermake_gb300 import __version__, align, io


@pytest.fixture(scope="module")
def layout(golden_dir):
    return json.load(open(os.path.join(golden_dir, "output_layout.json")))


@pytest.fixture(scope="module")
def args_array(layout):
    """ImageQueue.args_array (io.py:325): the parsed TOML through namespace_to_array."""
    settings = io.dict_to_namespace(tomllib.loads(layout["settings_toml"]))
    return np.array(io.namespace_to_array(settings))


def test_args_table_matches_reference_files(layout, args_array):
    want = np.array(layout["args"])
    assert args_array.shape == (30, 3) == want.shape
    assert args_array.dtype == want.dtype
    np.testing.assert_array_equal(args_array, want)


def check_npz(path, entry, extra_rows):
    d = np.load(path)  # plain NumPy, no pickles
    assert sorted(d.files) == sorted(entry["keys"])
    for k, (dt, shape) in entry["keys"].items():
        assert d[k].dtype.kind == np.dtype(dt).kind, k
        if k in extra_rows:
            assert d[k].dtype == np.dtype(dt) and d[k].shape == extra_rows[k].shape, k
            np.testing.assert_array_equal(d[k], extra_rows[k])
        elif k == "version":
            assert d[k].shape == () and str(d[k]) == __version__
        else:
            assert list(d[k].shape) == shape, k
    return d


def test_save_xfits_layout(tmp_path, layout, args_array):
    """A colour's file: version, args (30, 3) and Xh (N, 8) float32 under the
    reference's file name; an existing file is never overwritten
    (io.py:574)."""
    src = "tests/examples/single/H1_TEST_set1/Conv_zscan__020.zarr"
    name = io.output_name(src, 0, hyb_save=args_array[8, 2])
    assert name == layout["hyb"]["file"]
    rng = np.random.default_rng(0)
    Xh = rng.random((123, 8)).astype(np.float32)
    path = tmp_path / name
    io.save_xfits(str(path), args_array, Xh)
    d = check_npz(path, layout["hyb"], {"Xh": Xh})
    np.testing.assert_array_equal(d["args"], np.array(layout["args"]))
    io.save_xfits(str(path), args_array, Xh[:5])
    assert np.load(path)["Xh"].shape == (123, 8)


def test_save_dapi_layout(tmp_path, layout, args_array, golden_dir):
    """The DAPI file: Xh_plus / Xh_minus float32 beside version and args."""
    src = "tests/examples/single/H1_TEST_set1/Conv_zscan__020.zarr"
    name = io.output_name(src, -1, dapi_save=args_array[9, 2])
    assert name == layout["dapi"]["file"]
    feats = np.load(os.path.join(golden_dir, "dapi_features.npz"))
    path = tmp_path / name
    io.save_dapi(str(path), args_array, feats["Xh_plus"], feats["Xh_minus"])
    check_npz(path, layout["dapi"], {"Xh_plus": feats["Xh_plus"], "Xh_minus": feats["Xh_minus"]})


def test_output_names_follow_get_name():
    """ImageQueue.get_name (io.py:535-546) with the templates of the settings:
    ifov is the digits before .zarr and iset the digits after _set in the
    path.  (The reference's drift fixture, drift_Conv_zscan__020--_set1.pkl,
    was written by an earlier version whose ifov was the FOV name; its
    __main__.py default template 'drift_Conv_zscan__{ifov:0>3}--_set{iset}.pkl'
    gives that name from today's ifov.)"""
    p = "tests/examples/single/H1_TEST_set1/Conv_zscan__020.zarr"
    assert io.get_ifov(p) == 20 and io.get_iset(p) == 1
    assert io.output_name(p) == "drift_20--_set1.pkl"
    assert io.output_name(p, drift_save="drift_Conv_zscan__{ifov:0>3}--_set{iset}.pkl") == \
        "drift_Conv_zscan__020--_set1.pkl"
    assert io.output_name(p, 2) == "Conv_zscan__020--H1_TEST_set1--col2__Xhfits.npz"
    with pytest.raises(ValueError):
        io.get_ifov("a/b.npz")
    with pytest.raises(ValueError):
        io.get_iset("/a/b/c.zarr")


class _NoCupy(pickle.Unpickler):
    def find_class(self, module, name):
        assert not module.startswith("cupy"), "the pickle must not need CuPy"
        return super().find_class(module, name)


def _structure(obj):
    if isinstance(obj, (list, tuple)):
        return [type(obj).__name__] + [_structure(x) for x in obj]
    if isinstance(obj, np.ndarray):
        return "array"
    return type(obj).__name__


def test_drift_pickle_layout(tmp_path, layout, golden_dir):
    """drift_save (align.py:158-161) of drift()'s [drifts, files, ifov, ref_path]
    (align.py:163-176): the reference's nesting -- a list of (tzxyf, t+, t-,
    N+, N-) with three arrays and two ints, a list of folders, the FOV and the
    reference round's path -- readable without CuPy.  The values are the
    reference fixture's (decoded in drift_kat.json); the GPU test of drift()
    checks that drift() produces them."""
    kat = json.load(open(os.path.join(golden_dir, "drift_kat.json")))
    drifts = [(np.asarray(d[0]), np.asarray(d[1]), np.asarray(d[2]), int(d[3]), int(d[4])) for d in kat["drifts"]]
    data = [drifts, kat["files"], kat["ifov"], kat["ref_path"]]
    path = tmp_path / layout["drift"]["file"]
    align.drift_save(data, str(path))
    with open(path, "rb") as f:
        got = _NoCupy(f).load()
    assert _structure(got) == layout["drift"]["structure"]
    assert got[0][0][3:] == (621, 261)
