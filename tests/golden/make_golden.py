"""Regenerate the golden fixtures in this folder from the reference's own test data.

Run from the repository root in a checkout that has the reference mounted:

    python tests/golden/make_golden.py /path/to/MERMAKE

It reads (never writes) the reference tree and produces:

deconv_tiles.npz
    Input crops of the reference FOV fixture
    (``tests/examples/single/H1_TEST_set1``, colour 0, stored as the uint8 the
    zarr holds; the image is ``uint16(u8)**2`` as ``mermake/io.py:read_im``
    makes it) together with the reference's golden float16 deconvolution
    (``tests/examples/single/out/deconv.{ts}.{z}.npz``) over the output region
    each crop's tile writes, at every 5th z plane.  Each crop is exactly the
    input one tile reads (``Deconvolver.tiled``, deconvolver.py:186-206), so the
    tile can be recomputed alone.
psf_750.npz
    The reference PSF fixture ``tests/examples/psf_750_Scope0_final.npy``.
dapi_features.npz
    ``Xh_plus`` / ``Xh_minus`` from ``...--dapiFeatures.npz`` (drift input).
drift_kat.json
    The drift pickle ``drift_Conv_zscan__020--_set1.pkl`` decoded without CuPy:
    the self-alignment of the dapiFeatures fixture (t = 0, N+ = 621, N- = 261).
output_layout.json
    The layout of the reference's output files in ``tests/examples/single/out``:
    for each ``.npz`` its name, keys, dtypes and shapes and the ``args`` table;
    for the drift ``.pkl`` the types of its nested structure; and the settings
    the ``args`` table was written from, as TOML text (values typed back from
    their ``str`` form).
"""
import ast
import bz2
import json
import os
import pickle
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# (tile_size, tile origin x, tile origin y): the reflect-in corner and the
# reflect-out corner of the 1200x1200 FOV at tile 300, and the thin reflect-out
# corner tile at tile 500 (xd = yd = 289).
TILES = [(300, 0, 0), (300, 900, 900), (500, 1000, 1000)]
OVERLAP = 89
ZSTEP = 5


def read_zarr_u8(folder):
    """Minimal zarr-v2 reader for the fixture (bz2 chunks of one frame each,
    missing chunks are fill_value); frame 0 is dropped and the frames are split
    into 3 channels as mermake/io.py:116-146 does."""
    d = os.path.join(folder, "020", "data")
    meta = json.load(open(os.path.join(d, ".zarray")))
    n, X, Y = meta["shape"]
    frames = []
    for i in range(n):
        f = os.path.join(d, f"{i}.0.0")
        if os.path.exists(f):
            frames.append(np.frombuffer(bz2.decompress(open(f, "rb").read()), np.uint8).reshape(X, Y))
        else:
            frames.append(np.full((X, Y), meta["fill_value"], np.uint8))
    im = np.stack(frames)[1:]
    nch = 3  # <z_offsets> of the fixture's xml ends in ':3'
    nzs = (im.shape[0] // nch) * nch
    im = im[:nzs].reshape(im.shape[0] // nch, nch, X, Y).swapaxes(0, 1)
    return im


class _CupyFree(pickle.Unpickler):
    def find_class(self, module, name):
        if module.startswith("cupy"):
            return np.array
        return super().find_class(module, name)


def main(ref):
    ex = os.path.join(ref, "tests", "examples")
    im = read_zarr_u8(os.path.join(ex, "single", "H1_TEST_set1"))[0]
    Z, X, Y = im.shape
    out = {}
    for k, (ts, x, y) in enumerate(TILES):
        x0, x1 = max(x - OVERLAP, 0), min(x + ts + OVERLAP, X)
        y0, y1 = max(y - OVERLAP, 0), min(y + ts + OVERLAP, Y)
        xo1, yo1 = min(x + ts, X), min(y + ts, Y)
        zs = np.arange(0, Z, ZSTEP)
        gold = np.stack([np.load(os.path.join(ex, "single", "out", f"deconv.{ts}.{z}.npz"))["arr_0"][x:xo1, y:yo1]
                         for z in zs])
        out[f"t{k}_crop_u8"] = np.ascontiguousarray(im[:, x0:x1, y0:y1])
        out[f"t{k}_golden_f16"] = gold
        out[f"t{k}_meta"] = np.array([ts, x, y, x0, x1, y0, y1, X, Y, Z, OVERLAP, ZSTEP], np.int64)
    np.savez_compressed(os.path.join(HERE, "deconv_tiles.npz"), **out)

    psf = np.load(os.path.join(ex, "psf_750_Scope0_final.npy"))
    np.savez_compressed(os.path.join(HERE, "psf_750.npz"), psf=psf)

    d = np.load(os.path.join(ex, "single", "out", "Conv_zscan__020--H1_TEST_set1--dapiFeatures.npz"))
    np.savez_compressed(os.path.join(HERE, "dapi_features.npz"), Xh_plus=d["Xh_plus"], Xh_minus=d["Xh_minus"])

    with open(os.path.join(ex, "single", "out", "drift_Conv_zscan__020--_set1.pkl"), "rb") as f:
        drifts, files, ifov, refpath = _CupyFree(f).load()
    kat = {"drifts": [[np.asarray(t).tolist() for t in d[:3]] + [int(d[3]), int(d[4])] for d in drifts],
           "files": files, "ifov": ifov, "ref_path": refpath}
    with open(os.path.join(HERE, "drift_kat.json"), "w") as f:
        json.dump(kat, f, indent=1)


def _toml_value(v):
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, (int, float)):
        return repr(v)
    if isinstance(v, list):
        return "[" + ", ".join(_toml_value(x) for x in v) + "]"
    # literal strings (no escapes), triple-quoted where the value holds a quote
    return ("'''" + v + "'''") if "'" in v else ("'" + v + "'")


def _typed(text):
    try:
        v = ast.literal_eval(text)
    except (ValueError, SyntaxError):
        return text
    return v if isinstance(v, (bool, int, float, list)) and str(v) == text else text


def _structure(obj):
    if isinstance(obj, (list, tuple)):
        return [type(obj).__name__] + [_structure(x) for x in obj]
    if isinstance(obj, np.ndarray):
        return "array"
    return type(obj).__name__


def output_layout(ref):
    out_dir = os.path.join(ref, "tests", "examples", "single", "out")
    lay = {}
    for kind, name in (("hyb", "Conv_zscan__020--H1_TEST_set1--col0__Xhfits.npz"),
                       ("dapi", "Conv_zscan__020--H1_TEST_set1--dapiFeatures.npz")):
        d = np.load(os.path.join(out_dir, name))
        lay[kind] = {"file": name, "keys": {k: [d[k].dtype.str, list(d[k].shape)] for k in d.files},
                     "version": str(d["version"])}
        args = d["args"].tolist()
        lay["args"] = args
    blocks = {}
    for block, key, val in lay["args"]:
        blocks.setdefault(block, {})[key] = _typed(val)
    lay["settings_toml"] = "\n".join(
        "[%s]\n" % b + "".join("%s = %s\n" % (k, _toml_value(v)) for k, v in kv.items()) for b, kv in blocks.items())
    name = "drift_Conv_zscan__020--_set1.pkl"
    with open(os.path.join(out_dir, name), "rb") as f:
        obj = _CupyFree(f).load()
    lay["drift"] = {"file": name, "structure": _structure(obj)}
    with open(os.path.join(HERE, "output_layout.json"), "w") as f:
        json.dump(lay, f, indent=1)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MERMAKE_REF", "/root/reference")
    main(ref)
    output_layout(ref)
