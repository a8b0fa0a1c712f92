"""The serving form (mermake_gb300.serve): every result is the same alone and in
a mix of concurrent requests, admission respects the HBM budget, and later
rounds are drift-aligned against round 0 of their FOV."""
import numpy as np
import pytest
import torch

from oracle import ckernels as ck

pytestmark = pytest.mark.gpu

HYB = dict(tile_size=60, overlap=12, beta=1e-4, threshold=3600, blur_radius=10, delta=1, delta_fit=3,
           sigmaZ=1, sigmaXY=1.5)
DAPI = dict(tile_size=60, overlap=12, beta=0.01, threshold=3.0, blur_radius=20, delta=5, delta_fit=5,
            sigmaZ=1, sigmaXY=1.5)
SHAPES = {0: (10, 130, 120), 1: (8, 100, 150)}


@pytest.fixture(scope="module")
def mm():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mermake_gb300 import serve, synth
    return dict(serve=serve, synth=synth)


def requests(mm, n=6):
    synth = mm["synth"]
    out = []
    for i in range(n):
        fov, rnd = i % 2, i // 2
        Z, X, Y = SHAPES[fov]
        # sparse nuclei: after the RMS normalisation their maxima exceed the
        # drift threshold of 4 (a field filled to 7 % would top out near 3.9)
        dapi = synth.dapi_stack(Z, X, Y, 100 + fov, n_nuclei=6, radii=(2.0, 6.0, 6.0))
        if rnd:  # a known integer drift of the whole stack
            dapi = torch.roll(dapi, shifts=(0, 2 * rnd, -rnd), dims=(0, 1, 2))
        cols = [synth.hyb_stack(Z, X, Y, 250, 10 * i + c, gain=synth.flat_gain(X, Y)) for c in range(1 + i % 2)]
        flats = [torch.from_numpy(synth.flat_gain(X, Y)) for _ in cols]
        out.append(dict(fov=fov, round=rnd, dapi=dapi.pin_memory(), colours=[c.pin_memory() for c in cols],
                        flats=flats))
    return out


def run(mm, reqs, workers, budget, together):
    serve = mm["serve"]
    psf = mm["synth"].gaussian_psf((9, 9, 9), 2.0, 1.3)
    with serve.FovServer(psf, HYB, DAPI, hbm_budget=budget, workers=workers) as srv:
        if together:
            futs = [srv.submit(serve.FovRequest(**r)) for r in reqs]
            res = [f.result(timeout=600) for f in futs]
        else:
            res = [srv.submit(serve.FovRequest(**r)).result(timeout=600) for r in reqs]
        return res, srv.max_in_flight


def same(a, b):
    np.testing.assert_array_equal(ck.sort_rows(a.xh_plus), ck.sort_rows(b.xh_plus))
    np.testing.assert_array_equal(ck.sort_rows(a.xh_minus), ck.sort_rows(b.xh_minus))
    assert len(a.xh) == len(b.xh)
    for x, y in zip(a.xh, b.xh):
        np.testing.assert_array_equal(ck.sort_rows(x), ck.sort_rows(y))
    if a.drift is None:
        assert b.drift is None
    else:
        for u, v in zip(a.drift, b.drift):
            np.testing.assert_array_equal(np.asarray(u), np.asarray(v))


def test_same_alone_and_in_the_mix(mm):
    reqs = requests(mm)
    alone, _ = run(mm, reqs, workers=1, budget=1e12, together=False)
    mixed, peak = run(mm, reqs, workers=3, budget=1e12, together=True)
    assert peak >= 2  # requests really overlapped
    for a, b in zip(alone, mixed):
        same(a, b)
    for r in alone:
        assert len(r.xh_plus) > 0 and all(len(x) > 0 for x in r.xh)


def test_drift_against_round_zero(mm):
    reqs = requests(mm)
    res, _ = run(mm, reqs, workers=2, budget=1e12, together=True)
    for r in res:
        if r.request.round == 0:
            assert r.drift is None
        else:
            tzxyf = np.asarray(r.drift[0])
            assert r.drift[3] + r.drift[4] > 0  # matched points
            np.testing.assert_allclose(tzxyf, [0.0, -2.0 * r.request.round, 1.0 * r.request.round], atol=0.5)


def test_admission_respects_budget(mm):
    reqs = requests(mm, n=4)
    serve = mm["serve"]
    psf = mm["synth"].gaussian_psf((9, 9, 9), 2.0, 1.3)
    with serve.FovServer(psf, HYB, DAPI, hbm_budget=1.0, workers=3) as srv:
        futs = [srv.submit(serve.FovRequest(**r)) for r in reqs]
        for f in futs:
            f.result(timeout=600)
        assert srv.max_in_flight == 1  # nothing fits beside a running request


def test_device_memory_stays_within_budget(mm):
    """Admission is checked against the memory actually held -- torch's
    reserved memory (spectra, worker buffers, cached outputs) plus every
    worker's library scratch -- plus the growth reserved for requests in
    flight.  With room for the resident spectra and about one request, three
    workers run the requests one or two at a time, idle workers give their
    memory back when it is needed, the held total never exceeds the budget,
    and the results equal those of an unconstrained server."""
    reqs = requests(mm, n=6)
    serve = mm["serve"]
    psf = mm["synth"].gaussian_psf((9, 9, 9), 2.0, 1.3)
    free, _ = run(mm, reqs, workers=1, budget=1e12, together=False)
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    torch.cuda.reset_peak_memory_stats()
    base = torch.cuda.memory_reserved()
    with serve.FovServer(psf, HYB, DAPI, hbm_budget=1e12, workers=3) as srv:
        one = max(sum(srv._est(serve.FovRequest(**r))) for r in reqs)
        spectra = sum(srv._spectra_bytes(s) for s in SHAPES.values())
        srv.budget = base + spectra + 1.3 * one
        futs = [srv.submit(serve.FovRequest(**r)) for r in reqs]
        res = [f.result(timeout=600) for f in futs]
        budget, peak = srv.budget, srv.peak_bytes
    print("budget %.1f MB over the base, peak held %.1f MB, torch peak %.1f MB"
          % ((budget - base) / 1e6, (peak - base) / 1e6, (torch.cuda.max_memory_reserved() - base) / 1e6))
    assert peak <= budget
    assert torch.cuda.max_memory_reserved() <= budget
    for a, b in zip(free, res):
        same(a, b)
