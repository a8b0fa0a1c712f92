"""The allocation-free maxima entry point (mm_find_local_maxima_noalloc).

It serves callers that cannot allocate device memory while they run -- code
inside another framework's memory pool or under a fixed memory budget, and
real-time loops that must not take cudaMalloc's implicit synchronisation.
It keeps its candidate list in a static device array of the library.  This
test calls it through the C ABI and checks its rows against the regular entry
point (mm_find_local_maxima) on two calls in a row with different volumes, so
that a stale count or candidate list left by the first call would show.  It
passes run alone in a fresh process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import ckernels as ck

pytestmark = pytest.mark.gpu

MAX_VOXELS = 1 << 21


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from mermake_gb300 import _lib
    return _lib


def volume(seed, shape):
    rng = np.random.default_rng(seed)
    im = rng.random(shape).astype(np.float32)
    im[rng.random(shape) < 0.03] = 0.7  # plateaus: tied neighbours are both maxima
    raw = rng.integers(0, 4000, shape).astype(np.int32)
    return torch.from_numpy(im).cuda(), torch.from_numpy(raw).to(torch.uint16).cuda()


def call(L, fn, img, raw, cap, th, delta, dfit, use_ctx):
    out = torch.zeros((cap, 8), dtype=torch.float32, device="cuda")
    n = C.c_uint32(0)
    args = [L.ptr(img), *img.shape, img.stride(0), img.stride(1), L.ptr(raw), 1, raw.stride(0), raw.stride(1),
            th, delta, dfit, 1.0, 1.5, 0.0, 0, L.ptr(out), cap, C.byref(n), L.stream_ptr()]
    rc = fn(L.ctx(), *args) if use_ctx else fn(*args)
    return rc, out[: n.value].cpu().numpy(), n.value


def test_noalloc_matches_regular_entry_point_twice(lib):
    L = lib.lib()
    cases = [(1, (12, 50, 60), 0.5, 1, 3), (2, (20, 64, 48), 0.55, 2, 2)]
    for seed, shape, th, delta, dfit in cases:
        img, raw = volume(seed, shape)
        rc0, want, n0 = call(lib, L.mm_find_local_maxima, img, raw, 1 << 15, th, delta, dfit, True)
        rc1, got, n1 = call(lib, L.mm_find_local_maxima_noalloc, img, raw, 1 << 15, th, delta, dfit, False)
        assert rc0 == 0 and rc1 == 0, lib.last_error()
        assert n1 == n0 > 100
        got, want = ck.match_rows(got, want)
        np.testing.assert_allclose(got, want, rtol=1e-6, atol=1e-6)


def test_noalloc_reports_overflow_and_rejects_large_volumes(lib):
    L = lib.lib()
    img, raw = volume(3, (10, 40, 40))
    rc, _, n = call(lib, L.mm_find_local_maxima_noalloc, img, raw, 4, 0.5, 1, 1, False)
    assert rc == lib.MM_EOVERFLOW and n > 4
    shape = (2, 1024, 1025)  # 2,099,200 voxels, each dimension valid
    assert np.prod(shape) > MAX_VOXELS
    big = torch.zeros(shape, device="cuda")
    rbig = torch.zeros(shape, dtype=torch.int32, device="cuda").to(torch.uint16)
    rc, _, _ = call(lib, L.mm_find_local_maxima_noalloc, big, rbig, 4, 0.5, 1, 1, False)
    assert rc == lib.MM_EINVAL
    assert "limit" in lib.last_error()


def test_noalloc_allocates_no_device_memory_after_first_call(lib):
    """The property the entry point exists for: once its first call on the
    device has loaded the device code and reserved the static array, further
    calls -- of other shapes and settings -- leave the device's free memory
    unchanged.  Inputs and outputs are allocated before the measurement."""
    L = lib.lib()
    cases = [(4, (12, 50, 60), 0.5, 1, 3), (5, (20, 64, 48), 0.55, 2, 2), (6, (8, 100, 90), 0.6, 3, 1)]
    prepared = []
    for seed, shape, th, delta, dfit in cases:
        img, raw = volume(seed, shape)
        out = torch.zeros((1 << 15, 8), dtype=torch.float32, device="cuda")
        prepared.append((img, raw, out, th, delta, dfit))

    def run(img, raw, out, th, delta, dfit):
        n = C.c_uint32(0)
        rc = L.mm_find_local_maxima_noalloc(lib.ptr(img), *img.shape, img.stride(0), img.stride(1), lib.ptr(raw), 1,
                                            raw.stride(0), raw.stride(1), th, delta, dfit, 1.0, 1.5, 0.0, 0,
                                            lib.ptr(out), out.shape[0], C.byref(n), lib.stream_ptr())
        assert rc == 0, lib.last_error()
        return n.value

    run(*prepared[0])  # first call: may load the module and reserve the array
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    counts = [run(*p) for p in prepared[1:]] + [run(*prepared[0])]
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert all(c > 0 for c in counts)
    assert free1 == free0, (free0, free1)
