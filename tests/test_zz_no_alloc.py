"""rmn_compose_noalloc: the composite + gamma + FXAA pass without device
allocation, for callers that cannot allocate device memory (their device
memory is owned by their own arena allocator, or their frame loop must not
let cudaMalloc/cudaFree synchronise the device). Its intermediate image lives
in a fixed device array of RMN_NOALLOC_MAX_PIXELS pixels.

Checked through the C ABI against rmn_compose, the allocating entry point,
on two calls in a row (the shared array keeps the previous call's contents).
This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from raym0nade_gb300 import _lib, api  # noqa: E402

MAX_PIXELS = 1 << 21


def _photo(w, h, seed):
    rng = np.random.default_rng(seed)
    ph = api.Photo(w, h)
    n = w * h
    for k in ("radiance_Dd", "radiance_Ds", "radiance_Id", "radiance_Is"):
        getattr(ph, k).copy_(torch.from_numpy((rng.random((n, 4), dtype=np.float32) ** 2) * 1.5))
    g = rng.random((n, api.GBUFFER_FLOATS), dtype=np.float32)
    g[::7, 6] = np.nan  # some primary misses
    ph.Gbuffer.copy_(torch.from_numpy(g))
    return ph


@pytest.mark.parametrize("w,h,opts", [(640, 360, api.Full | api.GAMMA | api.DoFXAA), (1920, 1080, api.Full | api.GAMMA | api.DoFXAA),
                                      (97, 61, api.Full | api.GAMMA)])
def test_compose_noalloc_matches_compose(w, h, opts):
    lib = _lib.load()
    for call, seed in enumerate((1, 2)):  # two calls in a row, different inputs
        ph = _photo(w, h, seed + w)
        ref = ph.shade(opts).cpu().numpy()
        out = torch.full((h, w, 3), -1.0, device="cuda")
        img = ph.c_image()
        st = lib.rmn_compose_noalloc(ctypes.byref(img), w, h, 1.0, opts, ctypes.c_void_p(out.data_ptr()), None)
        assert st == 0, lib.rmn_last_error()
        np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=2e-6, atol=1e-7)


def test_compose_noalloc_limits():
    lib = _lib.load()
    ph = _photo(8, 8, 3)
    img = ph.c_image()
    out = torch.empty((8, 8, 3), device="cuda")
    # beyond the fixed scratch
    st = lib.rmn_compose_noalloc(ctypes.byref(img), 2049, 1024, 1.0, api.Full | api.DoFXAA,
                                 ctypes.c_void_p(out.data_ptr()), None)
    assert st == 1 and b"scratch" in lib.rmn_last_error()
    # host buffers would need staging allocations: rejected
    host = np.empty((8, 8, 3), np.float32)
    st = lib.rmn_compose_noalloc(ctypes.byref(img), 8, 8, 1.0, api.Full, ctypes.c_void_p(host.ctypes.data), None)
    assert st == 1 and b"device memory" in lib.rmn_last_error()
