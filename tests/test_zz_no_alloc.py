"""rmn_compose_noalloc: the composite + gamma + FXAA pass without device
allocation, for callers that cannot allocate device memory (their device
memory is owned by their own arena allocator, or their frame loop must not
let cudaMalloc/cudaFree synchronise the device). Its intermediate image lives
in a fixed device array of RMN_NOALLOC_MAX_PIXELS pixels.

Checked through the C ABI against rmn_compose, the allocating entry point,
on two calls in a row (the shared array keeps the previous call's contents),
and checked to allocate nothing: after a first call (which loads the array's
module), further calls leave the device's free memory and the stream-ordered
allocator's default pool unchanged. This file is collected last on purpose.
"""
import ctypes
import glob
import os

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


def _cudart():
    """The CUDA runtime torch loaded (for the default memory pool's counters),
    or None."""
    import torch.cuda
    names = ["libcudart.so.13", "libcudart.so.12", "libcudart.so"]
    here = os.path.dirname(torch.__file__)
    names += glob.glob(os.path.join(here, "..", "nvidia", "cu*", "lib", "libcudart.so*"))
    names += glob.glob(os.path.join(here, "..", "nvidia", "cuda_runtime", "lib", "libcudart.so*"))
    for n in names:
        try:
            return ctypes.CDLL(n)
        except OSError:
            continue
    return None


def _pool_counters(rt):
    """(reserved, used) bytes of the current device's default memory pool."""
    if rt is None:
        return None
    dev = ctypes.c_int()
    pool = ctypes.c_void_p()
    if rt.cudaGetDevice(ctypes.byref(dev)) or rt.cudaDeviceGetDefaultMemPool(ctypes.byref(pool), dev):
        return None
    out = []
    for attr in (5, 7):  # cudaMemPoolAttrReservedMemCurrent, cudaMemPoolAttrUsedMemCurrent
        v = ctypes.c_uint64()
        if rt.cudaMemPoolGetAttribute(pool, attr, ctypes.byref(v)):
            return None
        out.append(v.value)
    return tuple(out)


def test_compose_noalloc_allocates_nothing():
    """1920 x 1080 with FXAA (near the 2^21-pixel limit): once the first call
    has run, two more calls change neither the device's free memory nor the
    default memory pool's reserved and used bytes."""
    lib = _lib.load()
    w, h = 1920, 1080
    opts = api.Full | api.GAMMA | api.DoFXAA
    ph = _photo(w, h, 11)
    out = torch.empty((h, w, 3), device="cuda")
    img = ph.c_image()
    call = lambda: lib.rmn_compose_noalloc(ctypes.byref(img), w, h, 1.0, opts, ctypes.c_void_p(out.data_ptr()), None)
    assert call() == 0, lib.rmn_last_error()
    torch.cuda.synchronize()
    rt = _cudart()
    free0, pool0 = torch.cuda.mem_get_info()[0], _pool_counters(rt)
    for _ in range(2):
        assert call() == 0, lib.rmn_last_error()
    torch.cuda.synchronize()
    free1, pool1 = torch.cuda.mem_get_info()[0], _pool_counters(rt)
    assert free1 == free0
    assert pool1 == pool0
    # after rmn_release_cached_memory the address is resolved again
    assert lib.rmn_release_cached_memory() == 0
    assert call() == 0, lib.rmn_last_error()
    np.testing.assert_allclose(out.cpu().numpy(), ph.shade(opts).cpu().numpy(), rtol=2e-6, atol=1e-7)


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
