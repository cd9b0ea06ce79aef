"""GPU parity of Photo's post passes (spatialClamp, filter, bloom, depth of
field, postProcessing, the export set), through the C ABI.

The oracle (oracle/port, pinned bit for bit to the reference's own
src/image.cpp) runs the same passes on the same records. Passes without
transcendental functions -- spatialClamp and the depth-of-field blur -- must
be bit-identical; bloom (powf), the filter's edge-stopping weight (powf,
expf) and gamma (tanhf, powf) use CUDA's functions, whose last bit may differ
from glibc's, so their images are compared within a relative 1e-4 on nearly
every value.
"""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from raym0nade_gb300 import api, scenes  # noqa: E402
from tests.golden.make_golden import PHOTO_POST, photo_records  # noqa: E402

GB_FROM_REC = [16, 17, 18, 19, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31, 32, 33, 35, 36, 37]


def photo_from_records(rec, post=PHOTO_POST, device=True):
    h, w = rec.shape[:2]
    ph = api.Photo(w, h, post["exposure"], device=device)
    r = rec.reshape(-1, 40)
    conv = (lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()) if device else np.ascontiguousarray
    ph.radiance_Dd, ph.radiance_Ds = conv(r[:, 0:4]), conv(r[:, 4:8])
    ph.radiance_Id, ph.radiance_Is = conv(r[:, 8:12]), conv(r[:, 12:16])
    ph.Gbuffer = conv(r[:, GB_FROM_REC])
    ph.focus, ph.CoC, ph.cameraPosition = post["focus"], post["coc"], post["camera"]
    return ph


def radiance(ph):
    t = lambda x: x.cpu().numpy() if isinstance(x, torch.Tensor) else x
    return np.concatenate([t(ph.radiance_Dd), t(ph.radiance_Ds), t(ph.radiance_Id), t(ph.radiance_Is)], 1)


def np_(x):
    return x.cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x)


def close_frac(a, b, rtol=1e-4, atol=1e-6):
    return np.isclose(a, b, rtol=rtol, atol=atol, equal_nan=True).mean()


def render_records(port):
    """A Cornell render from inside the box (every pixel a hit), as records."""
    w, h = 48, 32
    acc = math.tan(math.radians(30.0)) / (w / 2.0)
    cam = scenes.Camera((0.5, 0.5, 0.3), (0.0, 0.0, 1.0), (0.0, -1.0, 0.0), (-1.0, 0.0, 0.0), acc, w, h, 16)
    return port.scene(scenes.cornell()).render(cam, seed=5, mode=1)


@pytest.mark.parametrize("which", ["synthetic", "render"])
def test_spatial_clamp_bit_exact(port, which):
    rec = photo_records(96, 64, 11) if which == "synthetic" else render_records(port)
    ph = photo_from_records(rec)
    ph.spatialClamp()
    ref, _ = port.photo(rec, 1)
    assert np.array_equal(radiance(ph), ref.reshape(-1, 40)[:, :16])


def test_filter_matches_oracle(port):
    rec = photo_records(96, 64, 12, miss=0.05)
    ph = photo_from_records(rec)
    ph.filter()
    ref, _ = port.photo(rec, 2)
    got, want = radiance(ph), ref.reshape(-1, 40)[:, :16]
    assert close_frac(got, want) >= 0.999
    assert np.nanmax(np.abs(got - want) / (np.abs(want) + 1e-3)) < 1e-2
    assert np.abs(got[:, 8:11] - rec.reshape(-1, 40)[:, 8:11]).mean() > 0.01  # it did filter


def test_bloom_matches_oracle(port):
    rec = photo_records(96, 64, 13)
    ph = photo_from_records(rec)
    got = np_(ph.post_process(api.Full | api.DoBloom))
    _, want = port.photo(rec, 8, api.Full | api.DoBloom, **PHOTO_POST)
    assert close_frac(got, want, rtol=1e-5) >= 0.999
    _, plain = port.photo(rec, 8, api.Full, **PHOTO_POST)
    assert (got - plain).max() > 0.1


@pytest.mark.parametrize("coc,miss", [(8.0, 0.0), (40.0, 0.0), (8.0, 0.1)])
def test_depth_of_field_bit_exact(port, coc, miss):
    """The gather in the reference's scatter order: bit-identical, also
    with a radius above the 8-pixel minimum tile and with pixels without a
    hit (NaN depth)."""
    rec = photo_records(80, 56, 14, miss=miss)
    post = dict(PHOTO_POST, coc=coc)
    ph = photo_from_records(rec, post)
    got = np_(ph.post_process(api.Full | api.DoDepthFieldBlur))
    _, want = port.photo(rec, 8, api.Full | api.DoDepthFieldBlur, **post)
    assert np.array_equal(got, want, equal_nan=True)
    _, plain = port.photo(rec, 8, api.Full, **post)
    assert np.nanmean(np.abs(got - plain)) > 0.01


def test_post_processing_full_chain(port):
    rec = photo_records(96, 64, 15)
    opts = api.Full | api.DoDepthFieldBlur | api.DoBloom | api.DoFXAA
    for device in (True, False):
        ph = photo_from_records(rec, device=device)
        got = np_(ph.postProcessing(opts))
        _, want = port.photo(rec, 4, opts, **PHOTO_POST)
        assert close_frac(got, want) >= 0.99


def test_export_set_matches_oracle_sequence(port):
    """rmn_export_set against the reference's export sequence run by the
    oracle (postProcessing per export, spatialClamp after export 3, filter
    after export 11, the depth-of-field exports when CoC > eps)."""
    rec = render_records(port)
    post = dict(exposure=1.0, focus=0.5, coc=6.0, camera=(0.5, 0.5, 0.3))
    ph = photo_from_records(rec, post)
    out = ph.export_set()
    assert len(out) == api.EXPORTS + api.EXPORTS_DOF
    lib = api._lib.load()
    r = rec
    for k in range(api.EXPORTS + api.EXPORTS_DOF):
        if k == 4:
            r, _ = port.photo(r, 1)
        if k == 12:
            r, _ = port.photo(r, 2)
        _, want = port.photo(r, 4, lib.rmn_export_options(k) & ~api.GAMMA, **post)
        tag = lib.rmn_export_tag(k).decode()
        assert close_frac(np_(out[tag]), want) >= 0.99, tag
    # the buffers were clamped and filtered on the way, as in the reference
    assert close_frac(radiance(ph), r.reshape(-1, 40)[:, :16]) >= 0.999
    ph2 = photo_from_records(rec, dict(post, coc=0.0))
    assert len(ph2.export_set()) == api.EXPORTS


def test_render_multithread_writes_the_export_set(tmp_path):
    """The render_multiThread mirror: a render, then the reference's 25
    exports (depth of field on) as PNG files named savePath(tag).png."""
    from tests.test_library import _read_png
    cam = scenes.cornell_camera(32, 24, 8)
    a = api.RenderArgs.from_camera(cam, seed=2, savePath=str(tmp_path / "out" / "img"))
    a.focus, a.CoC = 1.5, 2.0
    api.render_multiThread(api.Model(scenes.cornell()), a)
    lib = api._lib.load()
    for k in range(api.EXPORTS + api.EXPORTS_DOF):
        tag = lib.rmn_export_tag(k).decode()
        img = _read_png(str(tmp_path / "out" / f"img({tag}).png"))
        assert img.shape == (24, 32, 3)
