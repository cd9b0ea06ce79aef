"""GPU parity of the texture layer, through the C ABI.

The scene is the textured room (raym0nade_gb300.scenes.textured_room):
diffuse, specular, emissive and normal-map textures with mip chains, uvs
wrapping outside [0, 1], alpha-tested cutouts including a stack of ten
layers past the reference's eight retries, an emissive-texture light object.

* Ray queries (rmn_trace_closest / rmn_trace_shadow) involve no
  transcendental function -- the alpha test reads level 0 -- so ids, t and
  occlusion answers must be identical to the oracle's (itself pinned to the
  reference built with its own src/material.cpp).
* Rendering: texel colours pass through powf(x, 2.2) and the level of detail
  through log2f, whose last bit may differ between CUDA and glibc. The
  G-buffer's geometry, material ids, opacity and specular-texture data are
  exact; base colour and surface normal agree to 1e-5; on the same random
  streams (oracle mode 1) nearly every pixel's radiance agrees to 1e-3.
* Statistically against the reference's own mt19937 stream (oracle mode 0).
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from raym0nade_gb300 import api, scenes  # noqa: E402
from tests.golden.make_golden import room_rays, scene_from  # noqa: E402
from tests.test_gpu_render import LUM, gpu_records, linear_image, _photo_np  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_textured_queries_match_oracle(port):
    room = scenes.textured_room()
    m = api.Model(room)
    ps = port.scene(room)
    rays = room_rays(200000, 71)
    f, t, b = api.split_hits(m.rayHit(torch.from_numpy(rays).cuda()))
    pf, pt, pb = ps.trace_closest(rays)
    assert np.array_equal(f, pf) and np.array_equal(t, pt)
    assert np.array_equal(b[pf >= 0], pb[pf >= 0])
    srays = room_rays(200000, 72, shadow=True)
    occ = m.rayHit_test(torch.from_numpy(srays).cuda()).cpu().numpy()
    assert np.array_equal(occ, ps.trace_shadow(srays))
    # the alpha test matters for these rays: without it (a t_min other than
    # eps takes the bare BVH query) some stop at a cut-away texel
    raw = rays.copy()
    raw[:, 3] = np.float32(1.5e-4)
    rf, _, _ = api.split_hits(m.rayHit(torch.from_numpy(raw).cuda()))
    assert (rf != f).sum() > 100


def test_textured_queries_golden():
    z = np.load(os.path.join(GOLDEN, "render_textured.npz"))
    m = api.Model(scene_from(z))
    f, t, b = api.split_hits(m.rayHit(torch.from_numpy(z["rays"]).cuda()))
    assert np.array_equal(f, z["face"]) and np.array_equal(t, z["t"])
    hit = f >= 0
    assert np.array_equal(b[hit], z["bary"][hit])
    occ = m.rayHit_test(torch.from_numpy(z["shadow_rays"]).cuda()).cpu().numpy()
    assert np.array_equal(occ, z["occluded"])


def compare_textured(gpu, ora, frac):
    # geometry, ids, opacity, eta, entering and the level-0 specular texture: exact
    for a, b in [(22, 25), (25, 28)]:
        assert np.array_equal(gpu[..., a:b], ora[..., a:b], equal_nan=True), (a, b)
    for k in (31, 32, 33, 35, 36, 37):
        assert np.array_equal(gpu[..., k], ora[..., k]), k
    hit = ~np.isnan(ora[..., 22])
    # base colour (powf), emission and surface normal (normal map at a
    # log2f level of detail): last-bit differences only
    for a, b in [(16, 19), (19, 22), (28, 31)]:
        np.testing.assert_allclose(gpu[..., a:b][hit], ora[..., a:b][hit], rtol=1e-5, atol=1e-6)
    li, lo = linear_image(gpu), linear_image(ora)
    close = np.isclose(li, lo, rtol=1e-3, atol=1e-5).all(-1)
    assert close.mean() >= frac, f"only {close.mean():.4f} of pixels agree"
    assert abs(li.mean() - lo.mean()) <= 5e-3 * abs(lo.mean()) + 1e-6
    return close.mean()


@pytest.mark.parametrize("sky,spp,p_direct", [(True, 16, 0.7), (False, 12, 0.7), (True, 6, 0.0)])
def test_textured_paths_match_oracle(port, sky, spp, p_direct):
    room = scenes.textured_room(sky=sky)
    cam = scenes.textured_camera(96, 64, spp, p_direct=p_direct)
    g, _ = gpu_records(api.Model(room), cam, seed=19)
    o = port.scene(room).render(cam, seed=19, mode=1)
    assert set(np.unique(o[..., 36]).astype(int)) == set(range(6))
    compare_textured(g, o, frac=0.95)


def test_textured_mean_matches_reference_stream(port):
    """The GPU's counter streams against the reference's own mt19937 stream
    (the oracle in mode 0): mean luminance within 2 %."""
    room = scenes.textured_room()
    cam = scenes.textured_camera(48, 32, 256)
    g, _ = gpu_records(api.Model(room), cam, seed=29)
    o = port.scene(room).render(cam, seed=29, mode=0)
    lg, lo = linear_image(g) @ LUM, linear_image(o) @ LUM
    assert abs(lg.mean() - lo.mean()) <= 0.02 * lo.mean()


def test_textured_scene_info_and_errors():
    room = scenes.textured_room(sky=False)
    info = api.Model(room).info()
    assert info["num_lights"] == 1
    bad = scenes.textured_room()
    bad.textures = list(bad.textures)
    bad.textures[0] = bad.textures[0][..., :3].copy()  # RGB: not accepted
    with pytest.raises(AssertionError):
        bad.check()
    bad.check = lambda: None  # hand the RGB texture to the library anyway
    with pytest.raises(api.RmnError) as e:
        api.Model(bad)
    assert e.value.status == 4 and "channels" in str(e.value)
    bad2 = scenes.textured_room()
    bad2.mat_tex = bad2.mat_tex.copy()
    bad2.mat_tex[1, 0] = 99
    bad2.check = lambda: None
    with pytest.raises(api.RmnError) as e:
        api.Model(bad2)
    assert e.value.status == 1


def test_textured_batch_equals_individual_renders():
    room = api.Model(scenes.textured_room())
    cor = api.Model(scenes.cornell())
    specs = [(room, scenes.textured_camera(40, 24, 8), 3), (cor, scenes.cornell_camera(24, 24, 8), 4),
             (room, scenes.textured_camera(31, 17, 5, max_depth=6), 5)]
    items, solo = [], []
    for m, cam, seed in specs:
        a = api.RenderArgs.from_camera(cam, seed=seed)
        items.append((m, a, api.Photo(cam.width, cam.height)))
        solo.append(_photo_np(api.render(m, a)))
    b = api.Batch(items, use_graph=True)
    b.render()
    torch.cuda.synchronize()
    for (m, a, ph), ref in zip(items, solo):
        for x, y in zip(_photo_np(ph), ref):
            assert np.array_equal(x, y, equal_nan=True)


def test_adjoint_rejects_textured_scenes():
    room = api.Model(scenes.textured_room())
    cam = scenes.textured_camera(16, 16, 4)
    args = api.RenderArgs.from_camera(cam, seed=1)
    photo = api.render(room, args)
    with pytest.raises(api.RmnError) as e:
        api.adjoint(room, args, photo, torch.ones(16 * 16, 3, device="cuda"))
    assert e.value.status == 4


def test_mip_chains_match_oracle():
    """The device-built chains (rmn_scene_texture_get) level for level
    against ImageData::generateMipmaps restated in numpy, for the room's
    textures and for odd, thin and long sizes (depths 1 to 8)."""
    from oracle.image_codecs import mip_chain
    room = scenes.textured_room()
    rng = np.random.default_rng(12)
    extra = [rng.integers(0, 256, (h, w, 4)).astype(np.uint8)
             for h, w in [(21, 37), (1, 64), (3, 300), (16, 2048), (255, 257), (1, 1), (600, 5)]]
    room.textures = list(room.textures) + extra
    m = api.Model(room)
    for i, tex in enumerate(room.textures):
        want = mip_chain(tex)
        for level, w in enumerate(want):
            assert np.array_equal(m.texture(i, level), w), (i, level)
        with pytest.raises(api.RmnError):
            m.texture(i, len(want))
    with pytest.raises(api.RmnError):
        m.texture(len(room.textures), 0)
