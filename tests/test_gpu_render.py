"""GPU integrator parity, through the C ABI (rmn_render).

Three levels:
* per path -- the oracle re-runs the reference's estimator on the library's
  counter-based random streams (oracle mode 1), so both sides draw the same
  numbers: the G-buffer must be bit-identical and nearly every pixel's
  radiance must agree to 1e-3 (a path can still branch differently where
  CUDA's and glibc's sinf/cosf/powf/logf differ in the last bit);
* invariance -- the lane split of a pixel's samples (lanes_per_pixel) must
  not change the result beyond float summation order (rtol 1e-4);
* converged -- the reference's own renderer at 4096 spp, two independent
  renders per case (tests/golden/converged_<case>.npz, made from the
  compiled reference): the Cornell workload, a heightfield under the sun in
  sky mode, the glass Cornell box. The GPU at 4096 spp must sit within the
  reference's own noise floor (full-resolution relative MSE against the
  reference at most 1.1x the reference against itself), show no bias
  (z-scores of the per-pixel difference, with a variance from independent
  GPU renders), match mean luminance within 0.5%, and meet relative MSE
  <= 1e-3 on 4x4-binned images.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from raym0nade_gb300 import api, scenes  # noqa: E402
from tests.golden.make_golden import CONVERGED_CASES, converged_case  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
LUM = np.array([0.3, 0.6, 0.1], np.float32)


def gpu_records(model, cam, seed, lanes=0, host=False):
    args = api.RenderArgs.from_camera(cam, seed=seed, lanes_per_pixel=lanes)
    photo = api.Photo(cam.width, cam.height, cam.exposure, device=not host)
    api.render(model, args, photo)
    t = lambda x: x.cpu().numpy() if isinstance(x, torch.Tensor) else x
    g = t(photo.Gbuffer)
    rec = np.zeros((cam.height * cam.width, 40), np.float32)
    rec[:, 0:4], rec[:, 4:8] = t(photo.radiance_Dd), t(photo.radiance_Ds)
    rec[:, 8:12], rec[:, 12:16] = t(photo.radiance_Id), t(photo.radiance_Is)
    rec[:, 16:31] = g[:, 0:15]
    rec[:, 31], rec[:, 32], rec[:, 33], rec[:, 35], rec[:, 36] = g[:, 15], g[:, 16], g[:, 17], g[:, 18], g[:, 19]
    rec[:, 37] = g[:, 20]
    return rec.reshape(cam.height, cam.width, 40), photo


def linear_image(rec):
    rd = rec[..., 0:3] + rec[..., 8:11]
    rs = rec[..., 4:7] + rec[..., 12:15]
    return rec[..., 16:19] * rd + rs + rec[..., 19:22]


def compare_paths(gpu, ora, frac=0.98):
    # G-buffer: primary hit and shading are float-exact; the emission of a
    # miss pixel is SkyBox::get, whose atan2f/acosf/sinf may differ from
    # glibc's in the last bit (and, at a texel boundary, pick the neighbour)
    for a, b in [(16, 19), (22, 25), (25, 28), (28, 31)]:
        assert np.array_equal(gpu[..., a:b], ora[..., a:b], equal_nan=True), (a, b)
    assert np.array_equal(gpu[..., 31:34], ora[..., 31:34])
    assert np.array_equal(gpu[..., 35:38], ora[..., 35:38])  # eta, material id, entering
    hit = ~np.isnan(ora[..., 22])
    assert np.array_equal(gpu[..., 19:22][hit], ora[..., 19:22][hit])
    em = np.isclose(gpu[..., 19:22], ora[..., 19:22], rtol=1e-5, atol=0).all(-1)
    assert em.mean() >= 0.99
    li, lo = linear_image(gpu), linear_image(ora)
    close = np.isclose(li, lo, rtol=1e-3, atol=1e-5).all(-1)
    assert close.mean() >= frac, f"only {close.mean():.4f} of pixels agree"
    assert abs(li.mean() - lo.mean()) <= 5e-3 * abs(lo.mean()) + 1e-6
    return close.mean()


@pytest.mark.parametrize("maxd", [16, 8])
def test_cornell_paths_match_oracle(port, maxd):
    c = scenes.cornell()
    cam = scenes.cornell_camera(48, 48, 16, max_depth=maxd)
    g, _ = gpu_records(api.Model(c), cam, seed=11)
    o = port.scene(c).render(cam, seed=11, mode=1)
    compare_paths(g, o)


def test_sky_paths_match_oracle(port):
    hf = scenes.heightfield(40, seed=9, extent=4.0, patch=8)
    hf.env = scenes.sky_env(128, 64, sun_radiance=500.0, sun_diameter_deg=6.0)
    cam = scenes.Camera((0.3, 2.0, -0.8), (0.35, -0.45, 0.82), (0.0, -1.0, 0.0), (-1.0, 0.0, 0.0), 0.03, 40, 30, 12)
    g, _ = gpu_records(api.Model(hf), cam, seed=5)
    o = port.scene(hf).render(cam, seed=5, mode=1)
    compare_paths(g, o)


@pytest.mark.parametrize("spp,p_direct", [(1, 0.7), (5, 0.0), (4, 1.0), (33, 0.5)])
def test_sample_splits(port, spp, p_direct):
    c = scenes.cornell()
    cam = scenes.cornell_camera(24, 24, spp, p_direct=p_direct)
    g, _ = gpu_records(api.Model(c), cam, seed=3)
    o = port.scene(c).render(cam, seed=3, mode=1)
    compare_paths(g, o)


@pytest.mark.parametrize("p_direct", [0.7, 0.0])
def test_glass_paths_match_oracle(port, p_direct):
    """Transmissive and half-opaque boxes: refraction, the Fresnel split,
    media and absorption, the BTDF in light sampling, 16x samples behind
    glass -- against the oracle on the same random streams."""
    c = scenes.cornell_glass()
    cam = scenes.cornell_camera(40, 40, 8, p_direct=p_direct)
    g, _ = gpu_records(api.Model(c), cam, seed=17)
    o = port.scene(c).render(cam, seed=17, mode=1)
    assert (o[..., 33] < 1e-4).sum() > 50
    compare_paths(g, o, frac=0.95)


def test_glass_mean_matches_reference_stream(port):
    """Statistical: the GPU's counter streams against the reference's own
    mt19937 stream (the oracle in mode 0, pinned to the reference) at 1024 spp:
    mean luminance of the whole image (seed-to-seed spread 0.3 %) and of the
    glass box's pixels (spread 3.5 %: paths through glass to the light are
    rare and bright)."""
    c = scenes.cornell_glass()
    cam = scenes.cornell_camera(32, 32, 1024)
    g, _ = gpu_records(api.Model(c), cam, seed=23)
    o = port.scene(c).render(cam, seed=23, mode=0)
    lg, lo = linear_image(g) @ LUM, linear_image(o) @ LUM
    glass = o[..., 33] < 1e-4
    assert abs(lg.mean() - lo.mean()) <= 0.02 * lo.mean()
    assert abs(lg[glass].mean() - lo[glass].mean()) <= 0.12 * lo[glass].mean()


def test_lane_split_invariance():
    c = scenes.cornell()
    m = api.Model(c)
    cam = scenes.cornell_camera(40, 40, 64)
    base, _ = gpu_records(m, cam, seed=21, lanes=1)
    for k in (2, 8, 32):
        r, _ = gpu_records(m, cam, seed=21, lanes=k)
        np.testing.assert_allclose(linear_image(r), linear_image(base), rtol=1e-4, atol=1e-6)
        assert np.array_equal(r[..., 16:31], base[..., 16:31], equal_nan=True)


def test_host_buffers_match_device_buffers():
    c = scenes.cornell()
    m = api.Model(c)
    cam = scenes.cornell_camera(32, 32, 8)
    d, _ = gpu_records(m, cam, seed=2)
    h, _ = gpu_records(m, cam, seed=2, host=True)
    assert np.array_equal(d, h, equal_nan=True)


def test_emitter_and_miss_pixels(port):
    c = scenes.cornell()
    m = api.Model(c)
    # looking up at the light from below: emissive first hits
    up = scenes.Camera((0.5, 0.3, 0.5), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0), (1.0, 0.0, 0.0), 0.02, 24, 24, 8)
    g, _ = gpu_records(m, up, seed=4)
    o = port.scene(c).render(up, seed=4, mode=1)
    compare_paths(g, o)
    assert (g[..., 19:22].sum(-1) > 0).any()
    # looking out of the open front: every primary ray misses (no sky)
    out = scenes.Camera((0.5, 0.5, 0.5), (0.0, 0.0, -1.0), (0.0, -1.0, 0.0), (1.0, 0.0, 0.0), 0.001, 16, 16, 8)
    g2, _ = gpu_records(m, out, seed=4)
    assert np.isnan(g2[..., 22]).all() and np.all(g2[..., 0:16] == 0)


def test_render_argument_errors():
    m = api.Model(scenes.cornell())
    cam = scenes.cornell_camera(8, 8, 4)
    for field, value in [("P_Direct", 1.5), ("max_depth", 0), ("max_depth", 17), ("lanes_per_pixel", 65),
                         ("width", 0)]:
        a = api.RenderArgs.from_camera(cam)
        setattr(a, field, value)
        with pytest.raises(api.RmnError) as e:
            api.render(m, a, api.Photo(8, 8))
        assert e.value.status == 1, field


def _rel_mse(a, b):
    return ((a - b) ** 2).mean() / (b ** 2).mean()


def _bin(img, f=4):
    h, w, c = img.shape
    h, w = h // f * f, w // f * f
    return img[:h, :w].reshape(h // f, f, w // f, f, c).mean((1, 3))


# GPU renders per converged case: 8 for the estimate, 8 more (independent)
# for the per-pixel variance of the bias test
CONVERGED_GPU_SEEDS = tuple(range(101, 117))


@pytest.mark.parametrize("case", CONVERGED_CASES)
def test_converged_matches_reference(case):
    """North-star image parity at 4096 spp against the reference's own
    renderer, on the linear Photo::shade(Full) image.

    The reference's estimator is heavy-tailed, so relative MSE between two
    independent 4096-spp renders is well above 1e-3 for the reference
    against itself (Cornell 5.0e-3 to 6.7e-3: ten pixels carry a third of
    it). The gates therefore compare with the reference's own floor, from
    four independent reference renders:
    * relative MSE, GPU against each reference render, averaged over 8 GPU
      seeds and the 4 references: at most 1.1x the relative MSE between two
      reference renders, averaged over the pairs (equal in expectation for
      the same estimator, larger by the squared bias if the GPU were
      biased);
    * bias: per pixel, z = (mean of the reference renders - mean of 8 GPU
      renders) / sqrt(s2 (1/4 + 1/8)), s2 the luminance variance across 8
      further, independent GPU renders (so z has mean 0 exactly when the
      estimators agree, whatever the tails); the mean z over the image and
      over every 16 x 16 block must be within 4.5 and 5 standard errors of 0;
    * mean luminance within 0.5%; relative MSE <= 1e-3 on 4x4-binned
      images (the reference against itself: 4e-4 and below)."""
    z = np.load(os.path.join(GOLDEN, f"converged_{case}.npz"))
    R = [z[k].astype(np.float64) for k in sorted(z.files) if k.startswith("linear_")]
    A = R[0]
    sc, cam = converged_case(case)
    m = api.Model(sc)
    G = []
    for seed in CONVERGED_GPU_SEEDS:
        g, photo = gpu_records(m, cam, seed=seed)
        lin = photo.shade(api.Full).cpu().numpy().astype(np.float64).reshape(A.shape)
        if seed == CONVERGED_GPU_SEEDS[0]:
            assert np.allclose(lin, linear_image(g).reshape(A.shape), rtol=1e-5, atol=1e-6)
        G.append(lin)
    G = np.stack(G)
    k, nr = len(G) // 2, len(R)
    floor = np.mean([_rel_mse(R[i], R[j]) for i in range(nr) for j in range(nr) if i != j])
    gpu = np.mean([_rel_mse(g, r) for g in G[:k] for r in R])
    gpu_floor = np.mean([_rel_mse(G[i], G[j]) for i in range(k) for j in range(k) if i != j])
    binned = _rel_mse(_bin(G[0]), _bin(A))
    Rm = np.mean(R, axis=0)
    lum_g, lum_r = (G[:k] @ LUM).mean(), (Rm @ LUM).mean()
    # bias
    L = G @ LUM
    mean_g, var_g = L[:k].mean(0), L[k:].var(0, ddof=1)
    Lr = Rm @ LUM
    # pixels whose GPU renders vary by less than float rounding (misses,
    # emitters seen directly) are deterministic: compared directly below
    live = var_g > (1e-5 * np.maximum(np.abs(mean_g), 1e-12)) ** 2
    zs = (Lr - mean_g)[live] / np.sqrt(var_g[live] * (1.0 / nr + 1.0 / k))
    zmean = zs.mean() / (zs.std() / np.sqrt(zs.size))
    zmap = np.full(live.shape, np.nan)
    zmap[live] = zs
    h, w = zmap.shape
    blocks = []
    for y in range(0, h - 15, 16):
        for x in range(0, w - 15, 16):
            b = zmap[y:y + 16, x:x + 16]
            b = b[np.isfinite(b)]
            if b.size >= 64:
                blocks.append(b.mean() / (b.std() / np.sqrt(b.size)))
    blocks = np.array(blocks)
    # the deterministic pixels must equal the reference's (the sky's lookup
    # differs in the last bits between CUDA's and glibc's atan2f / acosf)
    np.testing.assert_allclose(L[0][~live], Lr[~live], rtol=2e-3, atol=1e-6)
    print(f"{case}: rel-MSE GPU-ref {gpu:.3e}, ref-ref {floor:.3e} (ratio {gpu / floor:.3f}), GPU-GPU "
          f"{gpu_floor:.3e}; binned {binned:.3e}; mean luminance {lum_g:.6f} vs {lum_r:.6f}; "
          f"z mean {zs.mean():+.4f} ({zmean:+.2f} se), |block z| max {np.abs(blocks).max():.2f} "
          f"over {blocks.size} blocks")
    assert gpu <= 1.1 * floor
    assert abs(zmean) <= 4.5
    assert np.abs(blocks).max() <= 5.0
    assert abs(lum_g - lum_r) <= 5e-3 * lum_r
    assert binned <= 1e-3


def _photo_np(ph):
    return [x.cpu().numpy() for x in (ph.radiance_Dd, ph.radiance_Ds, ph.radiance_Id, ph.radiance_Is, ph.Gbuffer)]


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_equals_individual_renders(use_graph):
    """A batch of uneven renders (two scenes, different sizes, spp, depths,
    lane splits) gives each item exactly the images of its own rmn_render."""
    cor = api.Model(scenes.cornell())
    hf = scenes.heightfield(30, seed=2, extent=3.0, patch=8)
    hf.env = scenes.sky_env(64, 32, sun_radiance=100.0, sun_diameter_deg=8.0)
    sky = api.Model(hf)
    skycam = scenes.Camera((0.3, 2.0, -0.8), (0.35, -0.45, 0.82), (0.0, -1.0, 0.0), (-1.0, 0.0, 0.0), 0.03, 33, 21, 9)
    gl = api.Model(scenes.cornell_glass())
    specs = [(cor, scenes.cornell_camera(40, 40, 16), 1, 4), (sky, skycam, 2, 0),
             (cor, scenes.cornell_camera(17, 29, 5, max_depth=6), 3, 1), (sky, skycam, 4, 32),
             (gl, scenes.cornell_camera(24, 24, 6), 5, 0)]
    items, solo = [], []
    for m, cam, seed, k in specs:
        a = api.RenderArgs.from_camera(cam, seed=seed, lanes_per_pixel=k)
        items.append((m, a, api.Photo(cam.width, cam.height)))
        solo.append(_photo_np(api.render(m, a)))
    b = api.Batch(items, use_graph=use_graph)
    for rep in range(2):
        b.render()
        torch.cuda.synchronize()
        for (m, a, ph), ref in zip(items, solo):
            got = _photo_np(ph)
            for x, y in zip(got, ref):
                assert np.array_equal(x, y, equal_nan=True)
    prof = b.profile()
    assert prof["pixels"] == sum(c.width * c.height for _, c, _, _ in specs)
    assert prof["closest_rays"] >= prof["pixels"] and prof["path_ms"] > 0


def test_render_profile_counts():
    m = api.Model(scenes.cornell())
    cam = scenes.cornell_camera(32, 32, 16)
    a = api.RenderArgs.from_camera(cam, seed=9)
    ref = _photo_np(api.render(m, a))
    ph, prof = api.render_profile(m, a)
    for x, y in zip(_photo_np(ph), ref):
        assert np.array_equal(x, y, equal_nan=True)
    assert prof["pixels"] == 32 * 32
    assert prof["sample_slots"] > 0 and prof["shadow_rays"] > 0 and prof["inner_visits"] > 0
    assert prof["triangle_tests"] >= prof["leaf_visits"] > 0


def test_batch_update_moves_cameras():
    """rmn_batch_update: new cameras and seeds for a built batch (its graph
    replayed) give the images of rmn_render with those arguments; a change of
    image size is refused."""
    import dataclasses
    cor = api.Model(scenes.cornell())
    gl = api.Model(scenes.cornell_glass())
    cams = [scenes.cornell_camera(32, 32, 8), scenes.cornell_camera(24, 20, 6)]
    models = [cor, gl]
    args = [api.RenderArgs.from_camera(c, seed=3 + k) for k, c in enumerate(cams)]
    items = [(m, a, api.Photo(c.width, c.height)) for m, a, c in zip(models, args, cams)]
    b = api.Batch(items, use_graph=True)
    b.render()
    moved = [dataclasses.replace(c, position=(0.45, 0.55, -1.3)) for c in cams]
    new_args = [api.RenderArgs.from_camera(c, seed=11 + k) for k, c in enumerate(moved)]
    b.update(new_args)
    b.render()
    torch.cuda.synchronize()
    for (m, a, ph), na in zip(items, new_args):
        ref = _photo_np(api.render(m, na))
        for x, y in zip(_photo_np(ph), ref):
            assert np.array_equal(x, y, equal_nan=True)
    assert b.update_bytes > 0
    bad = [api.RenderArgs.from_camera(scenes.cornell_camera(40, 40, 8), seed=1), new_args[1]]
    with pytest.raises(api.RmnError) as e:
        b.update(bad)
    assert e.value.status == 1
