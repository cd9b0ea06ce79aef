"""Pin the CPU restatement (oracle/port) against the reference.

Two sources of truth:
* the reference's own sources compiled with shims (oracle/_ref, fixture
  ``ref``) -- only where the reference checkout exists;
* the committed fixtures of tests/golden, generated from that build by
  tests/golden/make_golden.py -- everywhere.
Everything here is integer/bit-level: identical trees, identical hit ids and
t, identical occlusion answers, bit-identical renders under the reference's
own mt19937 stream, bit-identical composite and FXAA.
"""
import os

import numpy as np
import pytest

from raym0nade_gb300 import scenes
from tests.golden.make_golden import (PHOTO_CASES, PHOTO_POST, edge_rays, photo_records, reachable, room_rays,
                                      scene_from, tie_soup)

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def same(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)


# ------------------------------------------------------------ golden ------
def test_golden_trace(port):
    z = np.load(os.path.join(GOLDEN, "trace_soup.npz"))
    ps = port.scene(scene_from(z))
    boxes, ranges, order = ps.bvh()
    u = z["nodes"]
    assert same(reachable(ranges), u)
    assert same(boxes[u], z["boxes"]) and same(ranges[u], z["ranges"]) and same(order, z["order"])
    face, t, bc = ps.trace_closest(z["rays"])
    assert same(face, z["face"]) and same(t, z["t"]) and same(bc, z["bary"])
    assert same(ps.trace_shadow(z["shadow_rays"]), z["occluded"])


@pytest.mark.parametrize("name", ["render_cornell", "render_sky", "render_glass", "render_textured"])
def test_golden_render(port, name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    a = z["args"]
    cam = scenes.Camera(tuple(a[0:3]), tuple(a[3:6]), tuple(a[6:9]), tuple(a[9:12]), float(a[12]), int(a[17]),
                        int(a[18]), int(a[19]), float(a[16]), float(a[15]), float(a[13]), float(a[14]), int(a[21]))
    rec = port.scene(scene_from(z)).render(cam, seed=int(z["seed"]), mode=0)
    ref = z["records"]
    assert same(rec[..., :38], ref[..., :38])


def test_golden_textured_trace(port):
    z = np.load(os.path.join(GOLDEN, "render_textured.npz"))
    ps = port.scene(scene_from(z))
    face, t, bc = ps.trace_closest(z["rays"])
    assert same(face, z["face"]) and same(t, z["t"]) and same(bc, z["bary"])
    assert same(ps.trace_shadow(z["shadow_rays"]), z["occluded"])


def test_golden_photo(port):
    z = np.load(os.path.join(GOLDEN, "photo.npz"))
    for k, (stages, opt) in enumerate(PHOTO_CASES):
        r2, rgb = port.photo(z["records"], stages, opt, **PHOTO_POST)
        assert same(r2[..., :16], z["rec%d" % k] if stages & 3 else z["records"][..., :16]), (stages, opt)
        if rgb is not None:
            assert same(rgb, z["rgb%d" % k]), (stages, opt)


def test_golden_post(port):
    z = np.load(os.path.join(GOLDEN, "post.npz"))
    assert same(port.compose(z["records"], 1.0, gamma=False), z["linear"])
    assert same(port.compose(z["records"], 1.0, gamma=True), z["display"])
    assert same(port.fxaa(z["fxaa_in"]), z["fxaa_out"])


# ------------------------------------------------- live reference ---------
def _pair(port, ref, scene):
    return port.scene(scene), ref.scene(scene)


@pytest.mark.parametrize("n,seed", [(1, 1), (7, 2), (10, 3), (11, 4), (3000, 5), (20011, 6)])
def test_bvh_matches_reference(port, ref, n, seed):
    ps, rs = _pair(port, ref, scenes.random_soup(n, seed))
    bp, rp, op = ps.bvh()
    br, rr, orr = rs.bvh()
    assert bp.shape == br.shape
    u = reachable(rr)
    assert same(reachable(rp), u)
    assert same(bp[u], br[u]) and same(rp[u], rr[u]) and same(op, orr)


def test_cornell_lights_match_reference(port, ref):
    ps, rs = _pair(port, ref, scenes.cornell())
    assert same(ps.lights(), rs.lights())


@pytest.mark.parametrize("n", [1, 10, 5000])
def test_trace_matches_reference(port, ref, n):
    s = tie_soup(n, 21) if n > 60 else scenes.random_soup(n, 21)
    ps, rs = _pair(port, ref, s)
    rays = edge_rays(30000, 22)
    if n <= 10:  # aim every ray at the few triangles
        tgt = s.positions.reshape(-1, 3, 3).mean(1)[np.arange(rays.shape[0]) % n]
        d = tgt - rays[:, 0:3]
        rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    a, b = ps.trace_closest(rays), rs.trace_closest(rays)
    for x, y in zip(a, b):
        assert same(x, y)
    sr = scenes.random_rays(30000, 23, shadow=True)
    assert same(ps.trace_shadow(sr), rs.trace_shadow(sr))


def test_trace_cornell_matches_reference(port, ref):
    ps, rs = _pair(port, ref, scenes.cornell())
    rays = scenes.random_rays(20000, 31)
    rays[:, 0:3] = rays[:, 0:3] * 0.98 + 0.01  # inside the room
    for x, y in zip(ps.trace_closest(rays), rs.trace_closest(rays)):
        assert same(x, y)


@pytest.mark.parametrize("spp,p_direct", [(16, 0.7), (5, 0.0), (3, 1.0), (9, 0.5)])
def test_render_cornell_matches_reference(port, ref, spp, p_direct):
    ps, rs = _pair(port, ref, scenes.cornell())
    cam = scenes.cornell_camera(20, 20, spp, p_direct=p_direct)
    a = ps.render(cam, seed=5 + spp)
    b = rs.render(cam, seed=5 + spp)
    assert same(a[..., :38], b[..., :38])


def test_render_pixels_match_whole_renders(port, ref):
    """The pixel-list render (the benchmark's stratified CPU sample) gives each
    listed pixel exactly its record of a whole-image render."""
    c = scenes.cornell()
    cam = scenes.cornell_camera(20, 16, 6)
    rng = np.random.default_rng(3)
    px = rng.choice(20 * 16, 50, replace=False).astype(np.int32)
    for lib in (port, ref):
        whole = lib.scene(c).render(cam, seed=12).reshape(-1, 40)
        part = lib.scene(c).render_pixels(cam, 12, px)
        assert np.array_equal(part, whole[px], equal_nan=True)


@pytest.mark.parametrize("spp,p_direct", [(8, 0.7), (4, 0.0)])
def test_render_glass_matches_reference(port, ref, spp, p_direct):
    """Transmissive and semi-opaque materials: refraction, media, Fresnel
    split, the BTDF in light sampling, 16x indirect samples behind glass."""
    ps, rs = _pair(port, ref, scenes.cornell_glass())
    cam = scenes.cornell_camera(16, 16, spp, p_direct=p_direct)
    a = ps.render(cam, seed=11 + spp)
    b = rs.render(cam, seed=11 + spp)
    assert same(a[..., :38], b[..., :38])
    assert (a[..., 33] < 1e-4).sum() > 0  # some pixels see the glass


def test_render_sky_matches_reference(port, ref):
    hf = scenes.heightfield(20, seed=8, extent=3.0, patch=6)
    hf.env = scenes.sky_env(48, 24, sun_radiance=80.0, sun_diameter_deg=15.0)
    ps, rs = _pair(port, ref, hf)
    cam = scenes.Camera((0.2, 1.6, -0.6), (0.35, -0.45, 0.82), (0.0, -1.0, 0.0), (-1.0, 0.0, 0.0), 0.05, 14, 10, 12)
    assert same(ps.render(cam, seed=3)[..., :38], rs.render(cam, seed=3)[..., :38])


def test_post_matches_reference(port, ref):
    rng = np.random.default_rng(3)
    img = (rng.random((37, 53, 3)) ** 3).astype(np.float32) * 1.4
    img[:, 20:] += 0.5
    assert same(port.fxaa(img), ref.fxaa(img))
    assert same(port.gamma(img), ref.gamma(img))
    rec = rng.random((500, 40)).astype(np.float32)
    for g in (False, True):
        assert same(port.compose(rec, 1.3, gamma=g), ref.compose(rec, 1.3, gamma=g))


# ------------------------------------------------ textures (f2) -----------
def test_textured_lights_match_reference(port, ref_tex):
    for sky in (True, False):
        room = scenes.textured_room(sky=sky)
        assert same(port.scene(room).lights(), ref_tex.scene(room).lights())


def test_textured_trace_matches_reference(port, ref_tex):
    room = scenes.textured_room()
    ps, rs = port.scene(room), ref_tex.scene(room)
    rays = room_rays(20000, 41)
    a, b = ps.trace_closest(rays), rs.trace_closest(rays)
    assert all(same(x, y) for x, y in zip(a, b))
    srays = room_rays(20000, 42, shadow=True)
    assert same(ps.trace_shadow(srays), rs.trace_shadow(srays))
    # the cutouts matter: without the alpha test (a t_min other than eps
    # takes the bare BVH query) some rays stop at a cut-away texel instead
    raw = rays.copy()
    raw[:, 3] = np.float32(1.5e-4)
    assert (ps.trace_closest(raw)[0] != a[0]).sum() > 20


@pytest.mark.parametrize("sky,spp,p_direct", [(True, 16, 0.7), (False, 12, 0.7), (True, 6, 0.0)])
def test_render_textured_matches_reference(port, ref_tex, sky, spp, p_direct):
    room = scenes.textured_room(sky=sky)
    cam = scenes.textured_camera(64, 40, spp, p_direct=p_direct)
    a = port.scene(room).render(cam, seed=31)
    b = ref_tex.scene(room).render(cam, seed=31)
    assert same(a[..., :38], b[..., :38])
    assert set(np.unique(a[..., 36]).astype(int)) == set(range(6))


def test_ref_tex_refuses_constant_texels(ref_tex):
    room = scenes.textured_room()
    room.materials[2, 3] = 1.0  # a constant diffuse texel without a texture
    with pytest.raises(ValueError):
        ref_tex.scene(room)


# ------------------------------------------------ post passes (f3) ---------
def _inside_camera(w, h, spp):
    import math
    acc = math.tan(math.radians(30.0)) / (w / 2.0)
    return scenes.Camera((0.5, 0.5, 0.3), (0.0, 0.0, 1.0), (0.0, -1.0, 0.0), (-1.0, 0.0, 0.0), acc, w, h, spp)


@pytest.mark.parametrize("stages,opt", PHOTO_CASES)
def test_photo_passes_match_reference(port, ref, stages, opt):
    """spatialClamp, filter, bloom, depth of field and postProcessing on a
    Cornell render seen from inside the box (every pixel a hit) and on
    synthetic records with fireflies, bumpy normals and material patches."""
    rec = ref.scene(scenes.cornell()).render(_inside_camera(48, 32, 16), seed=5)
    for r, post in [(rec, dict(exposure=1.0, focus=0.5, coc=6.0, camera=(0.5, 0.5, 0.3))),
                    (photo_records(56, 36, 9), PHOTO_POST)]:
        a = port.photo(r, stages, opt, **post)
        b = ref.photo(r, stages, opt, **post)
        assert same(a[0], b[0])
        if a[1] is not None:
            assert same(a[1], b[1])


def test_photo_passes_change_the_image(port):
    """The cases are not vacuous: the clamp scales fireflies, the filter
    smooths, bloom adds light, depth of field blurs."""
    rec = photo_records(64, 40, 3)
    c, _ = port.photo(rec, 1)
    assert (c[..., :16] != rec[..., :16]).sum() > 30
    f, _ = port.photo(rec, 2)
    assert np.abs(f[..., 8:11] - rec[..., 8:11]).mean() > 0.01
    _, base = port.photo(rec, 8, 63, **PHOTO_POST)
    _, bl = port.photo(rec, 8, 63 | 256, **PHOTO_POST)
    _, dof = port.photo(rec, 8, 63 | 1024, **PHOTO_POST)
    assert (bl - base).min() >= 0.0 and (bl - base).max() > 0.1
    assert np.abs(dof - base).mean() > 0.01


# ------------------------------------------------------------- textures ----
MIP_SIZES = [(21, 37), (1, 64), (3, 300), (16, 2048), (255, 257), (1, 1), (600, 5), (64, 64)]


def test_mip_chain_matches_reference(ref_tex):
    """oracle/image_codecs.mip_chain (what the device-built chains are checked against)
    against the reference's own ImageData::generateMipmaps, level for level."""
    from oracle.image_codecs import mip_chain
    rng = np.random.default_rng(31)
    for h, w in MIP_SIZES:
        tex = rng.integers(0, 256, (h, w, 4)).astype(np.uint8)
        want = ref_tex.mip_chain(tex)
        got = mip_chain(tex)
        assert len(got) == len(want) and all(np.array_equal(a, b) for a, b in zip(got, want)), (h, w)


def test_golden_mip_chains():
    """The same pin carried by tests/golden/mips.npz (made from the
    reference by make_golden.py --mips)."""
    from oracle.image_codecs import mip_chain
    z = np.load(os.path.join(GOLDEN, "mips.npz"))
    for k in range(int(z["count"])):
        got = mip_chain(z[f"tex{k}"])
        want = [z[f"tex{k}_level{lv}"] for lv in range(int(z[f"tex{k}_depth"]))]
        assert len(got) == len(want) and all(np.array_equal(a, b) for a, b in zip(got, want)), k


def test_url_decode_matches_reference(ref_tex):
    from oracle.obj_import import url_decode
    for s in ["a%20b", "tex\\leaf.dds", "%41%42c", "x%4", "%2F%2f", "plain.dds", "100%25", "%e9t%C3%A9.png", ""]:
        assert url_decode(s) == ref_tex.url_decode(s), s


def test_imported_materials_match_reference(ref_tex, tmp_path):
    """The importer's materials (native rmn_model_read and the oracle's
    restatement) against the reference's own Material::loadMaterialProperties
    for the same names and opacities, including opacities within float
    rounding of the 0.99 threshold."""
    from oracle import obj_import
    from raym0nade_gb300 import assets
    cases = [("Ice", "d 0.5"), ("Water", "d 0.98"), ("White_Wine", "d 0.99"), ("Beer", "Tr 0.8"),
             ("Red_Wine", "d 0.98999999"), ("TransparentGlassWine", "d 0.9899999"), ("TransparentGlass", "d 0"),
             ("Other", "Tr 0.0"), ("Opaque", None), ("Half", "d 0.5"), ("Neg", "d -1")]
    mtl = "".join(f"newmtl {n}\n" + (f"{d}\n" if d else "") for n, d in cases)
    obj = "mtllib m.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\n" + "".join(f"usemtl {n}\nf 1 2 3\n" for n, _ in cases)
    (tmp_path / "m.mtl").write_text(mtl)
    (tmp_path / "m.obj").write_text(obj)
    folder = str(tmp_path) + "/"
    for sc in (assets.load_model(folder, "m.obj"), obj_import.load_model(folder, "m.obj")):
        for name, d in cases:
            op = None
            if d is not None:
                key, v = d.split()
                op = np.float32(float(v)) if key == "d" else np.float32(1.0) - np.float32(float(v))
            ref = ref_tex.material_properties(name, op)
            row = sc.materials[sc.material_names.index(name)]
            got = np.array([row[11], row[12], row[8], row[13], row[14], row[15]], np.float32)
            assert np.array_equal(got, ref[:6]), (name, d, got, ref)


def test_save_png_pixels_match_reference(ref, tmp_path):
    """rmn_save_png's decoded pixels against the rows the reference's own
    Photo::save hands to libpng (static_cast<png_byte>(v * 255)), on values
    in [0, 1] including every k / 255 boundary and its float neighbours."""
    from raym0nade_gb300 import _lib, build
    build.build()
    lib = _lib.load()
    k = np.arange(256, dtype=np.float32) / np.float32(255)
    edges = np.concatenate([k, np.nextafter(k, np.float32(0)), np.nextafter(k, np.float32(1))]).clip(0, 1)
    rng = np.random.default_rng(8)
    vals = np.concatenate([edges, rng.random(3 * 64 * 40 - edges.size, dtype=np.float32)])
    img = vals[:3 * 64 * 40].reshape(40, 64, 3)
    want = ref.save_rows(img, str(tmp_path / "ref.png"))
    p = str(tmp_path / "ours.png")
    assert lib.rmn_save_png(np.ascontiguousarray(img).ctypes.data, 64, 40, p.encode()) == 0
    from oracle.image_codecs import png_read
    assert np.array_equal(png_read(p), want)


def test_script_mirrors_feed_the_references_loaders(ref_tex, tmp_path, monkeypatch):
    """The reference's own SkyBox::load and Material::loadImageFromDDS,
    calling scripts/hdr_to_array.py and scripts/dds_to_array.py through
    their embedded-Python path, with those scripts being this package's
    mirrors: the reference ends up with the texels the library decodes."""
    from raym0nade_gb300 import assets, build
    from tests.golden import image_files as F
    build.build()
    (tmp_path / "scripts").mkdir()
    (tmp_path / "scripts" / "hdr_to_array.py").write_text("from raym0nade_gb300.assets import hdr_to_array\n")
    (tmp_path / "scripts" / "dds_to_array.py").write_text("from raym0nade_gb300.assets import dds_to_array\n")
    rng = np.random.default_rng(17)
    rgbe = F.float_to_rgbe(np.exp(rng.normal(0, 2, (12, 40, 3))))
    (tmp_path / "sky.hdr").write_bytes(F.encode_hdr(rgbe))
    pay = rng.integers(0, 256, 3 * 4 * 16).astype(np.uint8).tobytes()
    (tmp_path / "t.dds").write_bytes(F.encode_dds(13, 10, pay, b"DXT5"))
    monkeypatch.chdir(tmp_path)
    sky_load, dds_load = ref_tex.python_loaders()
    got = sky_load(str(tmp_path / "sky.hdr"))
    raw = assets.load_image(str(tmp_path / "sky.hdr"), assets.HDR)
    h, w = raw.shape[:2]
    phi = np.float32(np.pi) * (np.arange(h, dtype=np.float32) + np.float32(0.5)) / np.float32(h)
    area = np.sin(phi) * np.float32(2 * np.pi) / np.float32(w * h)
    np.testing.assert_allclose(got, raw * area[:, None, None], rtol=2e-6, atol=0)
    tex = dds_load(str(tmp_path / "t.dds"))
    assert np.array_equal(tex, assets.load_image(str(tmp_path / "t.dds"), assets.DDS))


def test_reverse_gamma_matches_reference(ref):
    """Photo.reverseGammaCorrection of the mirror against the reference's
    Photo::reverseGammaCorrection (glm::pow of floats), bit for bit, on every
    k / 255 a loaded PNG yields and on random values."""
    from raym0nade_gb300 import api
    rng = np.random.default_rng(6)
    k255 = (np.arange(256, dtype=np.float32) / np.float32(255.0))
    x = np.concatenate([np.repeat(k255, 3), rng.random(3 * 4000, dtype=np.float32)]).reshape(-1, 3)
    assert np.array_equal(api.Photo.reverseGammaCorrection(x), ref.reverse_gamma(x))
