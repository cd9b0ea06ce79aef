"""Generate the golden fixtures of tests/golden from the reference itself.

Run in a checkout that has the reference sources (the oracle/_ref harness is
built from them): ``python tests/golden/make_golden.py``. Every fixture stores
its inputs (scene arrays, rays, camera, seed) next to the reference's outputs,
so machines without the reference -- and platforms whose numpy math differs in
the last bit -- check the CPU restatement against the same numbers.

Fixtures (numpy .npz, compressed):
  trace_soup.npz     2,000-triangle soup + 4,096 closest-hit rays (incl.
                     axis-parallel and duplicate-triangle tie cases) and 4,096
                     shadow rays -> face ids, t, barycentrics, occlusion,
                     reachable BVH nodes and the leaf-order face permutation.
  render_cornell.npz 24 x 24 Cornell render, 16 spp, reference mt19937 stream.
  render_sky.npz     16 x 12 render of a small heightfield under a lat-long
                     sky (sky-mode light sampling, smooth normals).
  render_glass.npz   20 x 20 render of the Cornell box with a glass box and a
                     half-opaque box, 8 spp (refraction, media, Fresnel split).
                     ``--glass`` writes this fixture alone.
  render_textured.npz  48 x 32 render of the textured room (diffuse,
                     specular, emissive and normal-map textures, mip chains,
                     alpha-tested cutouts), 16 spp, from the reference built
                     with its own src/material.cpp (oracle/_ref/libref_tex.so);
                     plus 4,096 closest-hit and 4,096 shadow rays through the
                     room (alpha-test retries). ``--textured`` writes it alone.
  post.npz           Photo::shade(Full) + gammaCorrection of render records,
                     and Photo::FXAA of a 96 x 64 image with hard edges.
  photo.npz          Photo's post passes on 32 x 20 synthetic records
                     (``photo_records``): spatialClamp, filter, bloom, depth
                     of field, postProcessing with and without them (the
                     cases of PHOTO_CASES). ``--photo`` writes it alone.
  mips.npz           ImageData::generateMipmaps of the reference on five
                     textures of odd, thin and long sizes (``--mips``).
  images/, images.npz  small PNG, Radiance HDR and DDS files (every PNG
                     colour type family, Adam7, all filters, stored / fixed /
                     dynamic deflate; flat and run-length HDR scanlines;
                     BC1-BC3 and uncompressed DDS) and their decoded arrays:
                     the written samples through libpng's transforms, RGBE
                     m * 2^(e - 136), BC blocks through oracle/image_codecs.py.
                     Needs no reference; ``--images`` writes them alone.
  converged_<case>.npz  converged reference images for the image-parity
                     tests: Photo::shade(Full) before gamma (float16) of four
                     independent 4096-spp renders (per-pixel seeds 4096,
                     8192, 12288, 16384: linear_a .. linear_d) of each case
                     of CONVERGED_CASES -- the Cornell
                     workload (256 x 256, depth 16, P_Direct 0.7), a
                     heightfield under the synthetic sun in sky mode
                     (192 x 108) and the glass Cornell box (128 x 128).
                     Made by ``python tests/golden/make_golden.py
                     --converged [case ...]``.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
os.environ.setdefault("RMN_REFERENCE_DIR", "/root/reference")  # the reference checkout these fixtures come from

from oracle import bindings  # noqa: E402
from raym0nade_gb300 import scenes  # noqa: E402


def scene_arrays(s):
    d = dict(positions=s.positions, normals=s.normals, uvs=s.uvs, indices=s.indices, mesh_first=s.mesh_first,
             mesh_material=s.mesh_material, materials=s.materials)
    if s.env is not None:
        d["env"] = s.env
    if s.mat_tex is not None:
        d["mat_tex"] = s.mat_tex
        for i, t in enumerate(s.textures):
            d["tex%d" % i] = t
    return d


def scene_from(z, prefix=""):
    g = lambda k: z[prefix + k]
    env = z[prefix + "env"] if (prefix + "env") in z else None
    sc = scenes.Scene(g("positions"), g("normals"), g("uvs"), g("indices"), g("mesh_first"), g("mesh_material"),
                      g("materials"), env)
    if (prefix + "mat_tex") in z:
        sc.mat_tex = g("mat_tex")
        n = 0
        while (prefix + "tex%d" % n) in z:
            n += 1
        sc.textures = [g("tex%d" % i) for i in range(n)]
    return sc


def photo_records(w, h, seed, miss=0.0):
    """Synthetic render records (h, w, 40) for the post passes: a tilted,
    bumpy surface seen from (0, 0, -1) (positions, jittered shape and
    surface normals), random roughness / metallic / opacity patches, noisy
    radiance with Var, fireflies planted in every buffer, an emitter patch
    bright enough to bloom; a fraction ``miss`` of pixels without a hit."""
    rng = np.random.default_rng(seed)
    r = np.zeros((h, w, 40), np.float32)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    u, v = xx / w - 0.5, yy / h - 0.5
    z = 1.0 + 0.6 * u + 0.3 * v + 0.05 * np.sin(9 * u) * np.cos(7 * v)
    pos = np.stack([u * z, v * z, z], -1)
    n = np.stack([-0.6 + 0.2 * rng.standard_normal((h, w)), -0.3 + 0.2 * rng.standard_normal((h, w)),
                  -np.ones((h, w))], -1)
    sn = n / np.linalg.norm(n, axis=-1, keepdims=True)
    n2 = sn + 0.02 * rng.standard_normal((h, w, 3))
    n2 /= np.linalg.norm(n2, axis=-1, keepdims=True)
    for b in range(4):
        rad = rng.gamma(2.0, 0.15, (h, w, 3)) * (1.0 + 0.5 * np.sin(5 * u + b))[..., None]
        spikes = rng.random((h, w)) < 0.01
        rad[spikes] *= rng.uniform(20, 400, (spikes.sum(), 1))
        r[..., 4 * b:4 * b + 3] = rad
        r[..., 4 * b + 3] = rng.gamma(1.0, 0.05, (h, w))
    r[..., 16:19] = rng.uniform(0.05, 0.95, (h, w, 3))
    em = (np.abs(u - 0.2) < 0.06) & (np.abs(v + 0.1) < 0.08)
    r[..., 19:22][em] = rng.uniform(2.0, 8.0, (em.sum(), 3))
    r[..., 22:25] = pos
    r[..., 25:28] = sn
    r[..., 28:31] = n2
    patch = ((xx // 8) + 3 * (yy // 8)).astype(np.int64) % 7
    r[..., 31] = np.array([0.01, 0.03, 0.1, 0.3, 0.5, 0.8, 1.0])[patch]
    r[..., 32] = np.where(patch % 3 == 0, 0.8, 0.0)
    r[..., 33] = np.where(patch == 5, 0.0, 1.0)
    r[..., 34] = 0.04
    r[..., 35] = 1.0
    r[..., 36] = patch
    r[..., 37] = 1.0
    if miss > 0:
        m = rng.random((h, w)) < miss
        r[..., 22:25][m] = np.nan
        r[..., 25:31][m] = np.nan
    return r


# (stages, options) of the photo.npz cases; post arguments exposure 1,
# focus 0.9, CoC 8, camera (0, 0, -1)
PHOTO_CASES = [(1, 0), (2, 0), (3, 0), (8, 63 | 256), (8, 63 | 1024), (8, 63 | 1024 | 256), (4, 63 | 1024 | 256 | 512),
               (3 | 4, 63 | 512), (4, 64), (4, 128), (4, 1 | 512)]
PHOTO_POST = dict(exposure=1.0, focus=0.9, coc=8.0, camera=(0.0, 0.0, -1.0))


def photo(R=None):
    if R is None:
        bindings.build(with_reference=True)
        R = bindings.OracleLib("ref")
    rec = photo_records(32, 20, 3)
    out = {"records": rec}
    for k, (stages, opt) in enumerate(PHOTO_CASES):
        r2, rgb = R.photo(rec, stages, opt, **PHOTO_POST)
        if stages & 3:  # the passes that change the radiance buffers
            out["rec%d" % k] = r2[..., :16]
        if rgb is not None:
            out["rgb%d" % k] = rgb
    np.savez_compressed(os.path.join(HERE, "photo.npz"), **out)


def room_rays(n, seed, shadow=False):
    """Rays through the textured room: origins in its volume, uniform
    directions; shadow rays aim U(0, 6) ahead."""
    rng = np.random.default_rng(seed)
    r = np.empty((n, 8), np.float32)
    r[:, 0:3] = rng.uniform((-1.9, 0.05, 0.1), (1.8, 2.9, 5.9), (n, 3))
    r[:, 3] = np.float32(1e-4)
    d = rng.standard_normal((n, 3))
    r[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    r[:, 7] = rng.uniform(0.0, 6.0, n) if shadow else np.inf
    return r


def reachable(ranges):
    out, st = [], [1]
    while st:
        u = st.pop()
        out.append(u)
        if ranges[u, 1] == 0:
            st += [2 * u, 2 * u + 1]
    return np.array(sorted(out), np.int64)


def tie_soup(n, seed):
    """Random soup with a few exact duplicate triangles (exact t ties)."""
    s = scenes.random_soup(n, seed)
    k = 50
    dup = s.indices[:k]
    s.indices = np.concatenate([s.indices, dup]).astype(np.int32)
    s.mesh_first = np.array([0, s.indices.shape[0]], np.int32)
    return s


def edge_rays(n, seed):
    r = scenes.random_rays(n, seed)
    # a quarter of the rays with one or two direction components below the
    # 1e-4 axis-parallel cut-off of rayInBox
    q = n // 4
    r[:q, 4 + (np.arange(q) % 3)] = np.float32(5e-5)
    r[: q // 2, 4 + ((np.arange(q // 2) + 1) % 3)] = np.float32(-2e-5)
    d = r[:, 4:7].astype(np.float64)
    r[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    return r


def main():
    bindings.build(with_reference=True)
    R = bindings.OracleLib("ref")

    soup = tie_soup(2000, 11)
    rays = edge_rays(4096, 12)
    srays = scenes.random_rays(4096, 13, shadow=True)
    rs = R.scene(soup)
    boxes, ranges, order = rs.bvh()
    u = reachable(ranges)
    face, t, bc = rs.trace_closest(rays)
    occ = rs.trace_shadow(srays)
    np.savez_compressed(os.path.join(HERE, "trace_soup.npz"), **scene_arrays(soup), rays=rays, shadow_rays=srays,
                        face=face, t=t, bary=bc, occluded=occ, nodes=u, boxes=boxes[u], ranges=ranges[u], order=order)

    cor = scenes.cornell()
    cam = scenes.cornell_camera(24, 24, 16)
    rec = R.scene(cor).render(cam, seed=2024)
    np.savez_compressed(os.path.join(HERE, "render_cornell.npz"), **scene_arrays(cor), args=cam.packed(), seed=2024,
                        records=rec)

    hf = scenes.heightfield(24, seed=5, extent=3.0, patch=8)
    hf.env = scenes.sky_env(64, 32, sun_radiance=50.0, sun_diameter_deg=12.0)
    hcam = scenes.Camera((0.2, 1.6, -0.6), (0.35, -0.45, 0.82), (0.0, -1.0, 0.0), (-1.0, 0.0, 0.0), 0.05, 16, 12, 8)
    hrec = R.scene(hf).render(hcam, seed=77)
    np.savez_compressed(os.path.join(HERE, "render_sky.npz"), **scene_arrays(hf), args=hcam.packed(), seed=77,
                        records=hrec)

    glass(R)
    textured()
    photo(R)
    images()
    mips()

    rgb_lin = R.compose(rec, 1.0, gamma=False)
    rgb = R.compose(rec, 1.0, gamma=True)
    rng = np.random.default_rng(14)
    img = np.zeros((64, 96, 3), np.float32)
    img[:, 40:] = 0.9
    img[20:44, 10:30] = rng.random((24, 20, 3)).astype(np.float32)
    yy, xx = np.mgrid[0:64, 0:96]
    img[(xx - 70) ** 2 + (yy - 30) ** 2 < 200] = (0.1, 0.2, 0.05)
    img += rng.random(img.shape).astype(np.float32) * 0.05
    fx = R.fxaa(img)
    np.savez_compressed(os.path.join(HERE, "post.npz"), records=rec, linear=rgb_lin, display=rgb, fxaa_in=img,
                        fxaa_out=fx)
    print("fixtures written to", HERE)


def glass(R=None):
    if R is None:
        bindings.build(with_reference=True)
        R = bindings.OracleLib("ref")
    g = scenes.cornell_glass()
    cam = scenes.cornell_camera(20, 20, 8)
    rec = R.scene(g).render(cam, seed=909)
    np.savez_compressed(os.path.join(HERE, "render_glass.npz"), **scene_arrays(g), args=cam.packed(), seed=909,
                        records=rec)


def textured():
    bindings.build(with_reference=True)
    T = bindings.OracleLib("ref_tex")
    room = scenes.textured_room()
    cam = scenes.textured_camera(48, 32, 16)
    ts = T.scene(room)
    rec = ts.render(cam, seed=515)
    rays = room_rays(4096, 516)
    srays = room_rays(4096, 517, shadow=True)
    face, t, bc = ts.trace_closest(rays)
    occ = ts.trace_shadow(srays)
    np.savez_compressed(os.path.join(HERE, "render_textured.npz"), **scene_arrays(room), args=cam.packed(),
                        seed=515, records=rec, rays=rays, face=face, t=t, bary=bc, shadow_rays=srays, occluded=occ)


def images():
    import shutil
    import zlib

    from oracle import image_codecs
    from tests.golden import image_files as F
    d = os.path.join(HERE, "images")
    if os.path.isdir(d):
        shutil.rmtree(d)
    os.makedirs(d)
    rng = np.random.default_rng(2718)
    out = {}

    def png(name, h, w, ctype, depth, **kw):
        pal = kw.pop("palette", None)
        s = rng.integers(0, 1 << depth, (h, w, F.PNG_CHANNELS[ctype]))
        open(os.path.join(d, name), "wb").write(F.encode_png(s, ctype, depth, palette=pal, **kw))
        out[name] = F.png_expected_rgb(s, ctype, depth, pal)

    png("gray2_adam7.png", 9, 11, 0, 2, interlace=True, level=1, strategy=zlib.Z_FIXED, filters=(1, 2, 3, 4))
    png("rgb16_paeth.png", 6, 10, 2, 16, filters=(4, 3), level=9)
    png("palette4.png", 7, 9, 3, 4, palette=rng.integers(0, 256, (12, 3)), trns=bytes([0, 128]),
        filters=(0, 1))
    png("rgba8_stored.png", 5, 8, 6, 8, level=0, filters=(2, 4, 1))
    png("graya16.png", 5, 5, 4, 16, interlace=True, filters=(3,))

    def hdr(name, h, w, **kw):
        rgbe = F.float_to_rgbe(np.exp(rng.normal(0.0, 3.0, (h, w, 3))))
        rgbe[h // 2, :] = rgbe[h // 2, 0]
        open(os.path.join(d, name), "wb").write(F.encode_hdr(rgbe, **kw))
        out[name] = F.rgbe_expected(rgbe)

    hdr("sky_rle.hdr", 12, 40, flat_from=9)
    hdr("narrow_flat.hdr", 5, 4)

    def bc(name, h, w, kind):
        size = 8 if kind == 1 else 16
        pay = rng.integers(0, 256, ((w + 3) // 4) * ((h + 3) // 4) * size).astype(np.uint8).tobytes()
        open(os.path.join(d, name), "wb").write(F.encode_dds(w, h, pay, b"DXT%d" % (2 * kind - 1)))
        out[name] = image_codecs.bc_decode(pay, w, h, kind)

    bc("bc1.dds", 6, 10, 1)
    bc("bc2.dds", 8, 8, 2)
    bc("bc3.dds", 7, 13, 3)
    px = rng.integers(0, 256, (5, 6, 4)).astype(np.uint8)
    masks = (0x00FF0000, 0x0000FF00, 0x000000FF, 0xFF000000)
    open(os.path.join(d, "bgra32.dds"), "wb").write(
        F.encode_dds(6, 5, px.tobytes(), bitcount=32, masks=masks, alpha_flag=True))
    out["bgra32.dds"] = px[..., [2, 1, 0, 3]]
    open(os.path.join(d, "bgr24.dds"), "wb").write(
        F.encode_dds(6, 5, px[..., :3].tobytes(), bitcount=24, masks=masks[:3] + (0,)))
    out["bgr24.dds"] = px[..., [2, 1, 0]]
    np.savez_compressed(os.path.join(HERE, "images.npz"), **out)


def mips():
    """ImageData::generateMipmaps of the reference on textures of odd, thin
    and long sizes -> tests/golden/mips.npz."""
    bindings.build(with_reference=True)
    T = bindings.OracleLib("ref_tex")
    rng = np.random.default_rng(4242)
    out = {}
    sizes = [(21, 37), (3, 300), (63, 65), (1, 64), (300, 5)]
    for k, (h, w) in enumerate(sizes):
        tex = rng.integers(0, 256, (h, w, 4)).astype(np.uint8)
        levels = T.mip_chain(tex)
        out[f"tex{k}"] = tex
        out[f"tex{k}_depth"] = np.int64(len(levels))
        for lv, a in enumerate(levels):
            out[f"tex{k}_level{lv}"] = a
    out["count"] = np.int64(len(sizes))
    np.savez_compressed(os.path.join(HERE, "mips.npz"), **out)


CONVERGED_CASES = ("cornell", "sky", "glass")
CONVERGED_SEEDS = (4096, 8192, 12288, 16384)


def converged_case(name):
    """Scene and camera of a converged-image case (4096 spp).

    cornell: the Cornell workload, 256 x 256, depth 16.
    sky:     a 256 x 256-vertex heightfield with 0.1-wide cells (smooth
             normals, the 50/50 Lambertian / GGX-conductor patches) under
             the 2048 x 1024 synthetic sky with its 0.5-degree sun of
             radiance 5e4 -- sky-mode light sampling -- seen from the
             heightfield workload's camera at 192 x 108.
    glass:   the Cornell box with the glass tall box and the half-opaque
             short box, 128 x 128 (16x the indirect paths behind glass)."""
    if name == "cornell":
        return scenes.cornell(), scenes.cornell_camera(256, 256, 4096)
    if name == "sky":
        ext = 25.6
        hf = scenes.heightfield(256, seed=3, extent=ext, patch=16)
        hf.env = scenes.sky_env(2048, 1024)
        return hf, scenes.heightfield_camera(192, 108, 4096, extent=ext)
    if name == "glass":
        return scenes.cornell_glass(), scenes.cornell_camera(128, 128, 4096)
    raise ValueError(name)


def converged(names=CONVERGED_CASES):
    """Four independent 4096-spp renders of each case by the reference's own
    renderer (per-pixel mt19937 seeds differ between them), on all host
    threads; the linear composite of each is stored as float16."""
    import time
    bindings.build(with_reference=True)
    R = bindings.OracleLib("ref")
    for name in names:
        sc, cam = converged_case(name)
        rs = R.scene(sc)
        out = dict(args=cam.packed(), seeds=np.asarray(CONVERGED_SEEDS, np.int64))
        for tag, seed in zip("abcd", CONVERGED_SEEDS):
            t0 = time.time()
            rec = rs.render(cam, seed=seed, threads=os.cpu_count() or 8)
            lin = R.compose(rec, 1.0, gamma=False)
            assert np.isfinite(lin).all() and np.abs(lin).max() < 6e4, name
            out["linear_" + tag] = lin.astype(np.float16)
            print(f"{name} seed {seed}: {time.time() - t0:.1f} s", flush=True)
        np.savez_compressed(os.path.join(HERE, f"converged_{name}.npz"), **out)
    print("converged references written")


if __name__ == "__main__":
    if "--converged" in sys.argv:
        converged([a for a in sys.argv[1:] if not a.startswith("--")] or CONVERGED_CASES)
    elif "--glass" in sys.argv:
        glass()
        print("glass fixture written to", HERE)
    elif "--photo" in sys.argv:
        photo()
        print("photo fixture written to", HERE)
    elif "--mips" in sys.argv:
        mips()
        print("mip chains written to", HERE)
    elif "--images" in sys.argv:
        images()
        print("image files written to", os.path.join(HERE, "images"))
    elif "--textured" in sys.argv:
        textured()
        print("textured fixture written to", HERE)
    else:
        main()
