"""The asset front-end on the CPU: rmn_image_load's PNG / DDS / HDR decoders
and the OBJ/MTL importer (raym0nade_gb300.assets).

Files are written by tests/golden/image_files.py from content whose decoded
form is known: a PNG's sample array through libpng's transforms (strip_16,
gray and palette expansion, alpha dropped), an HDR's RGBE bytes
(m * 2^(e - 136)), a DDS's block bytes decoded by the oracle's numpy
restatement (oracle/image_codecs.py). Deflate streams come from Python's
zlib in all three block types. Decoding is bit-exact.
"""
import os
import zlib

import numpy as np
import pytest

from oracle import image_codecs, obj_import
from raym0nade_gb300 import _lib, assets, build, scenes
from tests.golden import image_files as F
from tests.golden import model_files

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def write(tmp_path, name, data):
    p = str(tmp_path / name)
    with open(p, "wb") as f:
        f.write(data)
    return p


def status_of(path, kind, capacity=None):
    """rmn_image_load's status for a file (full decode unless capacity is 0)."""
    lib = _lib.load()
    info = _lib.ImageDesc()
    st = lib.rmn_image_load(os.fsencode(path), kind, info, None, 0)
    if st != 0 or capacity == 0:
        return st
    buf = np.empty(info.width * info.height * info.channels * info.bytes_per_channel if capacity is None
                   else capacity, np.uint8)
    return lib.rmn_image_load(os.fsencode(path), kind, info, buf.ctypes.data, buf.nbytes)


# ------------------------------------------------------------------ PNG ----
PNG_CASES = [(0, 1), (0, 2), (0, 4), (0, 8), (0, 16), (2, 8), (2, 16), (3, 1), (3, 2), (3, 4), (3, 8),
             (4, 8), (4, 16), (6, 8), (6, 16)]
DEFLATE = [(0, zlib.Z_DEFAULT_STRATEGY), (1, zlib.Z_FIXED), (9, zlib.Z_DEFAULT_STRATEGY), (6, zlib.Z_RLE)]


@pytest.mark.parametrize("ctype,depth", PNG_CASES)
def test_png_every_colour_type(tmp_path, ctype, depth):
    """Every colour type and bit depth, all five filters, stored / fixed /
    dynamic deflate blocks, split IDAT chunks, Adam7 interlacing, sizes
    not a multiple of the pass spacing."""
    rng = np.random.default_rng(100 * ctype + depth)
    maxv = (1 << depth) - 1
    for k, ((h, w), interlace, (level, strategy)) in enumerate(
            [((1, 1), False, DEFLATE[0]), ((7, 13), True, DEFLATE[1]), ((17, 33), False, DEFLATE[2]),
             ((9, 6), True, DEFLATE[3]), ((12, 40), True, DEFLATE[2])]):
        pal = None
        if ctype == 3:
            pal = rng.integers(0, 256, (int(rng.integers(1, maxv + 2)), 3))  # indices may pass its end
        s = rng.integers(0, maxv + 1, (h, w, F.PNG_CHANNELS[ctype]))
        if k == 2:
            s[:, : w // 2] = s[0, 0]  # long runs for back-references
        data = F.encode_png(s, ctype, depth, palette=pal, filters=(0, 1, 2, 3, 4, 4, 3), level=level,
                            strategy=strategy, interlace=interlace, idat_split=23,
                            trns=b"\x00\x10" if ctype == 0 else None)
        got = assets.load_png(write(tmp_path, f"t{k}.png", data))
        assert got.dtype == np.uint8 and got.shape == (h, w, 3)
        assert np.array_equal(got, F.png_expected_rgb(s, ctype, depth, pal)), (h, w, interlace, level)


def test_png_large_image_dynamic_blocks(tmp_path):
    """A 300 x 211 RGBA image compressed into several dynamic blocks
    (codes longer than the decoder's 12-bit look-up table included)."""
    rng = np.random.default_rng(7)
    s = (rng.integers(0, 8, (211, 300, 4)) * rng.integers(1, 30, (211, 300, 4))).astype(np.int64) % 256
    s[50:90] = s[40]  # rows that repeat
    data = F.encode_png(s, 6, 8, filters=(1, 4, 2, 0, 3), level=9)
    got = assets.load_png(write(tmp_path, "big.png", data))
    assert np.array_equal(got, s[..., :3].astype(np.uint8))


def test_png_back_references_of_every_short_period(tmp_path):
    """Deflate matches whose distance is below, at and above 8 bytes, long
    and short, some ending on the last byte of the image data: gray rows
    that repeat a random pattern of 1-17 bytes."""
    rng = np.random.default_rng(11)
    for period in range(1, 18):
        for w in (period + 1, 19, 40, 263, 600):
            pattern = rng.integers(0, 256, period)
            h = int(rng.integers(1, 4))
            s = np.resize(pattern, (h, w, 1))
            data = F.encode_png(s, 0, 8, filters=(0,), level=9)
            got = assets.load_png(write(tmp_path, "p.png", data))
            assert np.array_equal(got, np.repeat(s, 3, axis=2).astype(np.uint8)), (period, w, h)


def test_png_large_stream_defects_in_order(tmp_path):
    """Images with more than 1 MiB of scanlines, whose rows the library
    unfilters while the stream still inflates: the stream's defects are
    reported before a row's, as when everything is inflated first -- a bad
    filter byte in an early row with a wrong checksum gives the checksum
    error, alone it gives the filter error, and a stream cut short is
    reported as such."""
    rng = np.random.default_rng(12)
    h, w = 400, 1024  # 400 x (1 + 3072) bytes of scanlines
    s = rng.integers(0, 256, (h, w, 3))
    good = F.encode_png(s, 2, 8, filters=(1, 4, 2), level=6)
    assert np.array_equal(assets.load_png(write(tmp_path, "ok.png", good)), s.astype(np.uint8))
    sig, ihdr = good[:8], good[8:33]
    rows = b"".join(bytes([4]) + s[y].astype(np.uint8).tobytes() for y in range(h))

    def png(raw, z=None):
        z = zlib.compress(raw, 6) if z is None else z
        return sig + ihdr + F._chunk(b"IDAT", z) + F._chunk(b"IEND", b"")

    bad_row = bytearray(rows)
    bad_row[3 * (1 + 3 * w)] = 9  # row 3's filter byte
    with pytest.raises(assets.ImageError, match="bad filter type 9"):
        assets.load_png(write(tmp_path, "f.png", png(bytes(bad_row))))
    z = bytearray(zlib.compress(bytes(bad_row), 6))
    z[-1] ^= 1  # and the Adler-32 wrong
    with pytest.raises(assets.ImageError, match="zlib checksum mismatch"):
        assets.load_png(write(tmp_path, "c.png", png(None, bytes(z))))
    z = zlib.compress(rows[: len(rows) // 2], 6)  # half the scanlines
    with pytest.raises(assets.ImageError, match="less image data"):
        assets.load_png(write(tmp_path, "s.png", png(None, z)))
    z = zlib.compress(bytes(bad_row), 6)
    with pytest.raises(assets.ImageError, match="truncated"):
        assets.load_png(write(tmp_path, "t.png", png(None, z[: len(z) // 3])))


def test_png_reads_what_save_png_writes(tmp_path):
    lib = _lib.load()
    rng = np.random.default_rng(3)
    rgb = rng.uniform(-0.2, 1.2, (37, 70, 3)).astype(np.float32)
    rgb[0, 0] = np.nan
    p = str(tmp_path / "saved.png")
    assert lib.rmn_save_png(rgb.ctypes.data, 70, 37, p.encode()) == 0
    want = np.where(np.isnan(rgb), 0, np.clip(rgb * np.float32(255), 0, 255)).astype(np.uint8)
    assert np.array_equal(assets.load_png(p), want)


def test_png_rejects_malformed_files(tmp_path):
    s = np.arange(48).reshape(4, 4, 3) * 5
    good = F.encode_png(s, 2, 8)
    assert status_of(write(tmp_path, "ok.png", good), assets.PNG) == 0
    bad_sig = b"\x88" + good[1:]
    assert status_of(write(tmp_path, "sig.png", bad_sig), assets.PNG) == 1
    ihdr_crc = bytearray(good)
    ihdr_crc[29] ^= 1  # a byte of IHDR's CRC
    assert status_of(write(tmp_path, "crc.png", bytes(ihdr_crc)), assets.PNG) == 1
    assert status_of(write(tmp_path, "short.png", good[:-20]), assets.PNG) == 1
    # a damaged deflate stream (fixed CRC so that only zlib notices)
    z = zlib.compress(b"\x00" + bytes(12) * 4)
    z = z[:-4] + bytes([z[-4] ^ 0xFF]) + z[-3:]  # Adler-32 wrong
    sig, ihdr = good[:8], good[8:33]
    idat = F._chunk(b"IDAT", z)
    assert status_of(write(tmp_path, "adler.png", sig + ihdr + idat + F._chunk(b"IEND", b"")), assets.PNG) == 1
    too_little = F._chunk(b"IDAT", zlib.compress(bytes(10)))
    assert status_of(write(tmp_path, "little.png", sig + ihdr + too_little + F._chunk(b"IEND", b"")),
                     assets.PNG) == 1
    crit = F._chunk(b"ABCD", b"xyz")  # an unknown critical chunk
    assert status_of(write(tmp_path, "crit.png", sig + ihdr + crit + good[33:]), assets.PNG) == 4
    pal_missing = F.encode_png(np.zeros((2, 2, 1), np.int64), 3, 8, palette=None)
    assert status_of(write(tmp_path, "nopal.png", pal_missing), assets.PNG) == 1
    p = write(tmp_path, "cap.png", good)
    assert status_of(p, assets.PNG, capacity=47) == 1
    assert status_of(str(tmp_path / "missing.png"), assets.PNG) == 1
    with pytest.raises(assets.ImageError) as e:
        assets.load_png(str(tmp_path / "sig.png"))
    assert e.value.status == 1 and "not a PNG" in str(e.value)


# ------------------------------------------------------------------ HDR ----
@pytest.mark.parametrize("h,w", [(5, 7), (9, 40), (3, 300), (2, 8)])
def test_hdr_flat_and_run_length(tmp_path, h, w):
    rng = np.random.default_rng(h * w)
    f = np.exp(rng.normal(0.0, 6.0, (h, w, 3))).astype(np.float32)
    f[0, 0] = 0.0
    f[-1, :] = f[-1, 0]  # runs
    f[0, 1] = 1e-38      # exponent near the bottom of the range
    rgbe = F.float_to_rgbe(f)
    want = F.rgbe_expected(rgbe)
    for rle, flat_from in [(True, None), (False, None), (True, 1)]:
        p = write(tmp_path, "t.hdr", F.encode_hdr(rgbe, rle, flat_from))
        W, H, C, arr = assets.hdr_to_array(p)
        assert (W, H, C) == (w, h, 3) and arr.dtype == np.float32
        assert np.array_equal(arr, want)
    # RGBE keeps 8 mantissa bits of the largest component (Ward's encoder
    # writes pixels below 1e-32 as black)
    peak = f.max(-1, keepdims=True)
    assert (np.abs(want - f) <= np.where(peak > 1e-32, peak / 128.0, 1e-32)).all()


def test_hdr_rejects_and_unsupported(tmp_path):
    rgbe = F.float_to_rgbe(np.ones((4, 16, 3), np.float32))
    assert status_of(write(tmp_path, "ok.hdr", F.encode_hdr(rgbe)), assets.HDR) == 0
    crlf = F.encode_hdr(rgbe, header=b"#?RADIANCE\r\nFORMAT=32-bit_rle_rgbe\r\n\r\n").replace(b"+X 16\n", b"+X 16\r\n")
    assert status_of(write(tmp_path, "crlf.hdr", crlf), assets.HDR) == 0
    xyze = F.encode_hdr(rgbe, header=b"#?RADIANCE\nFORMAT=32-bit_rle_xyze\n\n")
    assert status_of(write(tmp_path, "xyze.hdr", xyze), assets.HDR) == 4
    rot = F.encode_hdr(rgbe).replace(b"-Y 4 +X 16", b"+Y 4 +X 16")
    assert status_of(write(tmp_path, "rot.hdr", rot), assets.HDR) == 4
    assert status_of(write(tmp_path, "cut.hdr", F.encode_hdr(rgbe)[:-5]), assets.HDR) == 1
    assert status_of(write(tmp_path, "notrad.hdr", b"P6\n4 4\n255\n" + bytes(48)), assets.HDR) == 1
    bad = bytearray(F.encode_hdr(rgbe))
    start = bad.index(b"+X 16\n") + 6
    bad[start + 4] = 200  # a run longer than the scanline
    assert status_of(write(tmp_path, "run.hdr", bytes(bad)), assets.HDR) == 1
    wrong_width = bytearray(F.encode_hdr(rgbe))
    wrong_width[start + 3] = 15
    assert status_of(write(tmp_path, "ww.hdr", bytes(wrong_width)), assets.HDR) == 1


# ------------------------------------------------------------------ DDS ----
@pytest.mark.parametrize("kind,fourcc", [(1, b"DXT1"), (2, b"DXT3"), (3, b"DXT5")])
def test_dds_blocks_match_oracle(tmp_path, kind, fourcc):
    rng = np.random.default_rng(kind)
    size = 8 if kind == 1 else 16
    for h, w in [(4, 4), (7, 13), (64, 32), (1, 2)]:
        n = ((w + 3) // 4) * ((h + 3) // 4)
        pay = rng.integers(0, 256, n * size).astype(np.uint8)
        if kind == 1:  # both orders of the endpoints, and equal endpoints
            pay.reshape(n, 8)[: n // 3, 0:2] = pay.reshape(n, 8)[: n // 3, 2:4]
        pay = pay.tobytes()
        W, H, C, data = assets.dds_to_array(write(tmp_path, "t.dds", F.encode_dds(w, h, pay, fourcc)))
        assert (W, H, C) == (w, h, 4) and isinstance(data, bytes)
        got = np.frombuffer(data, np.uint8).reshape(h, w, 4)
        assert np.array_equal(got, image_codecs.bc_decode(pay, w, h, kind))


def test_dds_known_answers(tmp_path):
    """Blocks whose interpolants are exact: red 0xF800 and blue 0x001F give
    (170, 0, 85) and (85, 0, 170) in four-colour mode; BC1 three-colour
    mode's index 3 is transparent black; BC3 alpha 252/0 in sevenths."""
    idx = bytes([0xE4, 0xE4, 0xE4, 0xE4])  # each row: indices 0, 1, 2, 3
    four = bytes([0x00, 0xF8, 0x1F, 0x00]) + idx
    W, H, C, data = assets.dds_to_array(write(tmp_path, "a.dds", F.encode_dds(4, 4, four, b"DXT1")))
    img = np.frombuffer(data, np.uint8).reshape(4, 4, 4)
    row = [[255, 0, 0, 255], [0, 0, 255, 255], [170, 0, 85, 255], [85, 0, 170, 255]]
    assert all(np.array_equal(img[r], row) for r in range(4))
    three = bytes([0x1F, 0x00, 0x00, 0xF8]) + idx  # color0 < color1
    img = np.frombuffer(assets.dds_to_array(write(tmp_path, "b.dds", F.encode_dds(4, 4, three, b"DXT1")))[3],
                        np.uint8).reshape(4, 4, 4)
    assert np.array_equal(img[0, 3], [0, 0, 0, 0]) and np.array_equal(img[0, 1], [255, 0, 0, 255])
    # BC3: a0 = 252, a1 = 0 (sevenths exact), indices 0..7 twice
    bits = sum((t % 8) << (3 * t) for t in range(16))
    alpha = bytes([252, 0]) + bits.to_bytes(6, "little")
    blk = alpha + four
    img = np.frombuffer(assets.dds_to_array(write(tmp_path, "c.dds", F.encode_dds(4, 4, blk, b"DXT5")))[3],
                        np.uint8).reshape(4, 4, 4)
    assert list(img[:2, :, 3].reshape(-1)) == [252, 0, 216, 180, 144, 108, 72, 36] * 1
    assert np.array_equal(img[0, :, :3], np.array(row)[:, :3])


def test_dds_uncompressed(tmp_path):
    rng = np.random.default_rng(5)
    px = rng.integers(0, 256, (5, 6, 4)).astype(np.uint8)  # B, G, R, A in memory
    bgra = px.tobytes()
    masks = (0x00FF0000, 0x0000FF00, 0x000000FF, 0xFF000000)
    d = F.encode_dds(6, 5, bgra, bitcount=32, masks=masks, alpha_flag=True)
    W, H, C, data = assets.dds_to_array(write(tmp_path, "a.dds", d))
    img = np.frombuffer(data, np.uint8).reshape(5, 6, 4)
    assert C == 4 and np.array_equal(img, px[..., [2, 1, 0, 3]])
    d = F.encode_dds(6, 5, bgra, bitcount=32, masks=masks[:3] + (0,), alpha_flag=False)
    img = np.frombuffer(assets.dds_to_array(write(tmp_path, "b.dds", d))[3], np.uint8).reshape(5, 6, 4)
    assert np.array_equal(img[..., :3], px[..., [2, 1, 0]]) and (img[..., 3] == 255).all()
    bgr = px[..., :3].tobytes()
    d = F.encode_dds(6, 5, bgr, bitcount=24, masks=masks[:3] + (0,))
    W, H, C, data = assets.dds_to_array(write(tmp_path, "c.dds", d))
    assert C == 3 and np.array_equal(np.frombuffer(data, np.uint8).reshape(5, 6, 3), px[..., [2, 1, 0]])


def test_dds_rejects_and_unsupported(tmp_path, capsys):
    blk = bytes(16)
    assert status_of(write(tmp_path, "dx10.dds", F.encode_dds(4, 4, blk, b"DX10")), assets.DDS) == 4
    assert status_of(write(tmp_path, "dxt2.dds", F.encode_dds(4, 4, blk, b"DXT2")), assets.DDS) == 4
    d16 = F.encode_dds(4, 4, bytes(32), bitcount=16, masks=(0xF800, 0x07E0, 0x001F, 0))
    assert status_of(write(tmp_path, "r16.dds", d16), assets.DDS) == 4
    assert status_of(write(tmp_path, "cut.dds", F.encode_dds(8, 8, blk, b"DXT5")), assets.DDS) == 1
    assert status_of(write(tmp_path, "magic.dds", b"DDX " + F.encode_dds(4, 4, blk, b"DXT5")[4:]), assets.DDS) == 1
    # the script mirrors' failure convention
    assert assets.dds_to_array(str(tmp_path / "cut.dds")) == (None, None, None, None)
    assert assets.hdr_to_array(str(tmp_path / "nothing.hdr")) == (None, None, None, None)
    out = capsys.readouterr().out
    assert out.count("Conversion failed: ") == 2


def test_image_load_argument_checks(tmp_path):
    lib = _lib.load()
    p = write(tmp_path, "ok.hdr", F.encode_hdr(F.float_to_rgbe(np.ones((2, 9, 3), np.float32))))
    info = _lib.ImageDesc()
    assert lib.rmn_image_load(os.fsencode(p), 7, info, None, 0) == 1
    assert lib.rmn_image_load(None, 2, info, None, 0) == 1
    assert lib.rmn_image_load(os.fsencode(p), 2, None, None, 0) == 1
    assert lib.rmn_image_load(os.fsencode(p), 2, info, None, 0) == 0
    assert (info.width, info.height, info.channels, info.bytes_per_channel) == (9, 2, 3, 4)


def test_golden_image_files():
    """Committed files (tests/golden/images/, made by make_golden.py --images)
    against their committed decoded arrays."""
    z = np.load(os.path.join(GOLDEN, "images.npz"))
    d = os.path.join(GOLDEN, "images")
    kinds = {"png": assets.PNG, "dds": assets.DDS, "hdr": assets.HDR}
    names = sorted(os.listdir(d))
    assert len(names) == len(z.files) >= 6
    for name in names:
        got = assets.load_image(os.path.join(d, name), kinds[name.rsplit(".", 1)[1]])
        assert np.array_equal(got, z[name]), name


# ------------------------------------------------------------- importer ----
def test_load_texture_dispatch(tmp_path, capsys):
    s = np.arange(2 * 3 * 3).reshape(2, 3, 3) * 9
    write(tmp_path, "a.PNG", F.encode_png(s, 2, 8))
    t = assets.load_texture(str(tmp_path / "a.PNG"))
    assert t.shape == (2, 3, 4) and (t[..., 3] == 255).all() and np.array_equal(t[..., :3], s)
    write(tmp_path, "a.jpg", b"\xff\xd8")
    assert assets.load_texture(str(tmp_path / "a.jpg")) is None
    assert "Unsupported file format: " in capsys.readouterr().out
    assert obj_import.url_decode("a%20b\\c%2f%41") == "a b\\c/A"


def test_load_model_obj_room(tmp_path, capfd):
    folder = str(tmp_path) + "/"
    exp = model_files.write_room(folder)
    sc = assets.load_model(folder, "room.obj", "sky.hdr")
    sc.check()
    assert "Unsupported file format: " in capfd.readouterr().err  # the .tga
    assert sc.material_names == exp["materials"]
    # one mesh per run of faces with the same object and material
    want_mats = [m for m, _ in exp["meshes"]]
    assert [sc.material_names[i] for i in sc.mesh_material] == want_mats
    tris = [sum(len(p) - 2 for p in polys) for _, polys in exp["meshes"]]
    assert list(np.diff(sc.mesh_first)) == tris
    # a vertex per face corner, fans from the first corner
    k = 0
    for (mat, polys), first in zip(exp["meshes"], sc.mesh_first[:-1]):
        t = first
        for poly in polys:
            for j in range(1, len(poly) - 1):
                tri = sc.indices[t]
                for c, corner in zip(tri, (poly[0], poly[j], poly[j + 1])):
                    np.testing.assert_allclose(sc.positions[c], corner[0], atol=1e-6)
                    np.testing.assert_allclose(sc.uvs[c], corner[1] if corner[1] is not None else (0, 0), atol=1e-6)
                t += 1
        k += 1
    assert sc.positions.shape[0] == sum(len(p) for _, polys in exp["meshes"] for p in polys)
    # normals: given ones kept, missing ones geometric, the inward cube flipped
    m_glow = want_mats.index("Glow")
    a, b = sc.mesh_first[m_glow], sc.mesh_first[m_glow + 1]
    nrm = sc.normals[sc.indices[a:b].reshape(-1)]
    assert np.allclose(np.abs(nrm[:, 1]), 1.0)
    m_odd = want_mats.index("Odd")
    c = sc.indices[sc.mesh_first[m_odd]:sc.mesh_first[m_odd + 1]].reshape(-1)
    outward = sc.positions[c] - np.array([0.0, 0.0, 10.0], np.float32)
    assert ((sc.normals[c] * outward).sum(1) > 0).all()
    m_walls = want_mats.index("Walls")
    c = sc.indices[sc.mesh_first[m_walls]:sc.mesh_first[m_walls + 1]].reshape(-1)
    assert np.allclose(sc.normals[c][:2], [0, 1, 0])  # the floor's, as written
    # materials: white, roughness 0.8, no constant texels; Water is glass
    names = sc.material_names
    w = sc.materials[names.index("Water")]
    assert (w[11], w[12], w[8]) == (0.0, np.float32(1.25), np.float32(5e-3)) and list(w[13:16]) == [1, 1, 1]
    assert sc.materials[names.index("Unused")][11] == 1.0
    for i in range(len(names)):
        if names[i] != "Water":
            assert list(sc.materials[i][[0, 1, 2, 3, 7, 8, 10, 11]]) == [1, 1, 1, 0, 0, np.float32(0.8), 0, 1]
    # textures: slots, RGBA expansion of RGB files, decoded DDS blocks
    mt = sc.mat_tex
    walls = mt[names.index("Walls")]
    assert np.array_equal(sc.textures[walls[0]][..., :3], exp["checker"])
    assert (sc.textures[walls[0]][..., 3] == 255).all()
    assert np.array_equal(sc.textures[walls[1]], image_codecs.bc_decode(exp["spec"], 16, 16, 1))
    assert walls[2] == -1 and np.array_equal(sc.textures[walls[3]][..., :3], exp["normal"])
    assert np.array_equal(sc.textures[mt[names.index("Glow"), 2]], image_codecs.bc_decode(exp["glow"], 8, 8, 3))
    leaf = sc.textures[mt[names.index("Leaf"), 0]]
    assert (leaf[:, :4, 3] == 0).all() and (leaf[:, 4:, 3] == 255).all()
    assert (mt[names.index("Odd")] == -1).all() and (mt[names.index("Plain")] == -1).all()
    assert np.array_equal(sc.env, exp["sky"])
    # without a sky map, and with one that fails to decode
    assert assets.load_model(folder, "room.obj").env is None
    write(tmp_path, "bad.hdr", b"#?RADIANCE\n")
    assert assets.load_model(folder, "room.obj", "bad.hdr").env is None
    assert "Conversion failed" in capfd.readouterr().err


def test_load_model_without_mtl_or_normals(tmp_path):
    obj = "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nusemtl Missing\nf 1 2 3 4\n"
    write(tmp_path, "q.obj", obj.encode())
    sc = assets.load_model(str(tmp_path) + "/", "q.obj")
    sc.check()
    assert sc.material_names == ["DefaultMaterial", "Missing"] and list(sc.mesh_material) == [1]
    assert np.allclose(sc.normals, [0, 0, 1]) and sc.textures is None and sc.mat_tex is None
    write(tmp_path, "e.obj", b"v 0 0 0\nl 1 1\n")
    with pytest.raises(ValueError):
        assets.load_model(str(tmp_path) + "/", "e.obj")
    # tabs, a continued line, and the errors a broken file gives (with its line)
    write(tmp_path, "t.obj", b"v\t0 0 0\nv 1 0 0\nv 0 1 \\\n 0\nf\t1 2 3\n")
    sc = assets.load_model(str(tmp_path) + "/", "t.obj")
    assert sc.num_triangles == 1 and np.allclose(sc.positions[2], [0, 1, 0])
    for bad, where in [(b"v 0 0\n", ":1:"), (b"v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 x\n", ":4:")]:
        write(tmp_path, "b.obj", bad)
        with pytest.raises(ValueError, match=where):
            assets.load_model(str(tmp_path) + "/", "b.obj")
    write(tmp_path, "c.obj", b"v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//2 3//1\n")
    with pytest.raises(ValueError, match="does not exist"):
        assets.load_model(str(tmp_path) + "/", "c.obj")


def test_imported_model_oracle_matches_reference(port, ref_tex, tmp_path):
    """The imported room (PNG/DDS textures, alpha cut-outs, glass, emissive
    DDS light, HDR sky) in the oracle and in the reference built with its own
    src/material.cpp: identical light objects, ray queries and paths."""
    folder = str(tmp_path) + "/"
    model_files.write_room(folder)
    for sky in ("sky.hdr", "null"):
        sc = assets.load_model(folder, "room.obj", sky)
        ps, rs = port.scene(sc), ref_tex.scene(sc)
        assert np.array_equal(ps.lights(), rs.lights())
        cam = model_files.room_camera(40, 30, 8)
        a, b = ps.render(cam, seed=13), rs.render(cam, seed=13)
        assert np.array_equal(a[..., :38], b[..., :38], equal_nan=True)
        ids = set(np.unique(a[..., 36][~np.isnan(a[..., 36])]).astype(int))
        assert {1, 3, 4, 5} <= ids  # walls, glass, cut-out leaf, box in view


def same_scene(a, b):
    for k in ("positions", "normals", "uvs", "indices", "mesh_first", "mesh_material", "materials"):
        x, y = getattr(a, k), getattr(b, k)
        assert x.dtype == y.dtype and np.array_equal(x, y, equal_nan=True), k
    assert a.material_names == b.material_names
    assert (a.env is None) == (b.env is None) and (a.env is None or np.array_equal(a.env, b.env))
    assert (a.textures is None) == (b.textures is None)
    if a.textures is not None:
        assert len(a.textures) == len(b.textures) and np.array_equal(a.mat_tex, b.mat_tex)
        assert all(np.array_equal(x, y) for x, y in zip(a.textures, b.textures))


def test_native_importer_matches_oracle(tmp_path, capfd):
    """rmn_model_read against the oracle's restatement (oracle/obj_import.py,
    with the oracle's own image readers): identical arrays."""
    folder = str(tmp_path) + "/"
    model_files.write_room(folder)
    for sky in ("sky.hdr", "null"):
        same_scene(assets.load_model(folder, "room.obj", sky), obj_import.load_model(folder, "room.obj", sky))


def _random_obj(rng, path, parts=(3, 8)):
    """Random OBJ text: objects, groups, material switches, polygons of 3-6
    corners with every corner form and negative indices, degenerate faces,
    normals pointing anywhere (the infacing test), comments, tabs, CRLF line
    ends, continued lines, lines and points."""
    out = ["mtllib lib.mtl", "# random model"]
    nv = nt = nn = 0
    mats = ["A", "B", "Glass", "Water", "Nope"]
    for k in range(int(rng.integers(*parts))):
        out.append(("o" if rng.random() < 0.5 else "g") + f" part{k}")
        for _ in range(int(rng.integers(4, 12))):
            out.append("v %.7g %.7g %.7g" % tuple(rng.normal(0, 2, 3) * 10.0 ** int(rng.integers(-2, 3))))
            nv += 1
            out.append("vt\t%.5f %.5f" % tuple(rng.uniform(-1, 2, 2)))
            nt += 1
            if rng.random() < 0.8:
                out.append("vn %.6f %.6f %.6f" % tuple(rng.normal(0, 1, 3)))
                nn += 1
        form = int(rng.integers(0, 4))
        for f in range(int(rng.integers(2, 9))):
            if rng.random() < 0.3:
                out.append("usemtl " + mats[int(rng.integers(0, len(mats)))])
            n = int(rng.integers(3, 7))
            toks = []
            for _ in range(n):
                vi = int(rng.integers(1, nv + 1))
                ti = int(rng.integers(1, nt + 1))
                ni = int(rng.integers(1, nn + 1)) if nn else 0
                if rng.random() < 0.3:
                    vi, ti = vi - nv - 1, ti - nt - 1
                toks.append([f"{vi}", f"{vi}/{ti}", f"{vi}//{ni}" if ni else f"{vi}/{ti}",
                             f"{vi}/{ti}/{ni}" if ni else f"{vi}/{ti}"][form])
            out.append("f " + " ".join(toks))
            if rng.random() < 0.1:
                out.append("l 1 2")
            if rng.random() < 0.1:
                out[-1] = out[-1] + " \\"
                out.append("")
    text = "\r\n".join(out) if rng.random() < 0.5 else "\n".join(out)
    with open(path, "w", newline="") as f:
        f.write(text + "\n")


def test_native_importer_matches_oracle_random_models(tmp_path):
    rng = np.random.default_rng(77)
    folder = str(tmp_path) + "/"
    with open(folder + "lib.mtl", "w") as f:
        f.write("newmtl A\nd 1\nnewmtl B\nTr 0.5\nnewmtl Glass\n  d\t0.2\nnewmtl Water\nd 0.995\n")
    for k in range(40):
        _random_obj(rng, folder + f"m{k}.obj")
        same_scene(assets.load_model(folder, f"m{k}.obj"), obj_import.load_model(folder, f"m{k}.obj"))


def test_native_importer_large_random_models(tmp_path):
    """Files of several hundred KB, which the library parses in pieces on
    separate threads: negative indices, material switches, objects and
    continued lines across the pieces' seams give the oracle's arrays; a bad
    statement in a late piece is reported with its line in the whole file."""
    rng = np.random.default_rng(78)
    folder = str(tmp_path) + "/"
    with open(folder + "lib.mtl", "w") as f:
        f.write("newmtl A\nd 1\nnewmtl B\nTr 0.5\nnewmtl Glass\n  d\t0.2\nnewmtl Water\nd 0.995\n")
    for k in range(3):
        _random_obj(rng, folder + f"big{k}.obj", parts=(900, 1000))
        assert os.path.getsize(folder + f"big{k}.obj") > 8 * 64 * 1024
        same_scene(assets.load_model(folder, f"big{k}.obj"), obj_import.load_model(folder, f"big{k}.obj"))
    lines = open(folder + "big0.obj", newline="").read().splitlines()
    at = len(lines) - 5
    while not lines[at].startswith("v "):
        at -= 1
    lines[at] = "v 1.0 oops 2.0"
    with open(folder + "bad.obj", "w", newline="") as f:
        f.write("\n".join(lines) + "\n")
    # lines as a reader counts them: a backslash at the end of a line joins the next
    line_no = ("\n".join(lines[:at]) + "\n").replace("\\\n", " ").count("\n") + 1
    with pytest.raises(ValueError, match=f"bad.obj:{line_no}: cannot read 'v 1.0 oops 2.0'"):
        assets.load_model(folder, "bad.obj")


@pytest.mark.parametrize("kind", ["smooth", "noise", "tiles", "tiny", "flat", "large"])
def test_save_png_compresses_and_round_trips(tmp_path, kind):
    """rmn_save_png's deflate stream: read back by Python's zlib (through
    the oracle's reader) and by the library's own decoder, pixel for pixel;
    smooth and repetitive images shrink, noise falls back to stored blocks.
    "large" (1080 x 1920) is filtered and compressed in pieces on several
    threads, the stream's segments joined by empty stored blocks."""
    lib = _lib.load()
    rng = np.random.default_rng(5)
    h, w = {"tiny": (1, 2), "tiles": (300, 700), "large": (1080, 1920)}.get(kind, (240, 320))
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float32)
    if kind == "smooth":
        img = np.stack([xx / w, yy / h, (xx + yy) / (w + h)], -1)
    elif kind == "noise":
        img = rng.random((h, w, 3), dtype=np.float32)
    elif kind == "tiles":
        tile = rng.random((20, 37, 3), dtype=np.float32)
        img = np.tile(tile, (h // 20 + 1, w // 37 + 1, 1))[:h, :w]
    elif kind == "flat":
        img = np.full((h, w, 3), 0.25, np.float32)
    elif kind == "large":  # a gradient with mild noise and a repeated band (matches across segments)
        img = np.stack([xx / w, yy / h, (xx + yy) / (w + h)], -1) + rng.normal(0, 0.01, (h, w, 3))
        img[500:560] = img[100:160]
    else:
        img = rng.random((h, w, 3), dtype=np.float32)
    img = np.ascontiguousarray(img, np.float32)
    p = str(tmp_path / f"{kind}.png")
    assert lib.rmn_save_png(img.ctypes.data, w, h, p.encode()) == 0
    want = np.clip(img * np.float32(255), 0, 255).astype(np.uint8)
    assert np.array_equal(image_codecs.png_read(p), want)
    assert np.array_equal(assets.load_png(p), want)
    data, at, chunks = open(p, "rb").read(), 8, 0
    while at < len(data):  # every chunk's CRC-32 as zlib computes it
        n = int.from_bytes(data[at:at + 4], "big")
        assert int.from_bytes(data[at + 8 + n:at + 12 + n], "big") == zlib.crc32(data[at + 4:at + 8 + n])
        at, chunks = at + 12 + n, chunks + 1
    assert at == len(data) and chunks >= 3
    size, raw = os.path.getsize(p), h * (1 + 3 * w)
    if kind in ("smooth", "flat"):
        assert size < 0.1 * raw
    if kind == "tiles":
        assert size < 0.2 * raw
    if kind == "large":
        assert size < 0.6 * raw
    if kind == "noise":
        assert size < raw * 1.01 + 200


def test_native_importer_many_textures(tmp_path, capfd):
    """Texture files decoded on several threads: indices in order of first
    use, shared files once, a missing DDS and an unsupported type left out
    with the reference's messages -- as the oracle's one-by-one loading."""
    rng = np.random.default_rng(2)
    folder = str(tmp_path) + "/"
    mtl = []
    for k in range(24):
        pay = rng.integers(0, 256, (64 // 4) * (48 // 4) * 16).astype(np.uint8).tobytes()
        (tmp_path / f"t{k}.dds").write_bytes(F.encode_dds(64, 48, pay, b"DXT5"))
        mtl.append(f"newmtl m{k}\nmap_Kd t{k}.dds\nmap_Ks t{(k * 7) % 24}.dds\n")
    mtl.append("newmtl bad\nmap_Kd missing.dds\nmap_Ks x.tga\n")
    (tmp_path / "m.mtl").write_text("".join(mtl))
    obj = "mtllib m.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\n" + "".join(f"usemtl m{k}\nf 1 2 3\n" for k in range(24))
    (tmp_path / "m.obj").write_text(obj + "usemtl bad\nf 1 2 3\n")
    same_scene(assets.load_model(folder, "m.obj"), obj_import.load_model(folder, "m.obj"))
    err = capfd.readouterr().err
    assert "Unsupported file format: " in err and "Conversion failed: " in err


def test_model_from_file_goes_native_to_scene_create(tmp_path):
    """api.Model(folder, name, sky) hands rmn_model_read's description
    straight to rmn_scene_create: it builds on a GPU, and without one it gets
    as far as the first device allocation (the description passes every
    argument check)."""
    from raym0nade_gb300 import api
    folder = str(tmp_path) + "/"
    model_files.write_room(folder)
    try:
        m = api.Model(folder, "room.obj", "sky.hdr")
    except api.RmnError as e:
        assert e.status == 2, str(e)  # RMN_ERR_CUDA: no device here
    else:
        assert m.num_triangles == assets.load_model(folder, "room.obj").num_triangles
        assert m.info()["num_lights"] == 1
    with pytest.raises(ValueError, match="could not read"):
        api.Model(folder, "missing.obj")


def test_decoders_and_importer_survive_mutated_files(tmp_path):
    """Malformed files give a status, never a crash: truncated, bit-flipped
    and spliced copies of the committed images (PNG chunk CRCs repaired so
    the damage reaches inflate and the filters), and of the OBJ/MTL room."""
    import zlib as _z
    rng = np.random.default_rng(99)
    d = os.path.join(GOLDEN, "images")
    kinds = {"png": assets.PNG, "dds": assets.DDS, "hdr": assets.HDR}

    def fix_crcs(b):
        at = 8
        while at + 12 <= len(b):
            n = int.from_bytes(b[at:at + 4], "big")
            if n > len(b) - at - 12:
                break
            b[at + 8 + n:at + 12 + n] = (_z.crc32(bytes(b[at + 4:at + 8 + n])) & 0xFFFFFFFF).to_bytes(4, "big")
            at += 12 + n

    statuses = set()
    for name in sorted(os.listdir(d)):
        kind = kinds[name.rsplit(".", 1)[1]]
        base = open(os.path.join(d, name), "rb").read()
        for _ in range(150):
            b = bytearray(base)
            if rng.random() < 0.3:
                b = b[:int(rng.integers(0, len(b)))]
            for _ in range(int(rng.integers(1, 6))):
                if b:
                    b[int(rng.integers(0, len(b)))] = int(rng.integers(0, 256))
            if kind == assets.PNG and rng.random() < 0.8:
                fix_crcs(b)
            p = write(tmp_path, "m.bin", bytes(b))
            statuses.add(status_of(p, kind))
    assert statuses <= {0, 1, 4} and 1 in statuses
    folder = str(tmp_path) + "/"
    model_files.write_room(folder)
    obj = open(folder + "room.obj").read()
    alphabet = "0123456789 -+./\\\n\tvfnt#%eE"
    for _ in range(150):
        t = list(obj)
        for _ in range(int(rng.integers(1, 8))):
            at = int(rng.integers(0, len(t)))
            op = rng.integers(0, 3)
            if op == 0:
                t[at] = alphabet[int(rng.integers(0, len(alphabet)))]
            elif op == 1:
                del t[at:at + int(rng.integers(1, 20))]
            else:
                t.insert(at, alphabet[int(rng.integers(0, len(alphabet)))])
        with open(folder + "m.obj", "w") as f:
            f.write("".join(t))
        try:
            sc = assets.load_model(folder, "m.obj")
        except ValueError:
            continue
        sc.check()
        assert (sc.indices >= 0).all() and (sc.indices < sc.positions.shape[0]).all()


def test_photo_load_and_reverse_gamma(tmp_path):
    """Photo::load (the PNG's RGB / 255) and reverseGammaCorrection, the
    first steps of the reference's fxaa.cpp tool, on a saved image and on a
    16-bit gray-alpha PNG."""
    from raym0nade_gb300 import api
    rng = np.random.default_rng(4)
    img = rng.random((9, 14, 3), dtype=np.float32)
    p = str(tmp_path / "a.png")
    api.Photo.save(img, p)
    got = api.Photo.load(p)
    want = (img * np.float32(255)).astype(np.uint8).astype(np.float32) / np.float32(255)
    assert got.dtype == np.float32 and np.array_equal(got, want)
    s = rng.integers(0, 65536, (5, 6, 2))
    q = write(tmp_path, "g.png", F.encode_png(s, 4, 16))
    g = api.Photo.load(q)
    assert np.array_equal(g[..., 0], (s[..., 0] >> 8).astype(np.float32) / np.float32(255))
    r = api.Photo.reverseGammaCorrection(got)
    np.testing.assert_allclose(r, np.power(got, np.float32(2.2)), rtol=3e-7, atol=0)
