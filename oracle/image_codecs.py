"""Oracle for the texture front-end. TEST INFRASTRUCTURE ONLY: imported by
tests/ to check rmn_image_load and the device mip chains against, never
by the library.

``mip_chain`` restates ImageData::generateMipmaps (src/material.cpp:107-129)
with its wrapped coordinates and truncating division.

``bc_decode`` restates the S3TC block formats that scripts/dds_to_array.py's
reader (imageio, absent here; the reference pins no version) decodes.

Formats (DirectX "Block compression" documentation, BC1-BC3):
* colour block: two RGB565 endpoints, bit-replicated to 8 bits, and 16
  2-bit indices (texel t at bits 2t); four colours, or for BC1 with
  color0 <= color1 three colours and transparent black;
  interpolants (2a + b) / 3, (a + 2b) / 3 and (a + b) / 2, truncated;
* BC2 alpha: 16 explicit 4-bit values, x 17;
* BC3 alpha: two 8-bit endpoints and 16 3-bit indices; 8 values
  interpolated by sevenths when a0 > a1, else 6 by fifths plus 0 and 255.

Parity unpinned: the rounding of the interpolants is not fixed by the
published format, and the library the reference calls is not available to
pin it; the known-answer tests use endpoints whose interpolants are exact.
"""
from __future__ import annotations

import numpy as np


def _expand565(c):
    r, g, b = (c >> 11) & 31, (c >> 5) & 63, c & 31
    return np.stack([(r << 3) | (r >> 2), (g << 2) | (g >> 4), (b << 3) | (b >> 2)], -1)


def _colour_blocks(blk: np.ndarray, bc1: bool) -> np.ndarray:
    """(n, 8) colour blocks -> (n, 16, 4) RGBA."""
    b = blk.astype(np.int64)
    c0 = b[:, 0] | (b[:, 1] << 8)
    c1 = b[:, 2] | (b[:, 3] << 8)
    e0, e1 = _expand565(c0), _expand565(c1)
    four = (c0 > c1) if bc1 else np.ones(len(b), bool)
    pal = np.zeros((len(b), 4, 4), np.int64)
    pal[:, 0, :3], pal[:, 1, :3] = e0, e1
    pal[:, :, 3] = 255
    pal[:, 2, :3] = np.where(four[:, None], (2 * e0 + e1) // 3, (e0 + e1) // 2)
    pal[:, 3, :3] = np.where(four[:, None], (e0 + 2 * e1) // 3, 0)
    pal[:, 3, 3] = np.where(four, 255, 0)
    idx = b[:, 4] | (b[:, 5] << 8) | (b[:, 6] << 16) | (b[:, 7] << 24)
    sel = (idx[:, None] >> (2 * np.arange(16))) & 3
    return np.take_along_axis(pal, sel[:, :, None].repeat(4, -1), 1)


def bc_decode(payload: bytes, width: int, height: int, kind: int) -> np.ndarray:
    """kind 1/2/3 = BC1/BC2/BC3 (DXT1/3/5) -> (height, width, 4) uint8."""
    size = 8 if kind == 1 else 16
    bw, bh = (width + 3) // 4, (height + 3) // 4
    blk = np.frombuffer(payload, np.uint8)[:bw * bh * size].reshape(bw * bh, size)
    tex = _colour_blocks(blk if kind == 1 else blk[:, 8:], kind == 1)
    a = blk[:, :8].astype(np.int64)
    if kind == 2:
        nib = np.stack([a & 15, a >> 4], -1).reshape(-1, 16)
        tex[:, :, 3] = nib * 17
    elif kind == 3:
        a0, a1 = a[:, 0], a[:, 1]
        k = np.arange(8)
        seven = ((8 - k) * a0[:, None] + (k - 1) * a1[:, None]) // 7
        five = ((6 - k) * a0[:, None] + (k - 1) * a1[:, None]) // 5
        five[:, 6], five[:, 7] = 0, 255
        pal = np.where((a0 > a1)[:, None], seven, five)
        pal[:, 0], pal[:, 1] = a0, a1
        bits = sum(a[:, 2 + i] << (8 * i) for i in range(6))
        sel = (bits[:, None] >> (3 * np.arange(16))) & 7
        tex[:, :, 3] = np.take_along_axis(pal, sel, 1)
    img = tex.reshape(bh, bw, 4, 4, 4).transpose(0, 2, 1, 3, 4).reshape(bh * 4, bw * 4, 4)
    return img[:height, :width].astype(np.uint8)


def mip_chain(tex: np.ndarray, max_levels: int = 8) -> list:
    """ImageData::generateMipmaps: level l is (h >> l, w >> l) texels, each
    channel the truncated mean of the 2 x 2 box of level l-1 at
    ((2y + dy) mod ph, (2x + dx) mod pw); it stops before a side would be 0,
    after at most 8 levels."""
    levels = [np.asarray(tex, np.uint8)]
    h, w = levels[0].shape[:2]
    for level in range(1, max_levels):
        cw, chh = w >> level, h >> level
        if cw == 0 or chh == 0:
            break
        prev = levels[-1].astype(np.int64)
        ph, pw = prev.shape[:2]
        ys, xs = np.arange(chh), np.arange(cw)
        s = 0
        for dy in range(2):
            for dx in range(2):
                s = s + prev[((2 * ys + dy) % ph)[:, None], ((2 * xs + dx) % pw)[None, :]]
        levels.append((s // 4).astype(np.uint8))
    return levels


# ------------------------------------------------------------------ readers
# Independent readers of the three formats (Python's zlib for deflate), so
# the model importer can be checked without the library's decoders.

def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def png_read(path: str) -> np.ndarray:
    """8-bit RGB as Material::loadImageFromPNG's libpng transforms give it."""
    import struct
    import zlib
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n", "not a PNG file"
    at, idat, pal = 8, b"", None
    while True:
        n = struct.unpack(">I", data[at:at + 4])[0]
        kind, body = data[at + 4:at + 8], data[at + 8:at + 8 + n]
        at += 12 + n
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            pal = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"IDAT":
            idat += body
        elif kind == b"IEND":
            break
    raw = zlib.decompress(idat)
    nch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bits = nch * depth
    bpp = max(1, bits // 8)
    passes = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)] \
        if interlace else [(0, 0, 1, 1)]
    out = np.zeros((h, w, 3), np.uint8)
    pos = 0
    for x0, y0, dx, dy in passes:
        if x0 >= w or y0 >= h:
            continue
        cols, rows = (w - x0 + dx - 1) // dx, (h - y0 + dy - 1) // dy
        stride = (cols * bits + 7) // 8
        prev = bytearray(stride)
        for r in range(rows):
            ft, src = raw[pos], raw[pos + 1:pos + 1 + stride]
            pos += 1 + stride
            cur = bytearray(stride)
            for i in range(stride):
                a = cur[i - bpp] if i >= bpp else 0
                b = prev[i]
                c = prev[i - bpp] if i >= bpp else 0
                cur[i] = (src[i] + [0, a, b, (a + b) >> 1, _paeth(a, b, c)][ft]) & 0xFF
            row = np.frombuffer(bytes(cur), np.uint8)
            if depth == 16:
                s = row[0::2][:cols * nch].reshape(cols, nch)
            elif depth == 8:
                s = row[:cols * nch].reshape(cols, nch)
            else:
                bitsarr = np.unpackbits(row)[:cols * depth].reshape(cols, depth)
                s = (bitsarr * (1 << np.arange(depth - 1, -1, -1))).sum(1).reshape(cols, 1)
            s = s.astype(np.int64)
            if ctype == 3:
                full = np.zeros((256, 3), np.int64)
                full[:len(pal)] = pal
                rgb = full[s[:, 0]]
            elif ctype in (0, 4):
                g = s[:, 0] * (255 // ((1 << depth) - 1)) if depth < 8 else s[:, 0]
                rgb = np.stack([g, g, g], 1)
            else:
                rgb = s[:, :3]
            out[y0 + r * dy, x0::dx][:cols] = rgb
            prev = cur
    return out


def dds_read(path: str) -> np.ndarray:
    """scripts/dds_to_array.py's image: BC1-BC3 -> RGBA, 32-bit -> RGBA,
    24-bit -> RGB (8-bit channel masks)."""
    import struct
    data = open(path, "rb").read()
    assert data[:4] == b"DDS " and struct.unpack("<I", data[4:8])[0] == 124, "not a DDS file"
    h, w = struct.unpack("<II", data[12:20])
    flags, fourcc, bitcount = struct.unpack("<I4sI", data[80:92])
    masks = struct.unpack("<IIII", data[92:108])
    pay = data[128:]
    if flags & 0x4:
        return bc_decode(pay, w, h, {b"DXT1": 1, b"DXT3": 2, b"DXT5": 3}[fourcc])
    nb = bitcount // 8
    px = np.frombuffer(pay[:w * h * nb], np.uint8).reshape(h, w, nb).astype(np.uint32)
    v = sum(px[..., k] << (8 * k) for k in range(nb))
    chans = [((v & m) >> (m & -m).bit_length() - 1).astype(np.uint8) for m in masks[:3]]
    if nb == 4:
        alpha = ((v & masks[3]) >> ((masks[3] & -masks[3]).bit_length() - 1)).astype(np.uint8) \
            if (flags & 0x1) and masks[3] else np.full((h, w), 255, np.uint8)
        chans.append(alpha)
    return np.stack(chans, -1)


def hdr_read(path: str) -> np.ndarray:
    """scripts/hdr_to_array.py's float32 RGB: Radiance RGBE, flat or
    run-length scanlines."""
    data = open(path, "rb").read()
    at = 0
    lines = []
    while True:
        end = data.index(b"\n", at)
        lines.append(data[at:end].rstrip(b"\r"))
        at = end + 1
        if len(lines) > 1 and lines[-1] == b"":
            break
    end = data.index(b"\n", at)
    parts = data[at:end].rstrip(b"\r").split()
    h, w = int(parts[1]), int(parts[3])
    at = end + 1
    rgbe = np.zeros((h, w, 4), np.uint8)
    for y in range(h):
        if w < 8 or w > 0x7FFF or data[at] != 2 or data[at + 1] != 2 or data[at + 2] & 0x80:
            rest = np.frombuffer(data[at:at + (h - y) * w * 4], np.uint8).reshape(h - y, w, 4)
            rgbe[y:] = rest
            break
        at += 4
        for ch in range(4):
            x = 0
            while x < w:
                count = data[at]
                at += 1
                if count > 128:
                    rgbe[y, x:x + count - 128, ch] = data[at]
                    at += 1
                    x += count - 128
                else:
                    rgbe[y, x:x + count, ch] = np.frombuffer(data[at:at + count], np.uint8)
                    at += count
                    x += count
    e = rgbe[..., 3].astype(np.int64)
    scale = np.where(e > 0, np.ldexp(1.0, e - 136), 0.0)
    return (rgbe[..., :3].astype(np.float64) * scale[..., None]).astype(np.float32)
