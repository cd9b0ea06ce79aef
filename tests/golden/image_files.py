"""Writers of PNG, Radiance HDR and DDS files for the decoder tests.

Test infrastructure: they produce files whose decoded content is known --
the sample array a PNG was written from, the RGBE bytes of an HDR, the block
bytes of a DDS (decoded by oracle/image_codecs.py) -- so that librmn's
rmn_image_load can be checked against them. Deflate streams come from
Python's zlib (stored, fixed-Huffman and dynamic-Huffman blocks).
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

PNG_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}
ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def _chunk(kind: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)


def _pack_row(row: np.ndarray, depth: int) -> bytes:
    """One row of samples (n,) to bytes at the bit depth (big-endian for 16)."""
    if depth == 8:
        return row.astype(np.uint8).tobytes()
    if depth == 16:
        return row.astype(">u2").tobytes()
    per = 8 // depth
    n = len(row)
    padded = np.zeros(((n + per - 1) // per) * per, np.uint16)
    padded[:n] = row
    g = padded.reshape(-1, per)
    out = np.zeros(g.shape[0], np.uint16)
    for k in range(per):
        out |= g[:, k] << (8 - depth * (k + 1))
    return out.astype(np.uint8).tobytes()


def _filter_row(raw: bytes, prev: bytes, ft: int, bpp: int) -> bytes:
    """PNG filter `ft` of one row (ISO/IEC 15948 section 9): the predictor
    of every byte uses the unfiltered left, up and up-left bytes."""
    x = np.frombuffer(raw, np.uint8).astype(np.int32)
    b = np.frombuffer(prev, np.uint8).astype(np.int32)
    a = np.concatenate([np.zeros(min(bpp, len(x)), np.int32), x[:-bpp]])[:len(x)]
    c = np.concatenate([np.zeros(min(bpp, len(b)), np.int32), b[:-bpp]])[:len(b)]
    if ft == 0:
        pred = np.zeros_like(x)
    elif ft == 1:
        pred = a
    elif ft == 2:
        pred = b
    elif ft == 3:
        pred = (a + b) >> 1
    else:  # Paeth: the neighbour closest to a + b - c, ties in the order a, b, c
        pa, pb, pc = np.abs(b - c), np.abs(a - c), np.abs(a + b - 2 * c)
        pred = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))
    return bytes([ft]) + ((x - pred) & 0xFF).astype(np.uint8).tobytes()


def encode_png(samples: np.ndarray, ctype: int, depth: int, palette=None, trns=None, filters=(0,),
               level: int = 6, strategy: int = zlib.Z_DEFAULT_STRATEGY, interlace: bool = False,
               idat_split: int = 0) -> bytes:
    """A PNG of `samples` (h, w, channels of the colour type; values < 2^depth)."""
    h, w, nch = samples.shape
    assert nch == PNG_CHANNELS[ctype]
    bits = nch * depth
    bpp = max(1, bits // 8)
    passes = ADAM7 if interlace else [(0, 0, 1, 1)]
    raw = bytearray()
    r_index = 0
    for x0, y0, dx, dy in passes:
        sub = samples[y0::dy, x0::dx]
        if sub.shape[0] == 0 or sub.shape[1] == 0:
            continue
        stride = (sub.shape[1] * bits + 7) // 8
        prev = bytes(stride)
        for r in range(sub.shape[0]):
            row = _pack_row(sub[r].reshape(-1), depth)
            raw += _filter_row(row, prev, filters[r_index % len(filters)], bpp)
            r_index += 1
            prev = row
    co = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
    z = co.compress(bytes(raw)) + co.flush()
    out = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, int(interlace)))
    out += _chunk(b"tEXt", b"Comment\x00decoder test")
    if palette is not None:
        out += _chunk(b"PLTE", np.asarray(palette, np.uint8).tobytes())
    if trns is not None:
        out += _chunk(b"tRNS", bytes(trns))
    step = idat_split or len(z) or 1
    for k in range(0, max(len(z), 1), step):
        out += _chunk(b"IDAT", z[k:k + step])
    return out + _chunk(b"IEND", b"")


def png_expected_rgb(samples: np.ndarray, ctype: int, depth: int, palette=None) -> np.ndarray:
    """What Material::loadImageFromPNG's libpng transforms give: 8-bit RGB
    (strip_16 keeps the high byte, gray 1/2/4-bit scales to 8, palette and
    gray expand to RGB, alpha is dropped)."""
    s = samples.astype(np.int64)
    if depth == 16:
        s = s >> 8
    if ctype == 3:
        pal = np.zeros((256, 3), np.int64)
        p = np.asarray(palette, np.int64).reshape(-1, 3)
        pal[:len(p)] = p
        return pal[s[..., 0]].astype(np.uint8)
    if ctype in (0, 4):
        g = s[..., 0] * (255 // ((1 << depth) - 1)) if depth < 8 else s[..., 0]
        return np.repeat(g[..., None], 3, -1).astype(np.uint8)
    return s[..., :3].astype(np.uint8)


def float_to_rgbe(rgb: np.ndarray) -> np.ndarray:
    """Ward's RGBE encoding: the largest component's frexp exponent shared,
    mantissas scaled to [0, 256)."""
    rgb = rgb.astype(np.float64)
    v = rgb.max(-1)
    m, e = np.frexp(v)
    scale = np.where(v > 1e-32, m * 256.0 / np.where(v > 1e-32, v, 1.0), 0.0)
    out = np.zeros(rgb.shape[:-1] + (4,), np.uint8)
    out[..., :3] = np.floor(rgb * scale[..., None]).clip(0, 255).astype(np.uint8)
    out[..., 3] = np.where(v > 1e-32, e + 128, 0).astype(np.uint8)
    return out


def _rle_channel(b: bytes) -> bytes:
    out = bytearray()
    i, n = 0, len(b)
    while i < n:
        run = 1
        while i + run < n and run < 127 and b[i + run] == b[i]:
            run += 1
        if run >= 3:
            out += bytes([128 + run, b[i]])
            i += run
            continue
        j = i  # literal bytes up to the next run of three
        while j < n and j - i < 128 and not (j + 2 < n and b[j] == b[j + 1] == b[j + 2]):
            j += 1
        out += bytes([j - i]) + b[i:j]
        i = j
    return bytes(out)


def encode_hdr(rgbe: np.ndarray, rle: bool = True, flat_from: int | None = None,
               header: bytes = b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\nEXPOSURE=1.0\n\n") -> bytes:
    """A Radiance file of (h, w, 4) RGBE bytes; scanlines from `flat_from` on
    are written flat (as a writer that stops encoding runs does)."""
    h, w, _ = rgbe.shape
    out = bytearray(header + b"-Y %d +X %d\n" % (h, w))
    for y in range(h):
        row = rgbe[y]
        if not rle or w < 8 or w > 0x7FFF or (flat_from is not None and y >= flat_from):
            out += row.tobytes()
            continue
        out += bytes([2, 2, w >> 8, w & 0xFF])
        for ch in range(4):
            out += _rle_channel(row[:, ch].tobytes())
    return bytes(out)


def rgbe_expected(rgbe: np.ndarray) -> np.ndarray:
    e = rgbe[..., 3].astype(np.int64)
    scale = np.where(e > 0, np.ldexp(1.0, e - 136), 0.0)
    return (rgbe[..., :3].astype(np.float64) * scale[..., None]).astype(np.float32)


def encode_dds(width: int, height: int, payload: bytes, fourcc: bytes | None = None, bitcount: int = 0,
               masks=(0, 0, 0, 0), alpha_flag: bool = False) -> bytes:
    """A DDS header (124 bytes after the magic) and the payload."""
    pf_flags = (0x4 if fourcc else 0x40) | (0x1 if alpha_flag else 0)
    pf = struct.pack("<II4sIIIII", 32, pf_flags, fourcc or b"\0\0\0\0", bitcount, *masks)
    hdr = struct.pack("<IIIIIII", 124, 0x1007, height, width, 0, 0, 1) + b"\0" * 44 + pf + \
        struct.pack("<IIIII", 0x1000, 0, 0, 0, 0)
    assert len(hdr) == 124
    return b"DDS " + hdr + payload
