"""Oracle for the texture front-end. TEST INFRASTRUCTURE ONLY: imported by
tests/ as the checker of rmn_image_load and of the device mip chains, never
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
