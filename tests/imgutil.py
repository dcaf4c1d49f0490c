"""Test helpers: a PNG reader (zlib + the five PNG row filters) and blockhash256.

blockhash256 follows the published block-mean-value method (blockhash.io) as used
by the reference's golden check (lib/zosimos/tests/util.rs:14-60, blockhash 1.0.0):
16x16 blocks, block value = sum of R+G+B (765 for fully transparent pixels),
one median per horizontal quarter band, bit = value > median (or, within 1 of the
median, 1 when the median is above half the block's maximum), hex with the first
bit as the most significant bit of a nibble.  Only the even-division case is
needed: every golden image is 512x512 or 400x400.
"""
from __future__ import annotations

import os
import struct
import zlib

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def read_png(path: str) -> np.ndarray:
    """8-bit RGBA / RGB / gray PNG (non-interlaced) -> (H, W, C) uint8."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat = 8, b""
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
            assert depth == 8 and interlace == 0
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    ch = {0: 1, 2: 3, 4: 2, 6: 4}[ctype]
    raw = np.frombuffer(zlib.decompress(idat), dtype=np.uint8)
    stride = w * ch
    out = np.zeros((h, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int32)
    p = 0
    for y in range(h):
        f = raw[p]
        line = raw[p + 1:p + 1 + stride].astype(np.int32)
        p += 1 + stride
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        elif f == 1:
            cur = line.copy()
            for x in range(ch, stride):
                cur[x] = (cur[x] + cur[x - ch]) & 255
        elif f == 3:
            cur = line.copy()
            for x in range(stride):
                a = cur[x - ch] if x >= ch else 0
                cur[x] = (cur[x] + ((a + prev[x]) >> 1)) & 255
        else:
            cur = line.copy()
            for x in range(stride):
                a = cur[x - ch] if x >= ch else 0
                b = prev[x]
                c = prev[x - ch] if x >= ch else 0
                pp = a + b - c
                pa, pb, pc = abs(pp - a), abs(pp - b), abs(pp - c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (cur[x] + pred) & 255
        out[y] = cur
        prev = cur
    return out.reshape(h, w, ch)


def golden_image(name: str) -> np.ndarray:
    return read_png(os.path.join(GOLDEN, name))


def golden_hashes() -> dict:
    out = {}
    with open(os.path.join(GOLDEN, "blockhash_goldens.txt")) as f:
        for line in f:
            if line.startswith("#") or ":" not in line:
                continue
            k, v = line.split(":", 1)
            out[k.strip()] = v.split()
    return out


def blockhash256(rgba: np.ndarray) -> str:
    """blockhash256 of an (H, W, 4) uint8 image whose sides are multiples of 16."""
    bits = 16
    h, w, _ = rgba.shape
    assert h % bits == 0 and w % bits == 0, "only the even-division case is implemented"
    bw, bh = w // bits, h // bits
    val = rgba[..., :3].astype(np.int64).sum(-1)
    val = np.where(rgba[..., 3] == 0, 765, val)
    blocks = val.reshape(bits, bh, bits, bw).sum(axis=(1, 3)).reshape(-1).astype(np.float64)
    half = bw * bh * 256 * 3 / 2
    band = len(blocks) // 4
    out = []
    for i in range(4):
        seg = blocks[i * band:(i + 1) * band]
        m = np.median(seg)
        out += [int(v > m or (abs(v - m) < 1 and m > half)) for v in seg]
    return "".join("%x" % (out[i] * 8 + out[i + 1] * 4 + out[i + 2] * 2 + out[i + 3])
                   for i in range(0, len(out), 4))


def luma_alpha16_to_rgba8(bytes_hw4: np.ndarray) -> np.ndarray:
    """View 4-byte texels as little-endian LumaA16 and convert like image's
    Rgba<u8> conversion of a 16-bit sample: round(v / 257)."""
    h, w = bytes_hw4.shape[0], bytes_hw4.shape[1] // 4 if bytes_hw4.ndim == 2 else bytes_hw4.shape[1]
    b = bytes_hw4.reshape(h, w, 4).astype(np.uint32)
    luma = b[..., 0] | (b[..., 1] << 8)
    alpha = b[..., 2] | (b[..., 3] << 8)
    l8 = ((luma + 128) // 257).astype(np.uint8)
    a8 = ((alpha + 128) // 257).astype(np.uint8)
    return np.stack([l8, l8, l8, a8], -1)
