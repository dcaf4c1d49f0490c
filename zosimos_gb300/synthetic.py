"""Seeded synthetic images for the benchmark workloads (no dataset is available).

Counter-based: every value is splitmix64(key(seed, image, pixel, channel)), so any
sub-rectangle or image of a batch can be generated independently and identically on
any machine.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_SYNTH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "libzs_synth.so")
_synth_lib = None


def _c():
    """The OpenMP C generator (synth/zs_synth.c, built by build.py) when it is built, else
    None (the numpy forms below then compute the same values, more slowly)."""
    global _synth_lib
    if _synth_lib is None:
        if not os.path.exists(_SYNTH):
            return None
        lib = ctypes.CDLL(_SYNTH)
        i32, p = ctypes.c_int32, ctypes.c_void_p
        lib.zs_synth_srgb_gradient_noise.argtypes = [i32, i32, i32, i32, i32, i32, p]
        lib.zs_synth_linear_gradient_gauss.argtypes = [i32, i32, i32, i32, ctypes.c_double, p]
        lib.zs_synth_premultiplied_layer.argtypes = [i32, i32, i32, i32, i32, p]
        _synth_lib = lib
    return _synth_lib

_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_GOLD = np.uint64(0x9E3779B97F4A7C15)


def splitmix64(x: np.ndarray) -> np.ndarray:
    z = x + _GOLD
    z = (z ^ (z >> np.uint64(30))) * _M1
    z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def _keys(seed: int, image: int, npx: int, channel: int, start: int = 0) -> np.ndarray:
    base = np.uint64(((seed & 0xFFFF) << 48) | ((image & 0xFFFF) << 32))
    px = np.arange(start, start + npx, dtype=np.uint64)
    return base ^ (px * np.uint64(4) + np.uint64(channel))


def srgb_gradient_noise(width: int, height: int, seed: int = 1, image: int = 0, noise: int = 16,
                        random_alpha: bool = True) -> np.ndarray:
    """RGBA8 sRGB: R = x ramp, G = y ramp, B = diagonal ramp, plus uniform integer noise
    in [-noise, noise] (clamped), alpha uniform in [0, 255] (or opaque)."""
    lib = _c()
    if lib is not None:
        out = np.empty((height, width, 4), dtype=np.uint8)
        lib.zs_synth_srgb_gradient_noise(width, height, seed, image, noise, int(random_alpha), out.ctypes.data)
        return out
    y, x = np.mgrid[0:height, 0:width]
    r = np.rint(255.0 * x / max(width - 1, 1))
    g = np.rint(255.0 * y / max(height - 1, 1))
    b = np.rint(255.0 * (x + y) / max(width + height - 2, 1))
    out = np.empty((height, width, 4), dtype=np.uint8)
    n = width * height
    for c, base in enumerate((r, g, b)):
        z = splitmix64(_keys(seed, image, n, c))
        nz = (z % np.uint64(2 * noise + 1)).astype(np.int64) - noise
        out[..., c] = np.clip(base.reshape(-1) + nz, 0, 255).reshape(height, width)
    if random_alpha:
        out[..., 3] = (splitmix64(_keys(seed, image, n, 3)) & np.uint64(255)).astype(np.uint8).reshape(height, width)
    else:
        out[..., 3] = 255
    return out


def linear_gradient_gauss(width: int, height: int, seed: int = 3, image: int = 0, sigma: float = 0.05,
                          dtype=np.float16) -> np.ndarray:
    """Linear RGBA: gradient ramps plus Gaussian noise (Box-Muller on splitmix64),
    clamped to [0, 1], alpha 1."""
    lib = _c()
    if lib is not None and dtype == np.float16:
        out = np.empty((height, width, 4), dtype=np.float16)
        lib.zs_synth_linear_gradient_gauss(width, height, seed, image, sigma, out.ctypes.data)
        return out
    y, x = np.mgrid[0:height, 0:width].astype(np.float64)
    base = [x / max(width - 1, 1), y / max(height - 1, 1), (x + y) / max(width + height - 2, 1)]
    n = width * height
    out = np.empty((height, width, 4), dtype=np.float64)
    for c in range(3):
        z1 = splitmix64(_keys(seed, image, n, c))
        z2 = splitmix64(z1)
        u1 = ((z1 >> np.uint64(11)).astype(np.float64) + 1.0) / 9007199254740993.0
        u2 = (z2 >> np.uint64(11)).astype(np.float64) / 9007199254740992.0
        g = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)
        out[..., c] = np.clip(base[c] + sigma * g.reshape(height, width), 0.0, 1.0)
    out[..., 3] = 1.0
    return out.astype(dtype)


def _uniform(seed: int, image: int, n: int, channel: int) -> np.ndarray:
    z = splitmix64(_keys(seed, image, n, channel))
    return (z >> np.uint64(11)).astype(np.float64) / 9007199254740992.0


def premultiplied_layer(width: int, height: int, seed: int = 5, image: int = 0, blobs: int = 8,
                        dtype=np.float16) -> np.ndarray:
    """Premultiplied linear RGBA: gradient + Gaussian-noise colour, alpha = clamped sum of
    2D Gaussian blobs (sigma in [128, 768] px at 4096 px, scaled with the image)."""
    lib = _c()
    if lib is not None and dtype == np.float16:
        out = np.empty((height, width, 4), dtype=np.float16)
        lib.zs_synth_premultiplied_layer(width, height, seed, image, blobs, out.ctypes.data)
        return out
    rgb = linear_gradient_gauss(width, height, seed=seed, image=image, dtype=np.float64)
    u = _uniform(seed, image ^ 0x8000, 4 * blobs, 7)
    y, x = np.mgrid[0:height, 0:width].astype(np.float64)
    scale = max(width, height) / 4096.0
    alpha = np.zeros((height, width))
    for b in range(blobs):
        cx, cy = u[4 * b] * width, u[4 * b + 1] * height
        sigma = (128.0 + 640.0 * u[4 * b + 2]) * scale
        amp = 0.3 + 0.7 * u[4 * b + 3]
        alpha += amp * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2.0 * sigma * sigma))
    alpha = np.clip(alpha, 0.0, 1.0)
    out = rgb.copy()
    out[..., :3] *= alpha[..., None]
    out[..., 3] = alpha
    return out.astype(dtype)


def layer_transforms(count: int, seed: int = 5):
    """Per layer: rotation U(-30, 30) degrees and a log-uniform scale in [0.5, 2]."""
    u = _uniform(seed, 0x7FFF, 2 * count, 9)
    rot = (u[0::2] * 60.0 - 30.0).tolist()
    scale = np.exp(np.log(0.5) + u[1::2] * (np.log(2.0) - np.log(0.5))).tolist()
    return list(zip(rot, scale))


def thumbnail_sizes(count: int = 1024, seed: int = 4, lo: int = 64, hi: int = 4096):
    """Image sides log-uniform in [lo, hi] (independent width and height)."""
    z = splitmix64(_keys(seed, 0xFFFF, 2 * count, 0))
    u = (z >> np.uint64(11)).astype(np.float64) / 9007199254740992.0
    sides = np.exp(np.log(lo) + u * (np.log(hi) - np.log(lo)))
    sides = np.clip(np.rint(sides), lo, hi).astype(np.int64)
    return sides[0::2], sides[1::2]
