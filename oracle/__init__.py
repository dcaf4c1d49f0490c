"""CPU oracle for the zosimos raster pipeline -- TEST INFRASTRUCTURE ONLY.

This package is the parity checker of the GB300 executor.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
it; the product package (``zosimos_gb300``) never does.

``liboracle.so`` (built from ``oracle.c`` by ``oracle/Makefile``) holds:

* ``zo_*``   -- the FP64 restatement of the reference's shader arithmetic, and
* ``zo32_*`` -- the same operations in FP32, one full pass per operation with
  OpenMP over rows: the plain per-op CPU pipeline timed as the CPU baseline.

Images handled here are numpy arrays: "linear" images are ``(H, W, 4)`` float64
(or float32 for the ``f32=True`` variants) holding the value a zosimos fragment
shader sees after staging decode; texel images are ``(H, row_bytes)`` uint8.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

# Codes follow lib/std/src/stage.frag:102-176 of the zosimos project, reached from the
# SampleBits names through ShaderData::serialize_bits (lib/zosimos/src/shaders/stage.rs:98-118),
# which maps UInt1010102 to stage.frag's Int2101010 (15) and UInt2101010 to Int1010102 (14).
BITS = dict(UInt8=0, UInt332=1, UInt233=2, UInt16=3, UInt4x4=4, UInt_444=5, UInt444_=6, UInt565=7,
            UInt8x2=8, UInt8x3=9, UInt8x4=10, UInt16x2=11, UInt16x3=12, UInt16x4=13,
            UInt1010102=15, UInt2101010=14, UInt101010_=16, UInt_101010=17, Float16x4=18,
            Float32x4=19)
PARTS = dict(A=0, R=1, G=2, B=3, Luma=4, LumaA=5, Rgb=6, Bgr=7, RgbA=8, Rgbx=9, BgrA=10, Bgrx=11,
             ARgb=12, Xrgb=13, ABgr=14, Xbgr=15, Yuv=16, Lab=17, LabA=18, Lch=19, LchA=20)
TRANSFER = dict(Bt709=0, Bt470M=1, Bt601=2, Smpte240=3, Linear=4, Srgb=5, Bt2020_10bit=6,
                Bt2020_12bit=7, Smpte2084=8, Bt2100Pq=9, Bt2100Hlg=10, LinearScene=11, LabLch=0x100)
TEXEL_BYTES = [1, 1, 1, 2, 2, 2, 2, 2, 2, 3, 4, 4, 6, 8, 4, 4, 4, 4, 8, 16]
WHITEPOINT = dict(A=0, B=1, C=2, D50=3, D55=4, D65=5, D75=6, E=7, F2=8, F7=9, F11=10)
PRIMARIES = dict(Bt601_525=0, Bt601_625=1, Bt709=2, Smpte240=3, Bt2020=4, Bt2100=5, P3=6,
                 AdobeRgb=7, Xyz=8)
ADAPT = dict(Xyz=0, VonKries=1, BradfordVonKries=2, BradfordNonLinear=3)
BLEND = dict(Over=0, Multiply=1, Screen=2, Add=3)
FILTER = dict(Box=0, Lanczos3=1, Triangle=2)


class _Fmt(ctypes.Structure):
    _fields_ = [("bits", ctypes.c_int32), ("parts", ctypes.c_int32),
                ("transfer", ctypes.c_int32), ("native", ctypes.c_int32)]


@dataclass(frozen=True)
class Format:
    """Texel encoding as seen by stage.frag: bits, parts, transfer and whether the
    reference stores it in a native (round-to-nearest) wgpu format."""
    bits: int
    parts: int
    transfer: int
    native: bool = False

    @property
    def bpp(self) -> int:
        return TEXEL_BYTES[self.bits]

    def _c(self):
        return _Fmt(self.bits, self.parts, self.transfer, int(self.native))


SRGB_RGBA8 = Format(BITS["UInt8x4"], PARTS["RgbA"], TRANSFER["Srgb"], True)
LINEAR_RGBA8 = Format(BITS["UInt8x4"], PARTS["RgbA"], TRANSFER["Linear"], True)
LINEAR_F32 = Format(BITS["Float32x4"], PARTS["RgbA"], TRANSFER["Linear"], False)
LINEAR_F16 = Format(BITS["Float16x4"], PARTS["RgbA"], TRANSFER["Linear"], False)


def build() -> str:
    """Compile liboracle.so with the committed Makefile (gcc, OpenMP)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = ctypes.CDLL(_LIB_PATH)
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _d9(m):
    m = np.ascontiguousarray(np.asarray(m, dtype=np.float64).reshape(9))
    return m, _p(m)


def _prefix(f32: bool) -> str:
    return "zo32_" if f32 else "zo_"


def _dtype(f32: bool):
    return np.float32 if f32 else np.float64


def set_threads(n: int) -> None:
    lib().zo_set_threads(ctypes.c_int32(n))


def max_threads() -> int:
    return int(lib().zo_max_threads())


# ---------------------------------------------------------------- texels


def decode(fmt: Format, texels: np.ndarray, width: int, height: int, f32: bool = False,
           row_stride: int | None = None) -> np.ndarray:
    t = np.ascontiguousarray(texels, dtype=np.uint8)
    rs = row_stride if row_stride is not None else width * fmt.bpp
    out = np.empty((height, width, 4), dtype=_dtype(f32))
    c = fmt._c()
    getattr(lib(), _prefix(f32) + "decode")(ctypes.byref(c), _p(t), ctypes.c_int64(rs),
                                            ctypes.c_int32(width), ctypes.c_int32(height), _p(out))
    return out


def encode(fmt: Format, img: np.ndarray, f32: bool = False) -> np.ndarray:
    img = np.ascontiguousarray(img, dtype=_dtype(f32))
    h, w = img.shape[:2]
    out = np.zeros((h, w * fmt.bpp), dtype=np.uint8)
    c = fmt._c()
    getattr(lib(), _prefix(f32) + "encode")(ctypes.byref(c), _p(img), ctypes.c_int32(w),
                                            ctypes.c_int32(h), _p(out), ctypes.c_int64(w * fmt.bpp))
    return out


# ---------------------------------------------------------------- colour


def _inplace(name, img, f32, *args):
    assert img.flags["C_CONTIGUOUS"] and img.dtype == _dtype(f32)
    n = img.size // 4
    getattr(lib(), _prefix(f32) + name)(_p(img), ctypes.c_int64(n), *args)
    return img


def mat3(img, m, f32=False):
    m, pm = _d9(m)
    return _inplace("mat3", img, f32, pm)


def clamp01_rgb(img, f32=False):
    return _inplace("clamp01_rgb", img, f32)


def oklab_encode(img, rgb_to_xyz, f32=False):
    m, pm = _d9(rgb_to_xyz)
    return _inplace("oklab_encode", img, f32, pm)


def oklab_decode(img, xyz_to_rgb, f32=False):
    m, pm = _d9(xyz_to_rgb)
    return _inplace("oklab_decode", img, f32, pm)


def srlab2_encode(img, rgb_to_xyz, f32=False):
    m, pm = _d9(rgb_to_xyz)
    return _inplace("srlab2_encode", img, f32, pm)


def srlab2_decode(img, xyz_to_rgb, whitepoint_xyz, f32=False):
    m, pm = _d9(xyz_to_rgb)
    wp = np.ascontiguousarray(np.asarray(whitepoint_xyz, dtype=np.float64).reshape(3))
    return _inplace("srlab2_decode", img, f32, pm, _p(wp))


def transfer(img, transfer_code, forward, f32=False):
    return _inplace("transfer", img, f32, ctypes.c_int32(transfer_code), ctypes.c_int32(int(forward)))


def inject(bg, fg, select, weights, f32=False):
    """inject.frag: bg = mix(bg, dot(fg, weights), select) (in place on bg)."""
    assert bg.shape == fg.shape and bg.flags["C_CONTIGUOUS"] and bg.dtype == _dtype(f32)
    fg = np.ascontiguousarray(fg, dtype=_dtype(f32))
    s = np.ascontiguousarray(np.asarray(select, np.float64))
    w = np.ascontiguousarray(np.asarray(weights, np.float64))
    getattr(lib(), _prefix(f32) + "inject")(_p(bg), _p(fg), ctypes.c_int64(bg.size // 4), _p(s), _p(w))
    return bg


def blend(below, above, offset=(0, 0), mode="Over", straight=True, f32=False):
    below = below if below.flags["C_CONTIGUOUS"] else np.ascontiguousarray(below)
    above = np.ascontiguousarray(above, dtype=_dtype(f32))
    bh, bw = below.shape[:2]
    ah, aw = above.shape[:2]
    getattr(lib(), _prefix(f32) + "blend")(
        _p(below), _p(above), ctypes.c_int32(bw), ctypes.c_int32(bh), ctypes.c_int32(aw),
        ctypes.c_int32(ah), ctypes.c_int32(offset[0]), ctypes.c_int32(offset[1]),
        ctypes.c_int32(BLEND[mode] if isinstance(mode, str) else mode), ctypes.c_int32(int(straight)))
    return below


def bilinear_construct(width, height, u_min, u_max, v_min, v_max, uv_min, uv_max, f32=False):
    p = np.ascontiguousarray(np.concatenate([u_min, u_max, v_min, v_max, uv_min, uv_max]).astype(np.float64))
    out = np.empty((height, width, 4), dtype=_dtype(f32))
    getattr(lib(), _prefix(f32) + "bilinear_construct")(_p(out), ctypes.c_int32(width),
                                                        ctypes.c_int32(height), _p(p))
    return out


def affine(below, above, inverse, bilinear, f32=False):
    inv = np.ascontiguousarray(np.asarray(inverse, dtype=np.float32).reshape(9))
    above = np.ascontiguousarray(above, dtype=_dtype(f32))
    bh, bw = below.shape[:2]
    ah, aw = above.shape[:2]
    getattr(lib(), _prefix(f32) + "affine")(_p(below), ctypes.c_int32(bw), ctypes.c_int32(bh),
                                            _p(above), ctypes.c_int32(aw), ctypes.c_int32(ah),
                                            _p(inv), ctypes.c_int32(int(bilinear)))
    return below


def affine_rows(band, y0, above, inverse, bilinear, f32=False):
    """Rows [y0, y0 + band height) of affine(): `band` holds those rows of the full-size
    `below` and is painted in place with the pixel centres of the full image."""
    inv = np.ascontiguousarray(np.asarray(inverse, dtype=np.float32).reshape(9))
    above = np.ascontiguousarray(above, dtype=_dtype(f32))
    nh, bw = band.shape[:2]
    ah, aw = above.shape[:2]
    getattr(lib(), _prefix(f32) + "affine_rows")(_p(band), ctypes.c_int32(bw), ctypes.c_int32(y0),
                                                 ctypes.c_int32(y0 + nh), _p(above), ctypes.c_int32(aw),
                                                 ctypes.c_int32(ah), _p(inv), ctypes.c_int32(int(bilinear)))
    return band


def resample_rows(src, width, height, y0, y1, filt="Lanczos3", f32=False):
    """Output rows [y0, y1) of resample(src, width, height, filt), same arithmetic."""
    src = np.ascontiguousarray(src, dtype=_dtype(f32))
    sh, sw = src.shape[:2]
    out = np.empty((y1 - y0, width, 4), dtype=_dtype(f32))
    getattr(lib(), _prefix(f32) + "resample_rows")(_p(src), ctypes.c_int32(sw), ctypes.c_int32(sh), _p(out),
                                                   ctypes.c_int32(width), ctypes.c_int32(height),
                                                   ctypes.c_int32(y0), ctypes.c_int32(y1),
                                                   ctypes.c_int32(FILTER[filt] if isinstance(filt, str) else filt))
    return out


def resample(src, width, height, filt="Lanczos3", f32=False):
    src = np.ascontiguousarray(src, dtype=_dtype(f32))
    sh, sw = src.shape[:2]
    out = np.empty((height, width, 4), dtype=_dtype(f32))
    getattr(lib(), _prefix(f32) + "resample")(_p(src), ctypes.c_int32(sw), ctypes.c_int32(sh), _p(out),
                                              ctypes.c_int32(width), ctypes.c_int32(height),
                                              ctypes.c_int32(FILTER[filt] if isinstance(filt, str) else filt))
    return out


# ---------------------------------------------------------------- matrices


DERIVATIVE = dict(Roberts=0, Prewitt=1, Sobel=2, Scharr3=3, Scharr4=4, Scharr5=5, Scharr3To4Bit=6, Scharr5Tab=7,
                  Scharr3To8Bit=8)
# Smoothing vectors of the implemented 3x3 operators (command.rs:3343-3409); the derivative
# vector is [0.5, 0, -0.5] for all of them.
DERIVATIVE_SMOOTHING = dict(Prewitt=(1 / 3, 1 / 3, 1 / 3), Sobel=(1 / 4, 1 / 2, 1 / 4),
                            Scharr3=(46.84 / 256, 162.32 / 256, 46.84 / 256),
                            Scharr3To4Bit=(3 / 16, 10 / 16, 3 / 16), Scharr3To8Bit=(47 / 256, 162 / 256, 47 / 256))


def derivative_matrix(method: str, width: bool = True) -> np.ndarray:
    """Row-major 3x3 of the operator as the reference builds it: the f32 outer product of
    smoothing and derivative vectors (RowMatrix::with_outer_product), transposed along the
    height (Direction::adjust_vertical_box)."""
    a = np.float32(DERIVATIVE_SMOOTHING[method])
    b = np.float32((0.5, 0.0, -0.5))
    m = (a[:, None] * b[None, :]).astype(np.float32)
    return (m if width else m.T).astype(np.float64)


def box3(src, m, f32=False):
    src = np.ascontiguousarray(src, dtype=_dtype(f32))
    h, w = src.shape[:2]
    out = np.empty_like(src)
    m, pm = _d9(m)
    getattr(lib(), _prefix(f32) + "box3")(_p(src), ctypes.c_int32(w), ctypes.c_int32(h), _p(out), pm)
    return out


def normal2d_with_diagonal(var0: float, var1: float) -> np.ndarray:
    """Parameters [mu0, mu1, inv00, inv01, inv10, inv11, pseudo_det] of a centred normal
    distribution with diagonal covariance, in f32 as shaders/distribution_normal2d.rs:24-38."""
    f = np.float32
    pi = f(np.pi)
    d0 = f(0) if var0 == 0 else f(1) / f(var0)
    d1 = f(0) if var1 == 0 else f(1) / f(var1)
    f0 = f(1) if var0 == 0 else f(2) * pi * f(var0)
    f1 = f(1) if var1 == 0 else f(2) * pi * f(var1)
    return np.array([0, 0, d0, 0, 0, d1, f0 * f1], np.float32)


def normal2d_with_direction(x: float, y: float) -> np.ndarray:
    """A 1-D normal distribution along `dir` (shaders/distribution_normal2d.rs:40-94): the
    pseudo inverse dir^T dir / |dir|^4 by the reference's reformulated f32 expressions."""
    f = np.float32
    x, y = f(x), f(y)
    length_sq = f(float(x) * float(x) + float(y) * float(y))

    def symmetric(a, b):
        hyp = f(np.hypot(a, b))
        up = (f(1) / hyp) * (a / hyp)
        low = a + b * (b / a)
        return f(up / low)

    def asymmetric(a, b):
        a, b = min(a, b), max(a, b)
        hyp = f(np.hypot(a, b))
        inner = f(float(a) * float(a / b) + float(b))      # mul_add: one rounding
        return f(((a / hyp) / inner) / hyp)

    inv = [symmetric(x, x), asymmetric(x, y), asymmetric(y, x), symmetric(y, y)]
    return np.array([0, 0, *inv, f(2) * f(np.pi) * length_sq], np.float32)


def normal2d(width: int, height: int, params) -> np.ndarray:
    """distribution_normal2d.frag: v = exp(-0.5 pos . (C^+ pos)) / sqrt(pseudo_det) at pixel
    centres, pos = 2 (uv - 0.5) - mu; (v, v, v, 1), FP64."""
    p = np.asarray(params, np.float64)
    u = (np.arange(width) + 0.5) / width
    v = (np.arange(height) + 0.5) / height
    px = 2.0 * (u[None, :] - 0.5) - p[0]
    py = 2.0 * (v[:, None] - 0.5) - p[1]
    # GLSL mat2 columns are (inv00, inv01) and (inv10, inv11) of the uploaded row-major data.
    q = px * (p[2] * px + p[4] * py) + py * (p[3] * px + p[5] * py)
    val = np.exp(-0.5 * q) / np.sqrt(p[6])
    out = np.empty((height, width, 4))
    out[..., 0] = out[..., 1] = out[..., 2] = val
    out[..., 3] = 1.0
    return out


def fractal_noise_with_octaves(num_octaves: int) -> np.ndarray:
    """FractalNoise::with_octaves (shaders/fractal_noise.rs:20-31): grid 100 x 100, damping 1,
    amplitude 1 / n in f64 rounded to f32.  [grid x, grid y, amplitude, damping, octaves]."""
    return np.array([100.0, 100.0, np.float32(1.0 / float(num_octaves)), 1.0, num_octaves], np.float32)


def fractal_noise_set_damping(params, damping: float) -> np.ndarray:
    """FractalNoise::set_damping (shaders/fractal_noise.rs:33-49), in f32."""
    p = np.asarray(params, np.float32).copy()
    f = np.float32
    d = f(damping)
    total = f(1.0) - f(np.power(d, f(p[4]), dtype=np.float32))
    p[2] = f(1.0) if abs(total) < f(1e-7) else f(f(1.0) - d) / total
    p[3] = d
    return p


def _pcg4d(x, y):
    """PCG4D (Jarzynski and Olano, JCGT 9(3) 2020) of uvec4(x, y, 0, 0), uint32 wraparound;
    fractal_noise.frag:20-28."""
    m = np.uint64(0xFFFFFFFF)
    v = [np.asarray(t, np.uint64) & m for t in (x, y, np.zeros_like(x), np.zeros_like(x))]
    v = [(t * np.uint64(1664525) + np.uint64(1013904223)) & m for t in v]

    def mix(v):
        v[0] = (v[0] + v[1] * v[3]) & m
        v[1] = (v[1] + v[2] * v[0]) & m
        v[2] = (v[2] + v[0] * v[1]) & m
        v[3] = (v[3] + v[1] * v[2]) & m
    mix(v)
    v = [t ^ (t >> np.uint64(16)) for t in v]
    mix(v)
    return v


def fractal_noise(width: int, height: int, params) -> np.ndarray:
    """fractal_noise.frag: fbm(uv) at pixel centres uv = ((x + 0.5) / W, (y + 0.5) / H), in
    f32 with every product and sum rounded separately; 4 uncorrelated channels.  The rotation
    between octaves is 2 mat3(cos .5, sin .5, 1, -sin .5, cos .5, 1, 0, 0, 1) with f32
    constants (only x and y feed the noise)."""
    f = np.float32
    p = np.asarray(params, np.float32)
    c5, c6 = f(2.0) * f(np.cos(0.5)), f(2.0) * f(np.sin(0.5))
    px = np.broadcast_to((np.arange(width, dtype=f) + f(0.5)) / f(width), (height, width)).astype(f)
    py = np.broadcast_to(((np.arange(height, dtype=f) + f(0.5)) / f(height))[:, None], (height, width)).astype(f)
    amp = f(p[2])
    acc = np.zeros((height, width, 4), f)
    for _ in range(int(p[4])):
        tx, ty = (px * p[0]).astype(f), (py * p[1]).astype(f)
        flx, fly = np.floor(tx), np.floor(ty)
        fx, fy = (tx - flx).astype(f), (ty - fly).astype(f)
        # float -> int32 saturates (as the GPU conversion), then reinterpreted as uint32.
        cx = np.clip(flx.astype(np.float64), -2.0 ** 31, 2.0 ** 31 - 1).astype(np.int64) & 0xFFFFFFFF
        cy = np.clip(fly.astype(np.float64), -2.0 ** 31, 2.0 ** 31 - 1).astype(np.int64) & 0xFFFFFFFF

        def corner(dx, dy):
            h = _pcg4d((cx + dx) & 0xFFFFFFFF, (cy + dy) & 0xFFFFFFFF)
            return np.stack([(t.astype(f) / f(4294967296.0)).astype(f) for t in h], axis=-1)
        A, B, C, D = corner(0, 0), corner(1, 0), corner(0, 1), corner(1, 1)
        ux = ((fx * fx).astype(f) * (f(3.0) - (f(2.0) * fx).astype(f))).astype(f)[..., None]
        uy = ((fy * fy).astype(f) * (f(3.0) - (f(2.0) * fy).astype(f))).astype(f)[..., None]
        m = (A * (f(1.0) - ux) + B * ux).astype(f)
        t1 = (((C - A) * uy).astype(f) * (f(1.0) - ux)).astype(f)
        t2 = (((D - B) * ux).astype(f) * uy).astype(f)
        n = ((m + t1).astype(f) + t2).astype(f)
        acc = (acc + (amp * n).astype(f)).astype(f)
        nx = ((c5 * px).astype(f) + (-c6 * py).astype(f)).astype(f)
        ny = ((c6 * px).astype(f) + (c5 * py).astype(f)).astype(f)
        px, py = nx, ny
        amp = f(amp * p[3])
    return acc.astype(np.float64)


def rgb_to_xyz(primaries="Bt709", whitepoint="D65") -> np.ndarray:
    out = np.zeros(9)
    lib().zo_rgb_to_xyz(ctypes.c_int32(PRIMARIES[primaries]), ctypes.c_int32(WHITEPOINT[whitepoint]), _p(out))
    return out.reshape(3, 3)


def whitepoint_xyz(whitepoint="D65") -> np.ndarray:
    out = np.zeros(3)
    lib().zo_whitepoint_xyz(ctypes.c_int32(WHITEPOINT[whitepoint]), _p(out))
    return out


def adaptation(method, src_wp, dst_wp) -> np.ndarray:
    out = np.zeros(9)
    rc = lib().zo_adaptation(ctypes.c_int32(ADAPT[method]), ctypes.c_int32(WHITEPOINT[src_wp]),
                             ctypes.c_int32(WHITEPOINT[dst_wp]), _p(out))
    if rc != 0:
        raise NotImplementedError(method)
    return out.reshape(3, 3)


# ---------------------------------------------------------------- integer gathers


def gather_quad(src, src_w, src_h, dst, dst_w, dst_h, bpp, target, selection=None):
    """Nearest quad copy (crop / inscribe): `selection` of src onto `target` of dst (in place)."""
    src = np.ascontiguousarray(src, dtype=np.uint8)
    assert dst.flags["C_CONTIGUOUS"] and dst.dtype == np.uint8
    sel = np.asarray(selection if selection is not None else (0, 0, src_w, src_h), dtype=np.int32)
    tgt = np.asarray(target, dtype=np.int32)
    lib().zo_gather_quad2(_p(src), ctypes.c_int64(src_w * bpp), ctypes.c_int32(src_w), ctypes.c_int32(src_h),
                          _p(sel), _p(dst), ctypes.c_int64(dst_w * bpp), ctypes.c_int32(dst_w),
                          ctypes.c_int32(dst_h), ctypes.c_int32(bpp), _p(tgt))
    return dst


def affine_nearest_bytes(above, aw, ah, dst, dw, dh, bpp, inverse):
    above = np.ascontiguousarray(above, dtype=np.uint8)
    inv = np.ascontiguousarray(np.asarray(inverse, dtype=np.float32).reshape(9))
    lib().zo_affine_nearest_bytes(_p(above), ctypes.c_int64(aw * bpp), ctypes.c_int32(aw), ctypes.c_int32(ah),
                                  _p(dst), ctypes.c_int64(dw * bpp), ctypes.c_int32(dw), ctypes.c_int32(dh),
                                  ctypes.c_int32(bpp), _p(inv))
    return dst


def resize_ref_index(src_len, dst_len) -> np.ndarray:
    out = np.zeros(dst_len, dtype=np.int32)
    lib().zo_resize_ref_index(ctypes.c_int32(src_len), ctypes.c_int32(dst_len), _p(out))
    return out


def palette_index(src_w, src_h, basis_u, basis_v):
    bu = np.ascontiguousarray(basis_u, dtype=np.float32)
    bv = np.ascontiguousarray(basis_v, dtype=np.float32)
    dh, dw = bu.shape
    ix = np.zeros((dh, dw), np.int32)
    iy = np.zeros((dh, dw), np.int32)
    lib().zo_palette_index(ctypes.c_int32(src_w), ctypes.c_int32(src_h), _p(bu), _p(bv), ctypes.c_int32(dw),
                           ctypes.c_int32(dh), _p(ix), _p(iy))
    return ix, iy


def resample_weights(src_len, dst_len, filt="Lanczos3"):
    f = FILTER[filt] if isinstance(filt, str) else filt
    taps = int(lib().zo_resample_max_taps(ctypes.c_int32(src_len), ctypes.c_int32(dst_len), ctypes.c_int32(f)))
    first = np.zeros(dst_len, np.int32)
    count = np.zeros(dst_len, np.int32)
    w = np.zeros((dst_len, taps), np.float64)
    lib().zo_resample_weights(ctypes.c_int32(src_len), ctypes.c_int32(dst_len), ctypes.c_int32(f), _p(first),
                              _p(count), _p(w), ctypes.c_int32(taps))
    return first, count, w


def f32_to_f16(values) -> np.ndarray:
    v = np.asarray(values, dtype=np.float32).reshape(-1)
    f = lib().zo_f32_to_f16
    f.restype = ctypes.c_uint16
    return np.array([f(ctypes.c_float(x)) for x in v], dtype=np.uint16)
