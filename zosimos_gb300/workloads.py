"""Canned Programs of the benchmark workloads, built with the public CommandBuffer API."""
from __future__ import annotations

import numpy as np

from . import (Bits, ChromaticAdaptationMethod, ColorKind, CommandBuffer, Descriptor, Parts, Transfer,
               Whitepoint)

# Oklab lightness x1.1, chroma x0.9 (a and b scaled), applied in Lab coordinates.
OKLAB_SCALE = [1.1, 0.0, 0.0, 0.0, 0.9, 0.0, 0.0, 0.0, 0.9]


def rgba_bytes(img: np.ndarray) -> np.ndarray:
    """(H, W, 4) uint8 -> (H, W*4) contiguous texel rows."""
    h, w = img.shape[:2]
    return np.ascontiguousarray(img, dtype=np.uint8).reshape(h, w * 4)


def color_chain(w: int, h: int):
    """sRGB -> linear -> XYZ D65 -> Bradford D50 -> Oklab -> L*1.1, C*0.9 -> back -> sRGB RGBA8.

    Expressed with the reference's ops (color_convert / chromatic_adaptation) plus the
    color_matrix extension; intermediates are declared FP32 so that no declared texel
    quantises them.  Returns (commands, input register, output register)."""
    c = CommandBuffer()
    src = Descriptor.srgb_rgba8(w, h)
    i = c.input(src)
    lin = c.color_convert(i, Descriptor.linear_rgba_f32(w, h))
    d50 = c.chromatic_adaptation(lin, ChromaticAdaptationMethod.BradfordVonKries, Whitepoint.D50)
    lab = c.color_convert(d50, Descriptor(w, h, Bits.Float32x4, Parts.LabA, ColorKind.Oklab,
                                          transfer=Transfer.Linear))
    scaled = c.color_matrix(lab, OKLAB_SCALE)
    back = c.color_convert(scaled, Descriptor.linear_rgba_f32(w, h, whitepoint=Whitepoint.D50))
    d65 = c.chromatic_adaptation(back, ChromaticAdaptationMethod.BradfordVonKries, Whitepoint.D65)
    out = c.color_convert(d65, src)
    o, _ = c.output(out)
    return c, i, o


def thumbnail_fit(w: int, h: int, canvas: int = 256):
    """Fitted size and centred origin of one thumbnail: the long side becomes `canvas`,
    the short side is rounded half away from zero (at least 1)."""
    if w >= h:
        tw, th = canvas, max(1, int(h * canvas / w + 0.5))
    else:
        tw, th = max(1, int(w * canvas / h + 0.5)), canvas
    return tw, th, (canvas - tw) // 2, (canvas - th) // 2


def thumbnail(w: int, h: int, canvas: int = 256):
    """One image of the batched-thumbnail workload as an ordinary program (the one launch
    per image form): the colour chain of `color_chain` in linear FP32, a box-filter fit,
    inscribed centred on a transparent linear canvas, sRGB RGBA8 out.
    Returns (commands, input register, output register)."""
    from . import Filter, Rectangle
    tw, th, x0, y0 = thumbnail_fit(w, h, canvas)
    c = CommandBuffer()
    src = Descriptor.srgb_rgba8(w, h)
    i = c.input(src)
    lin = c.color_convert(i, Descriptor.linear_rgba_f32(w, h))
    d50 = c.chromatic_adaptation(lin, ChromaticAdaptationMethod.BradfordVonKries, Whitepoint.D50)
    lab = c.color_convert(d50, Descriptor(w, h, Bits.Float32x4, Parts.LabA, ColorKind.Oklab,
                                          transfer=Transfer.Linear))
    scaled = c.color_matrix(lab, OKLAB_SCALE)
    back = c.color_convert(scaled, Descriptor.linear_rgba_f32(w, h, whitepoint=Whitepoint.D50))
    d65 = c.chromatic_adaptation(back, ChromaticAdaptationMethod.BradfordVonKries, Whitepoint.D65)
    small = c.resize_filtered(d65, (tw, th), Filter.Box)
    blank = c.solid_rgba(Descriptor.linear_rgba_f32(canvas, canvas), [0.0, 0.0, 0.0, 0.0])
    placed = c.inscribe_placed(blank, Rectangle(x0, y0, x0 + tw, y0 + th), small)
    out = c.color_convert(placed, Descriptor.srgb_rgba8(canvas, canvas))
    o, _ = c.output(out)
    return c, i, o


def blend_resize(w: int = 512, h: int = 512, out_w: int = 384, out_h: int = 384):
    """Two RGBA8 sRGB images: decode to linear FP32, alpha-over B onto A, bilinear affine
    resize (scale out/in) onto a transparent canvas, sRGB encode to RGBA8.
    Returns (commands, input A, input B, output register)."""
    from . import Affine, AffineSample, Blend, Rectangle
    c = CommandBuffer()
    src = Descriptor.srgb_rgba8(w, h)
    a = c.input(src)
    b = c.input(src)
    la = c.color_convert(a, Descriptor.linear_rgba_f32(w, h))
    lb = c.color_convert(b, Descriptor.linear_rgba_f32(w, h))
    over = c.blend(la, Rectangle(0, 0, w, h), lb, Blend.Alpha)
    canvas = c.solid_rgba(Descriptor.linear_rgba_f32(out_w, out_h), [0.0, 0.0, 0.0, 0.0])
    scale = Affine.new(AffineSample.BiLinear).scale(out_w / w, out_h / h)
    resized = c.affine(canvas, scale, over)
    out = c.color_convert(resized, Descriptor.srgb_rgba8(out_w, out_h))
    o, _ = c.output(out)
    return c, a, b, o


def resample(w: int, h: int, out_w: int, out_h: int, filt: int):
    """RGBA16F linear image -> separable filtered resize (Box / Lanczos3 / Triangle) ->
    RGBA16F.  Returns (commands, input, output)."""
    c = CommandBuffer()
    i = c.input(Descriptor.linear_rgba_f16(w, h))
    r = c.resize_filtered(i, (out_w, out_h), filt)
    o, _ = c.output(r)
    return c, i, o


BLEND_CYCLE = (0, 1, 2, 3)   # over, multiply, screen, add


def layer_affine(w: int, h: int, degrees: float, scale: float):
    """Rotate about the centre and scale, bilinear sampling."""
    import math

    from . import Affine, AffineSample
    return (Affine.new(AffineSample.BiLinear).shift(-w / 2.0, -h / 2.0).rotate(math.radians(degrees))
            .scale(scale, scale).shift(w / 2.0, h / 2.0))


def layer_stack(w: int, h: int, transforms):
    """Premultiplied RGBA16F layers, each under its own affine (bilinear) onto a transparent
    canvas and blended onto the stack with the modes cycling over / multiply / screen /
    add; accumulation declared FP32, result stored RGBA16F.
    Returns (commands, input registers, output register)."""
    c = CommandBuffer()
    d16 = Descriptor.linear_rgba_f16(w, h).with_color(alpha=1)
    d32 = Descriptor.linear_rgba_f32(w, h).with_color(alpha=1)
    acc = c.solid_rgba(d32, [0.0, 0.0, 0.0, 0.0])
    canvas = c.solid_rgba(d32, [0.0, 0.0, 0.0, 0.0])
    inputs = []
    from . import Rectangle
    for i, (deg, s) in enumerate(transforms):
        layer = c.input(d16)
        inputs.append(layer)
        wide = c.color_convert(layer, d32)
        placed = c.affine(canvas, layer_affine(w, h, deg, s), wide)
        acc = c.blend(acc, Rectangle(0, 0, w, h), placed, BLEND_CYCLE[i % 4])
    out = c.color_convert(acc, d16)
    o, _ = c.output(out)
    return c, inputs, o


def rotation(w: int, h: int, degrees: float):
    """RGBA16F linear image rotated about its centre (bilinear) onto a transparent canvas
    of the same size.  Returns (commands, input, output)."""
    import math

    from . import Affine, AffineSample
    c = CommandBuffer()
    d = Descriptor.linear_rgba_f16(w, h)
    i = c.input(d)
    canvas = c.solid_rgba(d, [0.0, 0.0, 0.0, 0.0])
    rot = (Affine.new(AffineSample.BiLinear).shift(-w / 2.0, -h / 2.0).rotate(math.radians(degrees))
           .shift(w / 2.0, h / 2.0))
    r = c.affine(canvas, rot, i)
    o, _ = c.output(r)
    return c, i, o, rot
