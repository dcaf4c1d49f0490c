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
