"""GPU parity of the staged texel formats (stage.frag:527-747 demux/mux and parts order,
:279-425 transfer functions): packed 332 / 565 / 4444 / 1010102 / 2101010, 16-bit channels,
Luma / LumaA, BGRA / ARGB / ABGR orders, each with linear and sRGB transfer.

- A round trip through linear FP32 (decode, store FP32, encode) must give exactly the bytes
  the oracle's decode + encode give (integer work: bit-exact).
- A conversion to native sRGB RGBA8 must be within one 8-bit step of the FP64 oracle, and a
  conversion from sRGB RGBA8 into the format within one code of it (truncating quantisation
  of FP32 against FP64 values may fall on either side of a code boundary)."""
import numpy as np
import pytest

import oracle as O
import pipelines as P
import zosimos_gb300 as zs
from zosimos_gb300 import Bits, ColorKind, CommandBuffer, Descriptor, Parts, Pool, Primaries, Transfer, Whitepoint
from zosimos_gb300.synthetic import srgb_gradient_noise

pytestmark = pytest.mark.gpu

FORMATS = [("UInt8", "Luma"), ("UInt8x2", "LumaA"), ("UInt16", "Luma"), ("UInt16x2", "LumaA"), ("UInt332", "Rgb"),
           ("UInt565", "Rgb"), ("UInt4x4", "RgbA"), ("UInt8x3", "Rgb"), ("UInt8x4", "BgrA"), ("UInt8x4", "ARgb"),
           ("UInt8x4", "ABgr"), ("UInt1010102", "RgbA"), ("UInt2101010", "RgbA"), ("UInt16x4", "RgbA")]
W, H = 64, 8


def desc(bits, parts, transfer, w=W, h=H):
    return Descriptor(w, h, getattr(Bits, bits), getattr(Parts, parts), ColorKind.Rgb, Primaries.Bt709,
                      getattr(Transfer, transfer), Whitepoint.D65)


def ofmt(bits, parts, transfer):
    return O.Format(O.BITS[bits], O.PARTS[parts], O.TRANSFER[transfer], False)


def convert(src_desc, src_bytes, dst_desc, mode):
    c = CommandBuffer()
    i = c.input(src_desc)
    o, _ = c.output(c.color_convert(i, dst_desc))
    pool = Pool()
    k = pool.insert(src_desc, src_bytes)
    return P.run(c, pool, [(i, k)], [o], mode)[0]


@pytest.mark.parametrize("bits,parts", FORMATS)
@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_roundtrip_through_f32_is_exact(bits, parts, mode):
    d = desc(bits, parts, "Linear")
    f = ofmt(bits, parts, "Linear")
    raw = np.random.default_rng(11).integers(0, 256, size=(H, W * f.bpp), dtype=np.uint8)
    want = O.encode(f, O.decode(f, raw, W, H))
    c = CommandBuffer()
    i = c.input(d)
    wide = c.color_convert(i, Descriptor.linear_rgba_f32(W, H))
    o, _ = c.output(c.color_convert(wide, d))
    pool = Pool()
    k = pool.insert(d, raw)
    got = P.run(c, pool, [(i, k)], [o], mode)[0]
    assert (np.frombuffer(got, np.uint8).reshape(want.shape) == want).all()


@pytest.mark.parametrize("bits,parts", FORMATS)
@pytest.mark.parametrize("transfer", ["Linear", "Srgb"])
@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_to_srgb8_within_one_step(bits, parts, transfer, mode):
    f = ofmt(bits, parts, transfer)
    raw = np.random.default_rng(12).integers(0, 256, size=(H, W * f.bpp), dtype=np.uint8)
    got = convert(desc(bits, parts, transfer), raw, Descriptor.srgb_rgba8(W, H), mode)
    want = O.encode(O.SRGB_RGBA8, O.decode(f, raw, W, H))
    diff = np.abs(np.frombuffer(got, np.uint8).astype(np.int32).reshape(want.shape) - want.astype(np.int32))
    assert diff.max() <= 1


@pytest.mark.parametrize("bits,parts", FORMATS)
@pytest.mark.parametrize("transfer", ["Linear", "Srgb"])
def test_from_srgb8_within_one_code(bits, parts, transfer):
    f = ofmt(bits, parts, transfer)
    img = srgb_gradient_noise(W, H, seed=13)
    got = convert(Descriptor.srgb_rgba8(W, H), P.rgba_bytes(img), desc(bits, parts, transfer), zs.Mode.Fused)
    want_lin = O.decode(O.SRGB_RGBA8, P.rgba_bytes(img), W, H)
    # Decode both byte images back and compare per channel in units of the format's codes.
    got_v = O.decode(f, np.frombuffer(got, np.uint8).reshape(H, W * f.bpp), W, H)
    want_v = O.decode(f, O.encode(f, want_lin), W, H)
    step = 1.0 / {"UInt8": 255, "UInt16": 65535, "UInt332": 3, "UInt565": 31, "UInt4x4": 15, "UInt8x2": 255,
                  "UInt8x3": 255, "UInt8x4": 255, "UInt16x2": 65535, "UInt16x4": 65535, "UInt1010102": 3,
                  "UInt2101010": 3}[bits]
    # sRGB transfer stretches one code near black; compare in the transferred domain there.
    if transfer == "Srgb":
        fl = ofmt(bits, parts, "Linear")
        got_v = O.decode(fl, np.frombuffer(got, np.uint8).reshape(H, W * f.bpp), W, H)
        want_v = O.decode(fl, O.encode(f, want_lin), W, H)
    assert np.abs(got_v - want_v).max() <= step * 1.0001
