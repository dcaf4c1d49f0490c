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
           ("UInt8x4", "ABgr"), ("UInt1010102", "RgbA"), ("UInt2101010", "RgbA"), ("UInt16x4", "RgbA"),
           ("UInt233", "Rgb"), ("UInt_444", "Rgb"), ("UInt444_", "Rgb"), ("UInt101010_", "Rgb"),
           ("UInt_101010", "Rgb")]
# Levels of the coarsest channel of each layout: one code of it is the comparison step.
LEVELS = {"UInt8": 255, "UInt16": 65535, "UInt332": 3, "UInt233": 3, "UInt565": 31, "UInt4x4": 15, "UInt8x2": 255,
          "UInt8x3": 255, "UInt8x4": 255, "UInt16x2": 65535, "UInt16x4": 65535, "UInt1010102": 3,
          "UInt2101010": 3, "UInt_444": 15, "UInt444_": 15, "UInt101010_": 1023, "UInt_101010": 1023}
# The transfer functions of stage.frag:279-413 other than Linear and sRGB (Bt2100Pq and the
# Bt2100Hlg stub leave values unchanged there, as here).
TRANSFERS = ["Bt709", "Bt470M", "Bt601", "Smpte240", "Bt2020_10bit", "Bt2020_12bit", "Smpte2084", "Bt2100Pq",
             "Bt2100Hlg"]
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
    step = 1.0 / LEVELS[bits]
    # sRGB transfer stretches one code near black; compare in the transferred domain there.
    if transfer == "Srgb":
        fl = ofmt(bits, parts, "Linear")
        got_v = O.decode(fl, np.frombuffer(got, np.uint8).reshape(H, W * f.bpp), W, H)
        want_v = O.decode(fl, O.encode(f, want_lin), W, H)
    assert np.abs(got_v - want_v).max() <= step * 1.0001


@pytest.mark.parametrize("transfer", TRANSFERS)
@pytest.mark.parametrize("bits,parts", [("UInt8x4", "RgbA"), ("UInt16x4", "RgbA")])
@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_transfer_to_srgb8_within_one_step(transfer, bits, parts, mode):
    f = ofmt(bits, parts, transfer)
    raw = np.random.default_rng(14).integers(0, 256, size=(H, W * f.bpp), dtype=np.uint8)
    got = convert(desc(bits, parts, transfer), raw, Descriptor.srgb_rgba8(W, H), mode)
    want = O.encode(O.SRGB_RGBA8, O.decode(f, raw, W, H))
    diff = np.abs(np.frombuffer(got, np.uint8).astype(np.int32).reshape(want.shape) - want.astype(np.int32))
    assert diff.max() <= 1


@pytest.mark.parametrize("transfer", TRANSFERS)
@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_transfer_from_srgb8_within_one_code(transfer, mode):
    bits, parts = "UInt16x4", "RgbA"
    f, fl = ofmt(bits, parts, transfer), ofmt(bits, parts, "Linear")
    img = srgb_gradient_noise(W, H, seed=15)
    got = convert(Descriptor.srgb_rgba8(W, H), P.rgba_bytes(img), desc(bits, parts, transfer), mode)
    want_lin = O.decode(O.SRGB_RGBA8, P.rgba_bytes(img), W, H)
    # Codes of the transferred values (the layout decoded without its transfer).
    got_v = O.decode(fl, np.frombuffer(got, np.uint8).reshape(H, W * f.bpp), W, H)
    want_v = O.decode(fl, O.encode(f, want_lin), W, H)
    assert np.abs(got_v - want_v).max() <= 1.0001 / 65535


def test_packed_10bit_layouts_follow_serialize_bits():
    """SampleBits::UInt1010102 is stage.frag's Int2101010 layout and UInt2101010 its
    Int1010102 (ShaderData::serialize_bits, lib/zosimos/src/shaders/stage.rs:113-114): in
    UInt1010102 the first sample is bits 0-9 and alpha bits 30-31."""
    texels = np.array([[0x000003FF, 0xC0000000, 0x00000003, 0xFFFFFFFF]], dtype=np.uint32)
    got = convert(desc("UInt1010102", "RgbA", "Linear", 4, 1), texels.view(np.uint8),
                  Descriptor.linear_rgba_f32(4, 1), zs.Mode.Fused)
    rgba = np.frombuffer(got, np.float32).reshape(4, 4)
    assert np.allclose(rgba, [[1, 0, 0, 0], [0, 0, 0, 1], [3 / 1023, 0, 0, 0], [1, 1, 1, 1]])
    got = convert(desc("UInt2101010", "RgbA", "Linear", 4, 1), texels.view(np.uint8),
                  Descriptor.linear_rgba_f32(4, 1), zs.Mode.Fused)
    rgba = np.frombuffer(got, np.float32).reshape(4, 4)
    assert np.allclose(rgba, [[1, 255 / 1023, 0, 0], [0, 0, 0, 768 / 1023], [1, 0, 0, 0], [1, 1, 1, 1]])


def test_int444i_green_is_bits_8_to_11():
    """UInt444_ (stage.frag's Int444i): mux writes R, G, B at bits 4, 8, 12 (stage.frag:608);
    the demux here reads G back from bit 8, so the layout round-trips (stage.frag:547-548
    reads it from bit 9, which no reference path reaches: serialize_bits has no code for
    the padded layouts, stage.rs:98-118)."""
    d = desc("UInt444_", "Rgb", "Linear", 4, 1)
    texels = np.array([[0x0010, 0x0100, 0x1000, 0xFFF0]], dtype=np.uint16)
    got = convert(d, texels.view(np.uint8), Descriptor.linear_rgba_f32(4, 1), zs.Mode.Fused)
    rgba = np.frombuffer(got, np.float32).reshape(4, 4)
    assert np.allclose(rgba[:, :3], [[1 / 15, 0, 0], [0, 1 / 15, 0], [0, 0, 1 / 15], [1, 1, 1]])
