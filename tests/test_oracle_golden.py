"""The CPU oracle against the reference's own golden data (no GPU).

blockhash256 goldens: lib/zosimos/tests/reference/*.crc.png; exact pins:
transmute byte equality (tests/blend.rs:371-372), rectangle algebra (command.rs:3649-3658).
"""
import numpy as np
import pytest

import oracle as O
import pipelines as P
from imgutil import blockhash256, luma_alpha16_to_rgba8


def hamming(a: str, b: str) -> int:
    return bin(int(a, 16) ^ int(b, 16)).count("1")


def test_png_fixture_decodes(background, foreground):
    assert background.shape == (512, 512, 4) and foreground.shape == (151, 157, 4)


def test_blockhash_reproduces_background_golden(background, goldens):
    # convert_bt709 / swapped / crt goldens all equal the hash of the unmodified input.
    assert blockhash256(background) in goldens["convert_bt709"]


def test_oracle_composed(background, foreground, goldens):
    out = P.oracle_composed(background, foreground)
    assert blockhash256(out.reshape(512, 512, 4)) in goldens["composed"]


def test_oracle_composed_without_normalize_bug_differs(background, foreground, goldens):
    out = P.rgba_bytes(background).copy()
    O.gather_quad(P.rgba_bytes(foreground), 157, 151, out, 512, 512, 4, (0, 0, 157, 151))
    assert blockhash256(out.reshape(512, 512, 4)) not in goldens["composed"]


def test_oracle_affine(background, foreground, goldens):
    out = P.oracle_affine(background, foreground)
    assert blockhash256(out.reshape(512, 512, 4)) in goldens["affine"]


def test_oracle_adapted(background, goldens):
    out = P.oracle_adapted(background)
    assert blockhash256(out.reshape(512, 512, 4)) in goldens["adapted"]


def test_oracle_convert_bt709(background, goldens):
    out = P.oracle_convert_bt709(background)
    assert blockhash256(out.reshape(512, 512, 4)) in goldens["convert_bt709"]


def test_oracle_swapped(background, goldens):
    out = P.oracle_swapped(background).reshape(512, 512, 4)
    assert blockhash256(out) in goldens["swapped"]
    d = out.astype(int) - background[..., [1, 0, 2, 3]].astype(int)
    assert np.abs(d).max() <= 1


def test_transmute_golden(background, goldens):
    # The transmuted bytes are the input bytes (blend.rs:371-372), seen as LumaA16.
    img = luma_alpha16_to_rgba8(P.rgba_bytes(background))
    assert blockhash256(img) in goldens["transmute"]


def test_oracle_generic_palette_golden(background, goldens):
    # lib/zosimos/tests/generic.rs: the palette of the background indexed by a 2048^2 grid of
    # staged (truncated) Scalars texels; the hash is one of the accepted goldens exactly.
    h = blockhash256(P.oracle_generic(background).reshape(2048, 2048, 4))
    assert h in goldens["generic"]


def test_oracle_palette_close_to_goldens(background, goldens):
    h = blockhash256(P.oracle_palette(background).reshape(400, 400, 4))
    # The two accepted goldens differ from each other by 8 bits (device variance).
    assert min(hamming(h, g) for g in goldens["palette"]) <= 8


@pytest.mark.parametrize("space", ["oklab", "srlab2"])
def test_oracle_lab_grid(space, goldens):
    out = P.oracle_lab_grid(space).reshape(400, 400, 4)
    assert blockhash256(out) in goldens[space]


def test_srgb_roundtrip_exact():
    v = np.arange(256, dtype=np.uint8)
    img = np.stack([v, v[::-1], v, v], -1).reshape(1, 1024)
    assert (O.encode(O.SRGB_RGBA8, O.decode(O.SRGB_RGBA8, img, 256, 1)) == img).all()


@pytest.mark.parametrize("bits,parts", [("UInt8", "Luma"), ("UInt8x2", "LumaA"), ("UInt16", "Luma"),
                                        ("UInt16x2", "LumaA"), ("UInt565", "Rgb"), ("UInt4x4", "RgbA"),
                                        ("UInt8x4", "BgrA"), ("UInt8x4", "ARgb"), ("UInt8x4", "ABgr"),
                                        ("UInt1010102", "RgbA"), ("UInt2101010", "RgbA"), ("UInt16x4", "RgbA")])
def test_staged_roundtrip_exact(bits, parts):
    """demux -> mux of every code is the identity for linear transfer (truncation with
    IEEE division, stage.frag:533-641)."""
    f = O.Format(O.BITS[bits], O.PARTS[parts], O.TRANSFER["Linear"], False)
    rng = np.random.default_rng(7)
    raw = rng.integers(0, 256, size=(8, 64 * f.bpp), dtype=np.uint8)
    once = O.encode(f, O.decode(f, raw, 64, 8))
    twice = O.encode(f, O.decode(f, once, 64, 8))
    assert (once == twice).all()
    if bits in ("UInt8x4", "UInt16x4", "UInt16x2", "UInt4x4", "UInt8x2"):
        if parts in ("RgbA", "BgrA", "ARgb", "ABgr", "LumaA") and not (parts == "LumaA" and bits == "UInt16x2"):
            assert (once == raw).all()


def test_resample_weights_normalised():
    for src, dst in ((8192, 4096), (8192, 2214), (8192, 1024), (512, 384), (100, 300)):
        for f in ("Box", "Lanczos3", "Triangle"):
            first, count, w = O.resample_weights(src, dst, f)
            s = w.sum(axis=1)
            assert np.allclose(s, 1.0, atol=1e-12)
            assert (first >= 0).all() and (first + count <= src).all()


def test_half_conversion_matches_numpy():
    v = np.float32([0.0, 1.0, -2.5, 65504.0, 65520.0, 6e-8, 3e-8, 1e-3, 0.333333, 1e-5, -1e-6])
    ours = O.f32_to_f16(v)
    ref = v.astype(np.float16).view(np.uint16)
    assert (ours == ref).all()
    rng = np.random.default_rng(3)
    v = (rng.standard_normal(5000) * rng.choice([1e-6, 1e-3, 1, 100, 1e4], 5000)).astype(np.float32)
    assert (O.f32_to_f16(v) == v.astype(np.float16).view(np.uint16)).all()


def test_rectangle_algebra():
    from zosimos_gb300 import Rectangle
    small, large = Rectangle.with_width_height(2, 2), Rectangle.with_width_height(4, 4)
    assert large.join(small) == large and large.meet(small) == small
    assert large.contains(small) and not small.contains(large)


def test_chain_oracle_fp32_close_to_fp64():
    from zosimos_gb300.synthetic import srgb_gradient_noise
    img = srgb_gradient_noise(96, 64, seed=1)
    a = P.oracle_chain(img).astype(int)
    b = P.oracle_chain(img, f32=True).astype(int)
    assert np.abs(a - b).max() <= 1


@pytest.mark.parametrize("method", ["Prewitt", "Sobel", "Scharr3", "Scharr3To4Bit", "Scharr3To8Bit"])
def test_derivative_goldens(background, goldens, method):
    # tests/blend.rs:577-620: derivative along the width of background.png, stored as sRGB8.
    lin = O.decode(O.SRGB_RGBA8, background.reshape(512, 2048), 512, 512)
    out = O.encode(O.SRGB_RGBA8, O.box3(lin, O.derivative_matrix(method))).reshape(512, 512, 4)
    assert blockhash256(out) in goldens["derived_" + method]


LA16_SRGB = O.Format(O.BITS["UInt16x2"], O.PARTS["LumaA"], O.TRANSFER["Srgb"], False)
L8_SRGB = O.Format(O.BITS["UInt8"], O.PARTS["Luma"], O.TRANSFER["Srgb"], False)


def _hamming(h, accepted):
    return min(bin(int(h, 16) ^ int(a, 16)).count("1") for a in accepted)


def test_distribution_normal_goldens(goldens):
    # tests/blend.rs:227-311: 400 x 400 LumaA16 / Luma8 images of the normal density.
    img = O.normal2d(400, 400, O.normal2d_with_diagonal(0.2, 0.2))
    assert blockhash256(luma_alpha16_to_rgba8(O.encode(LA16_SRGB, img))) in goldens["distribution_normal2d"]
    img = O.normal2d(400, 400, O.normal2d_with_direction(0.04998, 0.0501))
    assert blockhash256(luma_alpha16_to_rgba8(O.encode(LA16_SRGB, img))) in goldens["distribution_normal1d"]
    l8 = O.encode(L8_SRGB, img).reshape(400, 400)
    rgba = np.stack([l8, l8, l8, np.full_like(l8, 255)], -1)
    # The two accepted hashes of the reference differ from each other by more than this.
    assert _hamming(blockhash256(rgba), goldens["distribution_u8"]) <= 3


def test_fractal_noise_golden(goldens):
    # tests/blend.rs:314-338: 400 x 400 sRGB RGBA8, FractalNoise::with_octaves(4).
    img = O.fractal_noise(400, 400, O.fractal_noise_with_octaves(4))
    assert blockhash256(O.encode(O.SRGB_RGBA8, img).reshape(400, 400, 4)) in goldens["distribution_fractal2d"]


def test_fractal_noise_damping_sums_to_one():
    # shaders/fractal_noise.rs:52-65: after set_damping(0.5) the 8 octave amplitudes sum to 1.
    p = O.fractal_noise_set_damping(O.fractal_noise_with_octaves(8), 0.5)
    amp, total = np.float32(p[2]), np.float32(0.0)
    for _ in range(8):
        total = np.float32(total + amp)
        amp = np.float32(amp * p[3])
    assert abs(1.0 - float(total)) < 1e-6


def test_oracle_packed_10bit_layouts_follow_serialize_bits():
    """UInt1010102 decodes with stage.frag's Int2101010 layout, UInt2101010 with Int1010102
    (lib/zosimos/src/shaders/stage.rs:113-114)."""
    texels = np.array([[0x000003FF, 0xC0000000, 0x00000003, 0xFFFFFFFF]], dtype=np.uint32).view(np.uint8)
    f = O.Format(O.BITS["UInt1010102"], O.PARTS["RgbA"], O.TRANSFER["Linear"], False)
    assert np.allclose(O.decode(f, texels, 4, 1).reshape(4, 4), [[1, 0, 0, 0], [0, 0, 0, 1], [3 / 1023, 0, 0, 0],
                                                                  [1, 1, 1, 1]])
    f = O.Format(O.BITS["UInt2101010"], O.PARTS["RgbA"], O.TRANSFER["Linear"], False)
    assert np.allclose(O.decode(f, texels, 4, 1).reshape(4, 4), [[1, 255 / 1023, 0, 0], [0, 0, 0, 768 / 1023],
                                                                  [1, 0, 0, 0], [1, 1, 1, 1]])


def test_oracle_int444i_round_trips():
    """UInt444_ (stage.frag's Int444i): R, G, B at bits 4, 8, 12, as mux writes them
    (stage.frag:608).  The demux reads G from bit 8 so that mux and demux invert each other;
    stage.frag:547-548 reads bit 9, a path the reference never reaches (serialize_bits has no
    code for the padded layouts, stage.rs:98-118)."""
    f = O.Format(O.BITS["UInt444_"], O.PARTS["Rgb"], O.TRANSFER["Linear"], False)
    texels = np.array([[0x0010, 0x0100, 0x1000, 0xFFF0]], dtype=np.uint16).view(np.uint8)
    rgba = O.decode(f, texels, 4, 1).reshape(4, 4)
    assert np.allclose(rgba[:, :3], [[1 / 15, 0, 0], [0, 1 / 15, 0], [0, 0, 1 / 15], [1, 1, 1]])
    every = np.arange(0, 1 << 16, 16, dtype=np.uint16).reshape(1, -1)
    back = O.encode(f, O.decode(f, every.view(np.uint8), every.shape[1], 1))
    assert (back.view(np.uint16) == every).all()
