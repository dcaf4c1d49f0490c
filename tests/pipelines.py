"""The reference's own test pipelines (lib/zosimos/tests/blend.rs) and the benchmark
workloads, each expressed twice: through the executor's API (``ours_*``, runs on the
GPU) and through the CPU oracle (``oracle_*``).  Both return texel bytes as
(H, row_bytes) uint8 arrays (or float arrays for float outputs)."""
from __future__ import annotations

import math

import numpy as np

import oracle as O
import zosimos_gb300 as zs
from zosimos_gb300 import (Affine, AffineSample, Bits, Capabilities, ChromaticAdaptationMethod, ColorKind,
                           CommandBuffer, Descriptor, Parts, Pool, Primaries, Rectangle, Transfer, Whitepoint)


from zosimos_gb300.workloads import rgba_bytes  # noqa: E402


def run(cmds, pool, binds, outputs, mode=zs.Mode.Fused, simt_resample=False):
    keys = zs.run_pipeline(cmds, pool, binds, outputs, Capabilities(mode=mode, simt_resample=simt_resample))
    return [pool.read(k) for k in keys]


def inv3_f32(m) -> np.ndarray:
    """Inverse of an f32 row-major 3x3 computed in FP64 by the adjugate, rounded to f32."""
    a = np.asarray(m, dtype=np.float64).reshape(9)
    c0 = a[4] * a[8] - a[5] * a[7]
    c1 = a[5] * a[6] - a[3] * a[8]
    c2 = a[3] * a[7] - a[4] * a[6]
    det = a[0] * c0 + a[1] * c1 + a[2] * c2
    r = np.array([c0, a[2] * a[7] - a[1] * a[8], a[1] * a[5] - a[2] * a[4], c1, a[0] * a[8] - a[2] * a[6],
                  a[2] * a[3] - a[0] * a[5], c2, a[1] * a[6] - a[0] * a[7], a[0] * a[4] - a[1] * a[3]]) / det
    return r.astype(np.float32)


# ---------------------------------------------------------------- blend.rs:83-120 composed


def ours_composed(bg, fg, mode=zs.Mode.Fused):
    pool = Pool()
    kb, kf = pool.insert_srgb(bg), pool.insert_srgb(fg)
    c = CommandBuffer()
    b = c.input(pool.descriptor(kb))
    f = c.input(pool.descriptor(kf))
    r = c.inscribe(b, Rectangle(0, 0, fg.shape[1], fg.shape[0]), f)
    o, _ = c.output(r)
    return run(c, pool, [(b, kb), (f, kf)], [o], mode)[0]


def oracle_composed(bg, fg):
    out = rgba_bytes(bg).copy()
    fh, fw = fg.shape[:2]
    # Rectangle::normalize (command.rs:3536-3543): max_y = y + width.
    O.gather_quad(rgba_bytes(fg), fw, fh, out, bg.shape[1], bg.shape[0], 4, (0, 0, fw, fw))
    return out


# ---------------------------------------------------------------- blend.rs:122-167 affine


def affine_45(bg, fg, sampling=AffineSample.Nearest) -> Affine:
    fh, fw = fg.shape[:2]
    bh, bw = bg.shape[:2]
    return (Affine.new(sampling).shift(-float(fw // 2), -float(fh // 2)).rotate(math.pi / 4.0)
            .shift(float(bw // 2), float(bh // 2)))


def ours_affine(bg, fg, sampling=AffineSample.Nearest, mode=zs.Mode.Fused):
    pool = Pool()
    kb, kf = pool.insert_srgb(bg), pool.insert_srgb(fg)
    c = CommandBuffer()
    b = c.input(pool.descriptor(kb))
    f = c.input(pool.descriptor(kf))
    r = c.affine(b, affine_45(bg, fg, sampling), f)
    o, _ = c.output(r)
    return run(c, pool, [(b, kb), (f, kf)], [o], mode)[0]


def oracle_affine(bg, fg):
    out = rgba_bytes(bg).copy()
    inv = inv3_f32(affine_45(bg, fg).transformation)
    fh, fw = fg.shape[:2]
    O.affine_nearest_bytes(rgba_bytes(fg), fw, fh, out, bg.shape[1], bg.shape[0], 4, inv)
    return out


def oracle_affine_bilinear(bg, fg):
    below = O.decode(O.SRGB_RGBA8, rgba_bytes(bg), bg.shape[1], bg.shape[0])
    above = O.decode(O.SRGB_RGBA8, rgba_bytes(fg), fg.shape[1], fg.shape[0])
    inv = inv3_f32(affine_45(bg, fg, AffineSample.BiLinear).transformation)
    O.affine(below, above, inv, True)
    return O.encode(O.SRGB_RGBA8, below)


# ---------------------------------------------------------------- blend.rs:169-197 adapted


def ours_adapted(bg, mode=zs.Mode.Fused):
    pool = Pool()
    kb = pool.insert_srgb(bg)
    c = CommandBuffer()
    b = c.input(pool.descriptor(kb))
    r = c.chromatic_adaptation(b, ChromaticAdaptationMethod.VonKries, Whitepoint.D50)
    o, _ = c.output(r)
    return run(c, pool, [(b, kb)], [o], mode)[0]


def oracle_adapted(bg):
    h, w = bg.shape[:2]
    lin = O.decode(O.SRGB_RGBA8, rgba_bytes(bg), w, h)
    m = np.linalg.inv(O.rgb_to_xyz("Bt709", "D50")) @ O.adaptation("VonKries", "D65", "D50") @ O.rgb_to_xyz()
    O.mat3(lin, m)
    return O.encode(O.SRGB_RGBA8, lin)


# ---------------------------------------------------------------- blend.rs:199-225 convert_bt709


def ours_convert_bt709(bg, mode=zs.Mode.Fused):
    pool = Pool()
    h, w = bg.shape[:2]
    d709 = Descriptor.srgb_rgba8(w, h).with_color(transfer=Transfer.Bt709)
    k = pool.insert(d709, rgba_bytes(bg))
    c = CommandBuffer()
    i = c.input(d709)
    r = c.color_convert(i, Descriptor.srgb_rgba8(w, h))
    o, _ = c.output(r)
    return run(c, pool, [(i, k)], [o], mode)[0]


def oracle_convert_bt709(bg):
    h, w = bg.shape[:2]
    f709 = O.Format(O.BITS["UInt8x4"], O.PARTS["RgbA"], O.TRANSFER["Bt709"], False)
    lin = O.decode(f709, rgba_bytes(bg), w, h)
    return O.encode(O.SRGB_RGBA8, lin)


# ---------------------------------------------------------------- blend.rs:423-447 swapped


def ours_swapped(bg, mode=zs.Mode.Fused):
    pool = Pool()
    kb = pool.insert_srgb(bg)
    c = CommandBuffer()
    i = c.input(pool.descriptor(kb))
    cr = c.extract(i, 0)
    cg = c.extract(i, 1)
    t = c.inject(i, 1, cr)
    s = c.inject(t, 0, cg)
    o, _ = c.output(s)
    return run(c, pool, [(i, kb)], [o], mode)[0]


def oracle_swapped(bg):
    h, w = bg.shape[:2]
    lin = O.decode(O.SRGB_RGBA8, rgba_bytes(bg), w, h)
    chans = []
    for part in ("R", "G"):
        f = O.Format(O.BITS["UInt8x4"], O.PARTS[part], O.TRANSFER["Srgb"], False)
        chans.append(O.decode(f, O.encode(f, lin), w, h))
    x = lin.copy()
    O.inject(x, chans[0], [0, 1, 0, 0], [1, 0, 0, 0])
    O.inject(x, chans[1], [1, 0, 0, 0], [0, 1, 0, 0])
    return O.encode(O.SRGB_RGBA8, x)


# ---------------------------------------------------------------- blend.rs:340-375 transmute


def luma_alpha16_desc(w, h) -> Descriptor:
    return Descriptor(w, h, Bits.UInt16x2, Parts.LumaA, ColorKind.Rgb, Primaries.Bt709, Transfer.Srgb,
                      Whitepoint.D65)


def ours_transmute(bg, mode=zs.Mode.Fused):
    pool = Pool()
    kb = pool.insert_srgb(bg)
    h, w = bg.shape[:2]
    c = CommandBuffer()
    i = c.input(pool.descriptor(kb))
    t = c.transmute(i, luma_alpha16_desc(w, h))
    o, _ = c.output(t)
    return run(c, pool, [(i, kb)], [o], mode)[0]


# ---------------------------------------------------------------- blend.rs:377-421 palette

RAMP = dict(u_min=[0.0, 0.0, 0.0, 1.0], u_max=[0.7, 0.0, 0.0, 1.0], v_min=[0.0, 0.0, 0.0, 1.0],
            v_max=[0.0, 0.7, 0.0, 1.0], uv_min=[0.0, 0.0, 0.0, 1.0], uv_max=[0.3, 0.3, 0.0, 1.0])


def ours_palette(bg, mode=zs.Mode.Fused):
    pool = Pool()
    kb = pool.insert_srgb(bg)
    c = CommandBuffer()
    i = c.input(pool.descriptor(kb))
    ramp = c.bilinear(Descriptor.srgb_rgba8(400, 400), **RAMP)
    p = c.palette(i, 0, 1, ramp)
    o, _ = c.output(p)
    return run(c, pool, [(i, kb)], [o], mode)[0]


def oracle_palette(bg):
    # The ramp is computed in f32 exactly like the GPU construct; encode and decode of the
    # sRGB8 texels are exact (FP64, correctly rounded to f32) like the GPU tables.
    ramp = O.bilinear_construct(400, 400, **RAMP, f32=True).astype(np.float64)
    rb = O.encode(O.SRGB_RGBA8, ramp)
    rd = O.decode(O.SRGB_RGBA8, rb, 400, 400).astype(np.float32)
    ix, iy = O.palette_index(bg.shape[1], bg.shape[0], rd[..., 0], rd[..., 1])
    return rgba_bytes(bg[iy, ix])


# ---------------------------------------------------------------- generic.rs:16-134 generic palette

GENERIC_IDX = dict(u_min=[0.0] * 4, u_max=[0.0] * 4, v_min=[0.0] * 4, v_max=[0.0] * 4, uv_min=[0.0] * 4,
                   uv_max=[1.0, 1.0, 0.0, 0.0])


def generic_palette_function() -> CommandBuffer:
    """The generic function of generic.rs:34-68: palette of a generic input indexed by a
    2048x2048 RGBA-u8 scalar bilinear grid, height from R and width from G."""
    f = CommandBuffer()
    a = f.generic()
    img = f.input_generic(a)
    idx_desc = Descriptor.srgb_rgba8(2048, 2048).with_color(color=ColorKind.Scalars, transfer=Transfer.Linear)
    idx = f.bilinear(idx_desc, **GENERIC_IDX)
    pal = f.palette(img, 1, 0, idx)
    f.output(pal)
    return f


def ours_generic(bg, mode=zs.Mode.Fused):
    pool = Pool()
    kb = pool.insert_srgb(bg)
    fn = generic_palette_function()
    c = CommandBuffer()
    conv = c.function(fn)
    i = c.input(pool.descriptor(kb))
    ty = c.register_descriptor(i)
    (res,) = c.invoke(conv, generics=[ty], arguments=[i])
    o, _ = c.output(res)
    prog = zs.Linker.from_included().link(c, [], [fn], [[1], []])
    exe = prog.lower_to(Capabilities(mode=mode))
    env = exe.from_pool(pool)
    env.bind(i, kb)
    ex = exe.launch(env)
    while ex.is_running():
        ex.step()
    return pool.read(ex.retire_output(o))


# The index grid's Scalars texels are not a native texture format (program.rs:781-946): they
# are staged, i.e. quantised by truncation (stage.frag).
SCALARS_U8 = O.Format(O.BITS["UInt8x4"], O.PARTS["RgbA"], O.TRANSFER["Linear"], False)


def oracle_generic(bg):
    idx = O.bilinear_construct(2048, 2048, **GENERIC_IDX, f32=True).astype(np.float64)
    ib = O.encode(SCALARS_U8, idx)
    idd = O.decode(SCALARS_U8, ib, 2048, 2048).astype(np.float32)
    ix, iy = O.palette_index(bg.shape[1], bg.shape[0], idd[..., 1], idd[..., 0])
    return rgba_bytes(bg[iy, ix])


# ---------------------------------------------------------------- blend.rs:449-575 oklab / srlab2

GRID = dict(u_min=[0.4, 0.0, 0.0, 1.0], v_min=[0.4, 0.0, 0.0, 1.0], u_max=[0.4, 0.0, 1.0, 1.0],
            v_max=[0.4, 1.0, 0.0, 1.0], uv_min=[0.0, 0.0, 0.0, 0.0], uv_max=[0.0, 0.0, 0.0, 0.0])


def ours_lab_grid(space: str, mode=zs.Mode.Fused):
    pool = Pool()
    c = CommandBuffer()
    dist = Descriptor.srgb_rgba8(400, 400).with_color(color=ColorKind.Scalars, transfer=Transfer.Linear)
    grid = c.bilinear(dist, **GRID)
    kind = ColorKind.Oklab if space == "oklab" else ColorKind.SrLab2
    lch = c.transmute(grid, dist.with_color(color=kind, parts=Parts.LchA, whitepoint=Whitepoint.D65))
    conv = c.color_convert(lch, Descriptor.srgb_rgba8(400, 400))
    o, _ = c.output(conv)
    return run(c, pool, [], [o], mode)[0]


def oracle_lab_grid(space: str):
    # bilinear.frag is f32 arithmetic; the construct is restated in f32 with the GPU's
    # operation order so that the truncating 8-bit grid holds the same bytes.
    grid = O.bilinear_construct(400, 400, **GRID, f32=True).astype(np.float64)
    fmt_u8 = O.Format(O.BITS["UInt8x4"], O.PARTS["RgbA"], O.TRANSFER["Linear"], False)
    gb = O.encode(fmt_u8, grid)
    lch = O.Format(O.BITS["UInt8x4"], O.PARTS["LchA"], O.TRANSFER["LabLch"], False)
    lab = O.decode(lch, gb, 400, 400)
    t = np.linalg.inv(O.rgb_to_xyz("Bt709", "D65"))
    if space == "oklab":
        O.oklab_decode(lab, t)
    else:
        O.srlab2_decode(lab, t, O.whitepoint_xyz("D65"))
    return O.encode(O.SRGB_RGBA8, lab)


# ---------------------------------------------------------------- the fused colour chain

from zosimos_gb300.workloads import OKLAB_SCALE, color_chain as chain_commands  # noqa: E402


def oracle_chain(img, f32=False):
    """The same chain, one full pass per op (f32=True: the plain per-op CPU pipeline)."""
    return O.encode(O.SRGB_RGBA8, oracle_chain_linear(img, f32), f32=f32)


def oracle_chain_linear(img, f32=False):
    h, w = img.shape[:2]
    x = O.decode(O.SRGB_RGBA8, rgba_bytes(img), w, h, f32=f32)
    a1 = np.linalg.inv(O.rgb_to_xyz("Bt709", "D50")) @ O.adaptation("BradfordVonKries", "D65", "D50") @ O.rgb_to_xyz()
    O.mat3(x, a1, f32=f32)
    O.oklab_encode(x, O.rgb_to_xyz("Bt709", "D50"), f32=f32)
    O.mat3(x, np.asarray(OKLAB_SCALE).reshape(3, 3), f32=f32)
    O.oklab_decode(x, np.linalg.inv(O.rgb_to_xyz("Bt709", "D50")), f32=f32)
    a2 = np.linalg.inv(O.rgb_to_xyz()) @ O.adaptation("BradfordVonKries", "D50", "D65") @ O.rgb_to_xyz("Bt709", "D50")
    O.mat3(x, a2, f32=f32)
    return x


def rgb_cube_image() -> np.ndarray:
    """4096 x 4096 RGBA8 holding every RGB triple exactly once: pixel i has colour
    (i * 0x9E3779B1) mod 2^24 (an odd multiplier permutes the 2^24 values), alpha a hash
    of i (all 256 codes occur)."""
    i = np.arange(1 << 24, dtype=np.uint64)
    c = (i * np.uint64(0x9E3779B1)) & np.uint64(0xFFFFFF)
    out = np.empty((4096, 4096, 4), dtype=np.uint8)
    flat = out.reshape(-1, 4)
    flat[:, 0] = (c >> np.uint64(16)).astype(np.uint8)
    flat[:, 1] = ((c >> np.uint64(8)) & np.uint64(255)).astype(np.uint8)
    flat[:, 2] = (c & np.uint64(255)).astype(np.uint8)
    flat[:, 3] = ((i ^ (i >> np.uint64(9)) ^ (i >> np.uint64(17))) & np.uint64(255)).astype(np.uint8)
    return out


# ---------------------------------------------------------------- batched uneven thumbnails


def fit_size(w, h, canvas):
    """Long side -> canvas, short side rounded half away from zero (as the batch kernel)."""
    from zosimos_gb300.workloads import thumbnail_fit
    return thumbnail_fit(w, h, canvas)[:2]


def oracle_thumbnails(images, canvas=256):
    out = []
    for img in images:
        h, w = img.shape[:2]
        tw, th = fit_size(w, h, canvas)
        lin = oracle_chain_linear(img)
        small = O.resample(lin, tw, th, "Box")
        full = np.zeros((canvas, canvas, 4))
        x0, y0 = (canvas - tw) // 2, (canvas - th) // 2
        full[y0:y0 + th, x0:x0 + tw] = small
        out.append(O.encode(O.SRGB_RGBA8, full))
    return out


def ours_thumbnails(images, canvas=256):
    c, _, _ = chain_commands(1, 1)
    exe = zs.Linker.from_included().compile(c).lower_to()
    bufs = []
    for img in images:
        b = zs.DeviceBuffer(img.nbytes)
        b.upload(rgba_bytes(img))
        bufs.append(b)
    out = zs.DeviceBuffer(len(images) * canvas * canvas * 4)
    exe.batch_thumbnails([b.ptr for b in bufs], [im.shape[1] for im in images], [im.shape[0] for im in images],
                         canvas, out.ptr)
    zs.device_synchronize()
    res = out.download(np.empty((len(images), canvas, canvas * 4), np.uint8))
    return [res[i] for i in range(len(images))]


def ours_thumbnail_program(img, canvas=256, mode=zs.Mode.Fused):
    """One thumbnail through its own program (chain -> box fit -> inscribe -> sRGB8)."""
    from zosimos_gb300.workloads import thumbnail
    h, w = img.shape[:2]
    c, i, o = thumbnail(w, h, canvas)
    pool = Pool()
    k = pool.insert_srgb(img)
    return run(c, pool, [(i, k)], [o], mode)[0]


def ours_chain(img, mode=zs.Mode.Fused):
    h, w = img.shape[:2]
    c, i, o = chain_commands(w, h)
    pool = Pool()
    k = pool.insert_srgb(img)
    return run(c, pool, [(i, k)], [o], mode)[0]


# ---------------------------------------------------------------- decode / blend / resize (two images)

from zosimos_gb300.workloads import blend_resize  # noqa: E402


def ours_blend_resize(img_a, img_b, out=(384, 384), mode=zs.Mode.Fused):
    h, w = img_a.shape[:2]
    c, a, b, o = blend_resize(w, h, *out)
    pool = Pool()
    ka, kb = pool.insert_srgb(img_a), pool.insert_srgb(img_b)
    return run(c, pool, [(a, ka), (b, kb)], [o], mode)[0]


def oracle_blend_resize(img_a, img_b, out=(384, 384)):
    h, w = img_a.shape[:2]
    la = O.decode(O.SRGB_RGBA8, rgba_bytes(img_a), w, h)
    lb = O.decode(O.SRGB_RGBA8, rgba_bytes(img_b), w, h)
    O.blend(la, lb, (0, 0), "Over", straight=True)
    canvas = np.zeros((out[1], out[0], 4))
    aff = Affine.new(AffineSample.BiLinear).scale(out[0] / w, out[1] / h)
    O.affine(canvas, la, inv3_f32(aff.transformation), True)
    return O.encode(O.SRGB_RGBA8, canvas)


# ---------------------------------------------------------------- resample sweep (RGBA16F)

from zosimos_gb300.workloads import resample as resample_cmds, rotation as rotation_cmds  # noqa: E402


def f16_bytes(img: np.ndarray) -> np.ndarray:
    h, w = img.shape[:2]
    return np.ascontiguousarray(img.astype(np.float16)).view(np.uint8).reshape(h, w * 8)


def f16_from_bytes(b: np.ndarray, w: int, h: int) -> np.ndarray:
    return np.ascontiguousarray(b).view(np.float16).reshape(h, w, 4).astype(np.float64)


def ours_resample(img16, out, filt, mode=zs.Mode.Fused, simt_resample=False):
    h, w = img16.shape[:2]
    c, i, o = resample_cmds(w, h, out[0], out[1], filt)
    pool = Pool()
    k = pool.insert(Descriptor.linear_rgba_f16(w, h), f16_bytes(img16))
    return f16_from_bytes(run(c, pool, [(i, k)], [o], mode, simt_resample)[0], out[0], out[1])


def resample_plan(w, h, out, filt, simt_resample=False) -> str:
    c, _, _ = resample_cmds(w, h, out[0], out[1], filt)
    exe = zs.Linker.from_included().compile(c).lower_to(Capabilities(simt_resample=simt_resample))
    return exe.describe()


def oracle_resample(img16, out, filt):
    return O.resample(img16.astype(np.float64), out[0], out[1], filt)


def ours_resample_srgb8(img8, out, filt, mode=zs.Mode.Fused):
    """resize_filtered of a native RGBA8 sRGB image (filtered in linear light, stored sRGB)."""
    h, w = img8.shape[:2]
    c = CommandBuffer()
    i = c.input(Descriptor.srgb_rgba8(w, h))
    o, _ = c.output(c.resize_filtered(i, out, filt))
    pool = Pool()
    k = pool.insert(Descriptor.srgb_rgba8(w, h), rgba_bytes(img8))
    return np.frombuffer(run(c, pool, [(i, k)], [o], mode)[0], np.uint8).reshape(out[1], out[0], 4)


def oracle_resample_srgb8(img8, out, filt):
    h, w = img8.shape[:2]
    f = O.Format(O.BITS["UInt8x4"], O.PARTS["RgbA"], O.TRANSFER["Srgb"], True)
    lin = O.decode(f, img8.reshape(h, w * 4), w, h)
    res = O.resample(lin, out[0], out[1], filt)
    return O.encode(f, res).reshape(out[1], out[0], 4)


def ours_rotation(img16, degrees, mode=zs.Mode.Fused):
    h, w = img16.shape[:2]
    c, i, o, _ = rotation_cmds(w, h, degrees)
    pool = Pool()
    k = pool.insert(Descriptor.linear_rgba_f16(w, h), f16_bytes(img16))
    return f16_from_bytes(run(c, pool, [(i, k)], [o], mode)[0], w, h)


def oracle_rotation_rows(img64, degrees, y0, y1):
    """Rows [y0, y1) of oracle_rotation (img64: the source as float64)."""
    h, w = img64.shape[:2]
    _, _, _, rot = rotation_cmds(w, h, degrees)
    band = np.zeros((y1 - y0, w, 4))
    O.affine_rows(band, y0, img64, inv3_f32(rot.transformation), True)
    return band


def oracle_rotation(img16, degrees):
    h, w = img16.shape[:2]
    _, _, _, rot = rotation_cmds(w, h, degrees)
    canvas = np.zeros((h, w, 4))
    O.affine(canvas, img16.astype(np.float64), inv3_f32(rot.transformation), True)
    return canvas


# ---------------------------------------------------------------- layer compositing stack

from zosimos_gb300.workloads import BLEND_CYCLE, layer_affine, layer_stack  # noqa: E402


def ours_layer_stack(layers16, transforms, mode=zs.Mode.Fused):
    h, w = layers16[0].shape[:2]
    c, inputs, o = layer_stack(w, h, transforms)
    pool = Pool()
    d16 = Descriptor.linear_rgba_f16(w, h).with_color(alpha=1)
    binds = [(reg, pool.insert(d16, f16_bytes(img))) for reg, img in zip(inputs, layers16)]
    return f16_from_bytes(run(c, pool, binds, [o], mode)[0], w, h)


def oracle_layer_stack(layers16, transforms):
    h, w = layers16[0].shape[:2]
    acc = np.zeros((h, w, 4))
    for i, (img, (deg, s)) in enumerate(zip(layers16, transforms)):
        placed = np.zeros((h, w, 4))
        O.affine(placed, img.astype(np.float64), inv3_f32(layer_affine(w, h, deg, s).transformation), True)
        O.blend(acc, placed, (0, 0), BLEND_CYCLE[i % 4], straight=False)
    return acc


def oracle_layer_stack_rows(layers16, transforms, y0, y1):
    """Rows [y0, y1) of oracle_layer_stack: each layer painted into the band with the pixel
    centres of the full image, then blended onto the band's accumulator."""
    h, w = layers16[0].shape[:2]
    acc = np.zeros((y1 - y0, w, 4))
    for i, (img, (deg, s)) in enumerate(zip(layers16, transforms)):
        placed = np.zeros((y1 - y0, w, 4))
        O.affine_rows(placed, y0, img.astype(np.float64), inv3_f32(layer_affine(w, h, deg, s).transformation), True)
        O.blend(acc, placed, (0, 0), BLEND_CYCLE[i % 4], straight=False)
    return acc


# ---------------------------------------------------------------- blend.rs:577-620 derivative


def ours_derivative(bg, method, direction=zs.Direction.Width, mode=zs.Mode.Fused):
    pool = Pool()
    kb = pool.insert_srgb(bg)
    c = CommandBuffer()
    i = c.input(pool.descriptor(kb))
    o, _ = c.output(c.derivative(i, method, direction))
    return run(c, pool, [(i, kb)], [o], mode)[0]


def oracle_derivative(bg, method: str, width=True):
    h, w = bg.shape[:2]
    lin = O.decode(O.SRGB_RGBA8, rgba_bytes(bg), w, h)
    return O.encode(O.SRGB_RGBA8, O.box3(lin, O.derivative_matrix(method, width)))
