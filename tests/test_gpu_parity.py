"""GPU parity: the executor's CUDA path against the CPU oracle and the reference's
golden hashes.  Integer work (copies, gathers, nearest coordinates, transmute) must
be bit-exact; 8-bit outputs of colour arithmetic within 1 LSB of the FP64 oracle."""
import numpy as np
import pytest

import pipelines as P
import zosimos_gb300 as zs
from imgutil import blockhash256
from zosimos_gb300.synthetic import srgb_gradient_noise

pytestmark = pytest.mark.gpu
LSB = 1   # tolerance of 8-bit outputs against the FP64 oracle


def maxdiff(a, b):
    return int(np.abs(a.astype(np.int64) - b.astype(np.int64)).max())


@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32, zs.Mode.PerOpF16])
@pytest.mark.parametrize("shape", [(256, 256), (29, 37), (1, 1), (3, 5)])
def test_chain_vs_oracle(mode, shape):
    h, w = shape
    img = srgb_gradient_noise(w, h, seed=1)
    ours = P.ours_chain(img, mode)
    ref = P.oracle_chain(img)
    assert ours.shape == ref.shape
    assert maxdiff(ours, ref) <= LSB
    # alpha is carried exactly
    assert (ours.reshape(h, w, 4)[..., 3] == img[..., 3]).all()


def test_identity_chain_is_bit_exact():
    """sRGB8 -> linear FP32 -> sRGB8 folds to an empty program: the fused kernel's
    decode table and exact round-to-nearest encode must reproduce every byte."""
    v = np.arange(256, dtype=np.uint8)
    img = np.stack(np.meshgrid(v, v[::-1]), -1)                     # 256 x 256 x 2
    img = np.concatenate([img, (img[..., :1] ^ 0x5A), img[..., 1:] ^ 0x33], -1).astype(np.uint8)
    c = zs.CommandBuffer()
    d = zs.Descriptor.srgb_rgba8(256, 256)
    i = c.input(d)
    lin = c.color_convert(i, zs.Descriptor.linear_rgba_f32(256, 256))
    back = c.color_convert(lin, d)
    o, _ = c.output(back)
    exe = zs.Linker.from_included().compile(c).lower_to()
    assert "fused chain kernel" in exe.describe()
    out = np.empty((256, 1024), np.uint8)
    exe.run_host([P.rgba_bytes(img)], [out])
    assert (out == P.rgba_bytes(img)).all()


def test_chain_is_one_kernel():
    c, _, _ = P.chain_commands(64, 64)
    exe = zs.Linker.from_included().compile(c).lower_to()
    assert exe.kernel_count() == 1
    assert "fused chain kernel" in exe.describe()


def test_chain_run_host_and_device_agree():
    img = srgb_gradient_noise(512, 384, seed=2)
    c, _, _ = P.chain_commands(512, 384)
    exe = zs.Linker.from_included().compile(c).lower_to()
    out_h = np.empty((384, 512 * 4), np.uint8)
    exe.run_host([P.rgba_bytes(img)], [out_h])
    src = zs.DeviceBuffer(img.nbytes)
    dst = zs.DeviceBuffer(img.nbytes)
    src.upload(P.rgba_bytes(img))
    exe.run_device([src.ptr], [dst.ptr])
    exe.run_device([src.ptr], [dst.ptr])     # graph replay
    zs.device_synchronize()
    out_d = dst.download(np.empty_like(out_h))
    assert (out_h == out_d).all()
    assert maxdiff(out_h, P.oracle_chain(img)) <= LSB


def test_chain_run_host_striped():
    # 2048 x 2050 RGBA8 (16.4 MiB): run_host splits the pixel-local chain into row stripes on
    # three streams; the result must equal the one-launch device path byte for byte.
    w, h = 2048, 2050
    img = srgb_gradient_noise(w, h, seed=6)
    c, _, _ = P.chain_commands(w, h)
    exe = zs.Linker.from_included().compile(c).lower_to()
    out_h = np.empty((h, w * 4), np.uint8)
    exe.run_host([P.rgba_bytes(img)], [out_h])
    src = zs.DeviceBuffer(img.nbytes)
    dst = zs.DeviceBuffer(img.nbytes)
    src.upload(P.rgba_bytes(img))
    exe.run_device([src.ptr], [dst.ptr])
    zs.device_synchronize()
    out_d = dst.download(np.empty_like(out_h))
    assert (out_h == out_d).all()
    assert maxdiff(out_h[:64], P.oracle_chain(img[:64])) <= LSB


@pytest.mark.parametrize("zero_copy", [True, False])
def test_chain_run_host_pinned(zero_copy):
    # Pinned host buffers: the lone chain runs zero copy (the kernel reads and writes host
    # memory directly) or, with zero_copy off, through staged row stripes; both give the
    # device-resident result byte for byte.
    import ctypes
    w, h = 2048, 2050
    img = P.rgba_bytes(srgb_gradient_noise(w, h, seed=8))
    c, _, _ = P.chain_commands(w, h)
    exe = zs.Linker.from_included().compile(c).lower_to(zs.Capabilities(zero_copy=zero_copy))
    lib = zs._lib()
    hin, hout = lib.zs_host_alloc(img.nbytes), lib.zs_host_alloc(img.nbytes)
    try:
        ctypes.memmove(hin, img.ctypes.data, img.nbytes)
        before = zs.kernel_launch_count()
        zs._check(lib.zs_run_host(exe._h, (ctypes.c_void_p * 1)(hin), 1, (ctypes.c_void_p * 1)(hout), 1))
        launches = zs.kernel_launch_count() - before
        out_h = np.empty_like(img)
        ctypes.memmove(out_h.ctypes.data, hout, img.nbytes)
    finally:
        lib.zs_host_free(hin)
        lib.zs_host_free(hout)
    assert launches == (1 if zero_copy else 8)
    src, dst = zs.DeviceBuffer(img.nbytes), zs.DeviceBuffer(img.nbytes)
    src.upload(img)
    exe.run_device([src.ptr], [dst.ptr])
    zs.device_synchronize()
    assert (out_h == dst.download(np.empty_like(img))).all()


def test_composed(background, foreground, goldens):
    ours = P.ours_composed(background, foreground)
    assert (ours == P.oracle_composed(background, foreground)).all()
    assert blockhash256(ours.reshape(512, 512, 4)) in goldens["composed"]


@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_affine_nearest(background, foreground, goldens, mode):
    ours = P.ours_affine(background, foreground, mode=mode)
    assert (ours == P.oracle_affine(background, foreground)).all()
    assert blockhash256(ours.reshape(512, 512, 4)) in goldens["affine"]


def test_affine_bilinear(background, foreground):
    ours = P.ours_affine(background, foreground, zs.AffineSample.BiLinear)
    assert maxdiff(ours, P.oracle_affine_bilinear(background, foreground)) <= LSB


def test_adapted(background, goldens):
    ours = P.ours_adapted(background)
    assert maxdiff(ours, P.oracle_adapted(background)) <= LSB
    assert blockhash256(ours.reshape(512, 512, 4)) in goldens["adapted"]


def test_convert_bt709(background, goldens):
    ours = P.ours_convert_bt709(background)
    assert maxdiff(ours, P.oracle_convert_bt709(background)) <= LSB
    assert blockhash256(ours.reshape(512, 512, 4)) in goldens["convert_bt709"]


@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_swapped(background, goldens, mode):
    ours = P.ours_swapped(background, mode)
    assert maxdiff(ours, P.oracle_swapped(background)) <= LSB
    assert blockhash256(ours.reshape(512, 512, 4)) in goldens["swapped"]


def test_transmute_bytes_exact(background):
    # tests/blend.rs:371-372: the transmuted image has exactly the input bytes.
    ours = P.ours_transmute(background)
    assert (ours == P.rgba_bytes(background)).all()


def test_palette(background, goldens):
    ours = P.ours_palette(background)
    assert (ours == P.oracle_palette(background)).all()
    h = blockhash256(ours.reshape(400, 400, 4))
    assert min(bin(int(h, 16) ^ int(g, 16)).count("1") for g in goldens["palette"]) <= 8


@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_generic_palette(background, goldens, mode):
    # lib/zosimos/tests/generic.rs: a generic palette function invoked on the background and
    # linked; the 2048^2 output is a byte-exact gather of the oracle's indices.
    ours = P.ours_generic(background, mode)
    assert (ours == P.oracle_generic(background)).all()
    assert blockhash256(ours.reshape(2048, 2048, 4)) in goldens["generic"]


def test_linked_instantiations_equal_flat_program():
    # one generic resize function called for two descriptors; the linked program's outputs are
    # the flat program's, byte for byte (both run on the device)
    img = srgb_gradient_noise(300, 200, seed=7)
    pool = zs.Pool()
    ka = pool.insert_srgb(img)
    kb = pool.insert(zs.Descriptor.linear_rgba_f32(300, 200), img.astype(np.float32) / 255.0)

    f = zs.CommandBuffer()
    a = f.generic()
    f.output(f.resize_filtered(f.input_generic(a), (96, 64), zs.Filter.Lanczos3))
    c = zs.CommandBuffer()
    fn = c.function(f)
    x = c.input(pool.descriptor(ka))
    y = c.input(pool.descriptor(kb))
    (rx,) = c.invoke(fn, generics=[c.register_descriptor(x)], arguments=[x])
    (ry,) = c.invoke(fn, generics=[c.register_descriptor(y)], arguments=[y])
    ox, _ = c.output(rx)
    oy, _ = c.output(ry)
    exe = zs.Linker.from_included().link(c, [], [f], [[1], []]).lower_to()
    env = exe.from_pool(pool)
    env.bind(x, ka)
    env.bind(y, kb)
    ex = exe.launch(env)
    while ex.is_running():
        ex.step()
    linked = [pool.read(ex.retire_output(o)) for o in (ox, oy)]

    flat = zs.CommandBuffer()
    x2 = flat.input(pool.descriptor(ka))
    y2 = flat.input(pool.descriptor(kb))
    o2 = [flat.output(flat.resize_filtered(r, (96, 64), zs.Filter.Lanczos3))[0] for r in (x2, y2)]
    keys = zs.run_pipeline(flat, pool, [(x2, ka), (y2, kb)], o2)
    for got, key in zip(linked, keys):
        assert (got == pool.read(key)).all()


@pytest.mark.parametrize("space", ["oklab", "srlab2"])
def test_lab_grid(space, goldens):
    ours = P.ours_lab_grid(space)
    assert maxdiff(ours, P.oracle_lab_grid(space)) <= LSB
    assert blockhash256(ours.reshape(400, 400, 4)) in goldens[space]


@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32, zs.Mode.PerOpF16])
def test_blend_resize(mode):
    a = srgb_gradient_noise(512, 512, seed=1, image=0)
    b = srgb_gradient_noise(512, 512, seed=1, image=1)
    ours = P.ours_blend_resize(a, b, mode=mode)
    assert maxdiff(ours, P.oracle_blend_resize(a, b)) <= LSB


F16_TOL = 2.0e-3   # max-abs error of RGBA16F outputs in [0, 1] against FP64 (f16 storage ~4.9e-4/step)


@pytest.mark.parametrize("filt", [zs.Filter.Lanczos3, zs.Filter.Box, zs.Filter.Triangle])
@pytest.mark.parametrize("factor", [2.0, 3.7, 8.0])
@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_resample(filt, factor, mode):
    from zosimos_gb300.synthetic import linear_gradient_gauss
    img = linear_gradient_gauss(1024, 768, seed=3)
    out = (int(round(1024 / factor)), int(round(768 / factor)))
    ours = P.ours_resample(img, out, filt, mode)
    ref = P.oracle_resample(img, out, filt)
    assert ours.shape == ref.shape
    assert np.abs(ours - ref).max() <= F16_TOL


def test_resample_upscale():
    from zosimos_gb300.synthetic import linear_gradient_gauss
    img = linear_gradient_gauss(100, 60, seed=5)
    ours = P.ours_resample(img, (317, 200), zs.Filter.Lanczos3)
    assert np.abs(ours - P.oracle_resample(img, (317, 200), zs.Filter.Lanczos3)).max() <= F16_TOL


@pytest.mark.parametrize("filt", [zs.Filter.Lanczos3, zs.Filter.Box, zs.Filter.Triangle])
@pytest.mark.parametrize("src,out", [((1024, 768), (512, 384)), ((1024, 768), (277, 208)), ((640, 300), (640, 131)),
                                     ((200, 130), (317, 200)), ((518, 390), (129, 97)), ((1024, 768), (128, 96)),
                                     ((1040, 300), (130, 37))])
def test_resample_tensor_cores(filt, src, out):
    # The vertical pass on the tensor cores (f16 band matrices, FP32 accumulation in TMEM),
    # against FP64, and against the FP32 SIMT kernel on the same input.
    from zosimos_gb300.synthetic import linear_gradient_gauss
    img = linear_gradient_gauss(src[0], src[1], seed=13)
    plan = P.resample_plan(src[0], src[1], out, filt)
    ours = P.ours_resample(img, out, filt)
    simt = P.ours_resample(img, out, filt, simt_resample=True)
    ref = P.oracle_resample(img, out, filt)
    assert np.abs(ours - ref).max() <= F16_TOL, plan
    assert np.abs(simt - ref).max() <= F16_TOL
    assert np.abs(ours - simt).max() <= F16_TOL


def test_resample_tensor_core_plan():
    # RGBA16F sources with 16-byte rows take the tensor-core kernel where the staged columns
    # of a tile fit one MMA; the SIMT flag and odd widths keep the FP32 SIMT kernel.
    assert "tensor cores" in P.resample_plan(1024, 768, (512, 384), zs.Filter.Lanczos3)
    assert "tensor cores" in P.resample_plan(1024, 768, (128, 96), zs.Filter.Lanczos3)   # 8 atoms, one accumulator
    assert "tensor cores" not in P.resample_plan(1024, 768, (512, 384), zs.Filter.Lanczos3, simt_resample=True)
    assert "tensor cores" not in P.resample_plan(1023, 768, (512, 384), zs.Filter.Lanczos3)


@pytest.mark.parametrize("src,out", [((301, 203), (150, 101)), ((301, 203), (37, 25)), ((257, 64), (600, 31))])
@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_resample_ragged(src, out, mode):
    # Row strides that are not a multiple of 16 bytes (rows staged with plain loads),
    # partial edge tiles, and a horizontal upscale with a vertical downscale.
    from zosimos_gb300.synthetic import linear_gradient_gauss
    img = linear_gradient_gauss(src[0], src[1], seed=11)
    ours = P.ours_resample(img, out, zs.Filter.Lanczos3, mode)
    assert np.abs(ours - P.oracle_resample(img, out, zs.Filter.Lanczos3)).max() <= F16_TOL


@pytest.mark.parametrize("filt", [zs.Filter.Lanczos3, zs.Filter.Box, zs.Filter.Triangle])
def test_resample_srgb8(filt):
    # 8-bit sRGB source and target: decoded through the LUT, filtered in FP32 linear light,
    # encoded with the exact round-to-nearest table; within one 8-bit step of FP64.
    from zosimos_gb300.synthetic import srgb_gradient_noise
    img = srgb_gradient_noise(640, 480, seed=9)
    out = (256, 192)
    ours = P.ours_resample_srgb8(img, out, filt).astype(np.int32)
    ref = P.oracle_resample_srgb8(img, out, filt).astype(np.int32)
    assert np.abs(ours - ref).max() <= 1


@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_rotation(mode):
    from zosimos_gb300.synthetic import linear_gradient_gauss
    img = linear_gradient_gauss(640, 480, seed=3)
    ours = P.ours_rotation(img, 17.0, mode)
    ref = P.oracle_rotation(img, 17.0)
    # coverage (pixel centre inside the rotated quad) is decided in identical f32 arithmetic
    assert ((ours[..., 3] == 0) == (ref[..., 3] == 0)).all()
    assert np.abs(ours - ref).max() <= F16_TOL


@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_layer_stack(mode):
    from zosimos_gb300.synthetic import layer_transforms, premultiplied_layer
    n, w, h = 6, 384, 256
    layers = [premultiplied_layer(w, h, seed=5, image=i) for i in range(n)]
    transforms = layer_transforms(n, seed=5)
    ours = P.ours_layer_stack(layers, transforms, mode)
    ref = P.oracle_layer_stack(layers, transforms)
    assert np.abs(ours - ref).max() <= F16_TOL


def test_layer_stack_is_one_kernel():
    from zosimos_gb300.synthetic import layer_transforms
    c, _, _ = P.layer_stack(256, 256, layer_transforms(32))
    exe = zs.Linker.from_included().compile(c).lower_to()
    assert exe.kernel_count() == 1 and "32 layers" in exe.describe()


def test_batch_thumbnails():
    from zosimos_gb300.synthetic import thumbnail_sizes
    ws, hs = thumbnail_sizes(10, seed=4, lo=40, hi=700)
    images = [srgb_gradient_noise(int(w), int(h), seed=4, image=i) for i, (w, h) in enumerate(zip(ws, hs))]
    images.append(srgb_gradient_noise(100, 60, seed=4, image=99))     # upscale case
    ours = P.ours_thumbnails(images, 256)
    ref = P.oracle_thumbnails(images, 256)
    for o, r in zip(ours, ref):
        assert maxdiff(o, r) <= LSB


def test_batch_thumbnails_graph_replay():
    """The batch launch is captured as a CUDA graph once and replayed for later batches with
    the same output buffer, count and canvas (the per-batch image table is uploaded before
    each replay); a different canvas captures anew.  Every batch matches the oracle."""
    from zosimos_gb300.synthetic import thumbnail_sizes
    c, _, _ = P.chain_commands(1, 1)
    exe = zs.Linker.from_included().compile(c).lower_to()
    out = zs.DeviceBuffer(6 * 128 * 128 * 4)
    for seed, canvas in ((6, 128), (7, 128), (8, 96), (9, 128)):
        ws, hs = thumbnail_sizes(6, seed=seed, lo=33, hi=900)
        images = [srgb_gradient_noise(int(w), int(h), seed=seed, image=i) for i, (w, h) in enumerate(zip(ws, hs))]
        bufs = []
        for img in images:
            b = zs.DeviceBuffer(img.nbytes)
            b.upload(P.rgba_bytes(img))
            bufs.append(b)
        exe.batch_thumbnails([b.ptr for b in bufs], [im.shape[1] for im in images], [im.shape[0] for im in images],
                             canvas, out.ptr)
        zs.device_synchronize()
        got = out.download(np.empty(out.nbytes, np.uint8))[:6 * canvas * canvas * 4].reshape(6, canvas, canvas * 4)
        for k, r in enumerate(P.oracle_thumbnails(images, canvas)):
            assert maxdiff(got[k], r) <= LSB, (seed, k)


@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_thumbnail_program_matches_batch(mode):
    # The one-program-per-image form of the batched thumbnails (chain, box fit, centred
    # inscribe onto a transparent canvas) gives the batch kernel's result within 1 LSB.
    from zosimos_gb300.synthetic import thumbnail_sizes
    ws, hs = thumbnail_sizes(4, seed=5, lo=40, hi=700)
    images = [srgb_gradient_noise(int(w), int(h), seed=5, image=i) for i, (w, h) in enumerate(zip(ws, hs))]
    images.append(srgb_gradient_noise(100, 60, seed=5, image=99))     # upscale case
    batch = P.ours_thumbnails(images, 256)
    ref = P.oracle_thumbnails(images, 256)
    for img, b, r in zip(images, batch, ref):
        one = P.ours_thumbnail_program(img, 256, mode)
        assert maxdiff(one, r) <= LSB
        assert maxdiff(one, b) <= LSB


def test_blend_resize_plan():
    c, _, _, _ = P.blend_resize()
    fused = zs.Linker.from_included().compile(c).lower_to()
    plain = zs.Linker.from_included().compile(c).lower_to(zs.Capabilities(mode=zs.Mode.PerOpF32))
    assert fused.kernel_count() < plain.kernel_count()


def test_bounded_wait_timeout_is_reported():
    # Failure detection without a GPU fault: a wait that nothing completes gives up after its
    # limit, the status word reports it once (reading clears it), and the context still works.
    import time
    assert zs.device_status(0) == 0
    t0 = time.perf_counter()
    zs.selftest_wait_timeout(0, 2000)
    assert time.perf_counter() - t0 < 5.0
    assert zs.device_status(0) == 1
    assert zs.device_status(0) == 0
    img = srgb_gradient_noise(64, 48, seed=1)
    assert maxdiff(P.ours_chain(img), P.oracle_chain(img)) <= LSB


@pytest.mark.parametrize("src,out", [((4, 2), (1, 1)), ((6, 7), (2, 3)), ((2, 2), (9, 5)), ((3, 2), (1, 1)),
                                     ((5, 7), (2, 3)), ((16, 1), (3, 1)), ((2, 300), (2, 7))])
@pytest.mark.parametrize("simt", [False, True])
def test_resample_tiny(src, out, simt):
    # Images smaller than one tile, one TMA box or one 16-byte row; 1 x 1 results.
    from zosimos_gb300.synthetic import linear_gradient_gauss
    img = linear_gradient_gauss(src[0], src[1], seed=17)
    for filt in (zs.Filter.Lanczos3, zs.Filter.Box, zs.Filter.Triangle):
        ours = P.ours_resample(img, out, filt, simt_resample=simt)
        assert np.abs(ours - P.oracle_resample(img, out, filt)).max() <= F16_TOL


@pytest.mark.parametrize("method", ["Prewitt", "Sobel", "Scharr3", "Scharr3To4Bit", "Scharr3To8Bit"])
@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_derivative(background, goldens, method, mode):
    # tests/blend.rs:577-620 (width), plus the height direction against the oracle.
    m = getattr(zs.DerivativeMethod, method)
    ours = P.ours_derivative(background, m, zs.Direction.Width, mode)
    assert maxdiff(ours, P.oracle_derivative(background, method, True)) <= LSB
    assert blockhash256(ours.reshape(512, 512, 4)) in goldens["derived_" + method]
    ours_h = P.ours_derivative(background, m, zs.Direction.Height, mode)
    assert maxdiff(ours_h, P.oracle_derivative(background, method, False)) <= LSB


@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_from_buffer(mode):
    # tests/buffer.rs:39-65: an 8 x 8 Luma8 image read from a buffer of 256-byte rows, all 0xFF
    # except row 1; the result is exactly those rows.
    import oracle as O
    luma = zs.Descriptor(8, 8, zs.Bits.UInt8, zs.Parts.Luma, zs.ColorKind.Rgb, zs.Primaries.Bt709,
                         zs.Transfer.Srgb, zs.Whitepoint.D65)
    a = np.full(8 * 256, 0xFF, np.uint8)
    a[256:264] = 0
    c = zs.CommandBuffer()
    o, _ = c.output(c.from_buffer(c.buffer_init(a), luma))
    ours = np.frombuffer(P.run(c, zs.Pool(), [], [o], mode)[0], np.uint8).reshape(8, 8)
    want = np.full((8, 8), 0xFF, np.uint8)
    want[1] = 0
    assert (ours == want).all()
    # RGBA8 rows of 100 texels (400 bytes, rows 512 bytes apart) from seeded bytes: the image is
    # bit-exact, and a colour conversion of it agrees with the oracle.
    rng = np.random.default_rng(7)
    buf = rng.integers(0, 256, 512 * 37 + 100, dtype=np.uint8)
    img = buf[:512 * 37].reshape(37, 512)[:, :400].reshape(37, 100, 4)
    c = zs.CommandBuffer()
    r = c.from_buffer(c.buffer_init(buf), zs.Descriptor.srgb_rgba8(100, 37))
    o1, _ = c.output(r)
    o2, _ = c.output(c.color_convert(r, zs.Descriptor.linear_rgba_f16(100, 37)))
    raw, lin = P.run(c, zs.Pool(), [], [o1, o2], mode)
    assert (np.frombuffer(raw, np.uint8).reshape(37, 400) == img.reshape(37, 400)).all()
    got = np.frombuffer(lin, np.float16).reshape(37, 100, 4).astype(np.float64)
    want = O.decode(O.SRGB_RGBA8, np.ascontiguousarray(img.reshape(37, 400)), 100, 37)
    assert np.abs(got - want).max() <= 1e-3


@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_distribution_fractal_noise(goldens, mode):
    # tests/blend.rs:314-338: 400 x 400 sRGB RGBA8 fractal noise, 4 octaves.  The hash and the
    # arithmetic are restated in f32 with the same rounding steps, so the linear values agree
    # with the oracle to a few ulps and the 8-bit result within one code.
    import oracle as O
    params = zs.fractal_noise_with_octaves(4)
    c = zs.CommandBuffer()
    o, _ = c.output(c.distribution_fractal_noise(zs.Descriptor.srgb_rgba8(400, 400), params))
    ours = np.frombuffer(P.run(c, zs.Pool(), [], [o], mode)[0], np.uint8).reshape(400, 1600)
    want = O.encode(O.SRGB_RGBA8, O.fractal_noise(400, 400, params))
    assert maxdiff(ours, want) <= LSB
    assert blockhash256(ours.reshape(400, 400, 4)) in goldens["distribution_fractal2d"]
    # Damped octaves and a non-square grid.
    p2 = zs.fractal_noise_set_damping(zs.fractal_noise_with_octaves(6), 0.6)
    p2[0], p2[1] = 37.0, 12.5
    c = zs.CommandBuffer()
    o, _ = c.output(c.distribution_fractal_noise(zs.Descriptor.srgb_rgba8(123, 77), p2))
    ours = np.frombuffer(P.run(c, zs.Pool(), [], [o], mode)[0], np.uint8).reshape(77, 123 * 4)
    assert maxdiff(ours, O.encode(O.SRGB_RGBA8, O.fractal_noise(123, 77, p2))) <= LSB


@pytest.mark.parametrize("case", ["normal2d", "normal1d", "u8"])
def test_distribution_normal2d(goldens, case):
    # tests/blend.rs:227-311.
    import oracle as O
    from imgutil import luma_alpha16_to_rgba8
    params = zs.normal2d_with_diagonal(0.2, 0.2) if case == "normal2d" else zs.normal2d_with_direction(0.04998, 0.0501)
    if case == "u8":
        d = zs.Descriptor(400, 400, zs.Bits.UInt8, zs.Parts.Luma, zs.ColorKind.Rgb, zs.Primaries.Bt709,
                          zs.Transfer.Srgb, zs.Whitepoint.D65)
        f = O.Format(O.BITS["UInt8"], O.PARTS["Luma"], O.TRANSFER["Srgb"], False)
    else:
        d = P.luma_alpha16_desc(400, 400)
        f = O.Format(O.BITS["UInt16x2"], O.PARTS["LumaA"], O.TRANSFER["Srgb"], False)
    c = zs.CommandBuffer()
    o, _ = c.output(c.distribution_normal2d(d, params))
    ours = np.frombuffer(P.run(c, zs.Pool(), [], [o])[0], np.uint8).reshape(400, -1)
    want = O.encode(f, O.normal2d(400, 400, params))
    # within one code of the FP64 oracle (truncating quantisation of FP32 against FP64)
    fl = O.Format(f.bits, f.parts, O.TRANSFER["Linear"], False)
    got_c, want_c = O.decode(fl, ours, 400, 400), O.decode(fl, want, 400, 400)
    assert np.abs(got_c - want_c).max() <= (1.0001 / 255 if case == "u8" else 1.0001 / 65535)
    if case == "u8":
        rgba = np.stack([ours, ours, ours, np.full_like(ours, 255)], -1)
        h = blockhash256(rgba)
        assert min(bin(int(h, 16) ^ int(a, 16)).count("1") for a in goldens["distribution_u8"]) <= 3
    else:
        assert blockhash256(luma_alpha16_to_rgba8(ours)) in goldens["distribution_" + case]


@pytest.mark.parametrize("rect", [(100, 50, 356, 306), (0, 0, 512, 512), (17, 301, 18, 512), (200, 10, 461, 139)])
@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_crop(background, rect, mode):
    """CommandBuffer::crop (command.rs:971): the result keeps the source descriptor and the
    selection is painted over it by the quad copy (copy.frag + box.vert): byte exact."""
    pool = zs.Pool()
    k = pool.insert_srgb(background)
    c = zs.CommandBuffer()
    i = c.input(pool.descriptor(k))
    o, _ = c.output(c.crop(i, zs.Rectangle(*rect)))
    ours = P.run(c, pool, [(i, k)], [o], mode)[0]
    want = np.zeros((512, 512 * 4), np.uint8)
    P.O.gather_quad(P.rgba_bytes(background), 512, 512, want, 512, 512, 4, (0, 0, 512, 512), selection=rect)
    assert (ours == want).all()


@pytest.mark.parametrize("size", [(384, 384), (157, 151), (1000, 700), (1, 1), (512, 3)])
@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_resize_reference_nearest(background, size, mode):
    """CommandBuffer::resize (command.rs:1675-1702): a bilinear coordinate grid stored as
    truncated 8-bit texels feeding a nearest palette lookup -- an integer gather, byte exact
    against the oracle's index tables."""
    pool = zs.Pool()
    k = pool.insert_srgb(background)
    c = zs.CommandBuffer()
    i = c.input(pool.descriptor(k))
    o, _ = c.output(c.resize(i, size))
    ours = P.run(c, pool, [(i, k)], [o], mode)[0]
    ix = P.O.resize_ref_index(512, size[0])
    iy = P.O.resize_ref_index(512, size[1])
    assert (ours == P.rgba_bytes(background[iy][:, ix])).all()


def test_pool_upload_device_resident_input():
    """Pool::upload (pool.rs:292): a device-resident pool image is bound without a host
    copy (zs_pool_device_ptr exposes it) and gives the same result as a host image."""
    img = srgb_gradient_noise(333, 211, seed=21)
    c, i, o = P.chain_commands(333, 211)
    pool = zs.Pool()
    k = pool.insert_srgb(img)
    pool.upload(k)
    ptr = pool.device_ptr(k)
    assert ptr
    # the device copy holds the image bytes
    dev = np.empty((211, 333 * 4), np.uint8)
    zs._check(zs._lib().zs_memcpy_d2h(dev.ctypes.data, ptr, dev.nbytes))
    assert (dev == P.rgba_bytes(img)).all()
    ours = P.run(c, pool, [(i, k)], [o])[0]
    assert maxdiff(ours, P.oracle_chain(img)) <= LSB


def test_resample_tile_widths_give_identical_bytes():
    """Every tile width the tensor-core resample fits (the autotuner's candidates) computes the
    same bytes, and the autotuner keeps one of them."""
    img = P.f16_bytes(np.random.default_rng(31).random((700, 900, 4)).astype(np.float16))
    from zosimos_gb300.workloads import resample as resample_cmds
    c, _, _ = resample_cmds(900, 700, 450, 350, zs.Filter.Lanczos3)
    exe = zs.Linker.from_included().compile(c).lower_to()
    assert "tensor cores" in exe.describe()
    src, dst = zs.DeviceBuffer(img.nbytes), zs.DeviceBuffer(450 * 350 * 8)
    src.upload(img)
    outs = []
    for tw in (8, 16, 32):
        exe.set_launch(zs.Tune.ResampleTile, tw)
        exe.run_device([src.ptr], [dst.ptr])
        zs.device_synchronize()
        outs.append(dst.download(np.empty((350, 450 * 8), np.uint8)))
    assert all((o == outs[0]).all() for o in outs[1:])
    exe.autotune([src.ptr], [dst.ptr], reps=3)
    assert exe.get_launch(zs.Tune.ResampleTile) in (8, 16, 32)
    exe.run_device([src.ptr], [dst.ptr])
    zs.device_synchronize()
    assert (dst.download(np.empty((350, 450 * 8), np.uint8)) == outs[0]).all()


def test_step_to_retire_input_and_recover_buffers():
    """Execution::step_to with StepLimits (run.rs:1394, 3000-3013), Retire::input (run.rs:2791)
    and Environment::recover_buffers (run.rs:1312-1347) on a two-kernel program (blend +
    bilinear resize, per-op FP32 so that an intermediate is held)."""
    a = srgb_gradient_noise(64, 64, seed=23, image=0)
    b = srgb_gradient_noise(64, 64, seed=23, image=1)
    from zosimos_gb300.workloads import blend_resize
    c, ia, ib, o = blend_resize(64, 64, 48, 48)
    exe = zs.Linker.from_included().compile(c).lower_to(zs.Capabilities(mode=zs.Mode.PerOpF32))
    pool = zs.Pool()
    ka, kb = pool.insert_srgb(a), pool.insert_srgb(b)
    for launch in range(2):
        env = exe.from_pool(pool)
        env.bind(ia, ka)
        env.bind(ib, kb)
        held = env.recover_buffers()
        assert (held > 0) == (launch > 0)       # intermediates exist after the first launch
        ex = exe.launch(env)
        total = 0
        while ex.is_running():
            n = ex.step_to(2)
            assert 1 <= n <= 2
            total += n
        assert ex.step_to(5) == 0 and total >= 2
        assert ex.retire_input(ia) == ka and ex.retire_input(ib) == kb
        with pytest.raises(zs.ZosimosError) as e:
            ex.retire_input(o)
        assert e.value.code == 3
        got = pool.read(ex.retire_output(o))
        assert maxdiff(got, P.oracle_blend_resize(a, b, (48, 48))) <= LSB


def test_two_chain_executables_on_the_per_device_path():
    """Two executables whose chains use different kernel specialisations (with and without
    cube roots), lowered for the same device and launched alternately: each launcher sets
    its kernel's shared-memory attribute for the device current at the launch."""
    img = srgb_gradient_noise(300, 200, seed=22)
    c1, i1, o1 = P.chain_commands(300, 200)
    c2 = zs.CommandBuffer()
    j = c2.input(zs.Descriptor.srgb_rgba8(300, 200))
    o2, _ = c2.output(c2.chromatic_adaptation(j, zs.ChromaticAdaptationMethod.BradfordVonKries,
                                              zs.Whitepoint.D50))
    e1 = zs.Linker.from_included().compile(c1).lower_to(zs.Capabilities(device=0))
    e2 = zs.Linker.from_included().compile(c2).lower_to(zs.Capabilities(device=0))
    assert "fused chain kernel" in e1.describe() and "fused chain kernel" in e2.describe()
    out1, out2 = np.empty((200, 1200), np.uint8), np.empty((200, 1200), np.uint8)
    for _ in range(2):
        e1.run_host([P.rgba_bytes(img)], [out1])
        e2.run_host([P.rgba_bytes(img)], [out2])
    assert maxdiff(out1, P.oracle_chain(img)) <= LSB
    lin = P.O.decode(P.O.SRGB_RGBA8, P.rgba_bytes(img), 300, 200)
    m = (np.linalg.inv(P.O.rgb_to_xyz("Bt709", "D50")) @ P.O.adaptation("BradfordVonKries", "D65", "D50")
         @ P.O.rgb_to_xyz())
    P.O.mat3(lin, m)
    assert maxdiff(out2, P.O.encode(P.O.SRGB_RGBA8, lin)) <= LSB


def test_chain_on_buffers_not_16_byte_aligned():
    """Texel-aligned buffers that the chain kernel cannot stream in 16-byte vectors run the
    same fused program on the generic raster kernel; buffers not even texel aligned are an
    argument error, raised before anything is launched."""
    img = srgb_gradient_noise(123, 77, seed=23)
    c, _, _ = P.chain_commands(123, 77)
    exe = zs.Linker.from_included().compile(c).lower_to()
    n = img.nbytes
    src, dst = zs.DeviceBuffer(n + 64), zs.DeviceBuffer(n + 64)
    host = np.zeros(n + 64, np.uint8)
    host[4:4 + n] = P.rgba_bytes(img).reshape(-1)
    src.upload(host)
    exe.run_device([src.ptr + 4], [dst.ptr + 4])
    zs.device_synchronize()
    out = dst.download(np.empty(n + 64, np.uint8))[4:4 + n].reshape(77, 123 * 4)
    assert maxdiff(out, P.oracle_chain(img)) <= LSB
    with pytest.raises(zs.ZosimosError) as err:
        exe.run_device([src.ptr + 1], [dst.ptr])
    assert err.value.code == 10


def _chain_outputs(exe, images):
    bufs, outs = [], []
    for img in images:
        b, o = zs.DeviceBuffer(img.nbytes), zs.DeviceBuffer(img.nbytes)
        b.upload(P.rgba_bytes(img))
        bufs.append(b)
        outs.append(o)
    return bufs, outs


def test_batch_run_device_matches_single_runs():
    """zs_batch_run_device: n runs of one executable as one replayed graph (independent runs on
    parallel branches) give exactly the bytes of n separate runs; the same pointer table again
    replays the cached graph, a new table captures anew."""
    c, _, _ = P.chain_commands(97, 61)
    exe = zs.Linker.from_included().compile(c).lower_to()
    images = [srgb_gradient_noise(97, 61, seed=30, image=k) for k in range(11)]
    bufs, outs = _chain_outputs(exe, images)
    for _ in range(2):
        exe.batch_run_device([[b.ptr] for b in bufs], [[o.ptr] for o in outs])
        zs.device_synchronize()
        for img, o in zip(images, outs):
            got = o.download(np.empty((61, 97 * 4), np.uint8))
            assert maxdiff(got, P.oracle_chain(img)) <= LSB
    single = zs.DeviceBuffer(images[3].nbytes)
    exe.run_device([bufs[3].ptr], [single.ptr])
    zs.device_synchronize()
    assert (single.download(np.empty((61, 97 * 4), np.uint8)) == outs[3].download(np.empty((61, 97 * 4), np.uint8))).all()
    # a different pointer table: a shorter batch over other buffers
    exe.batch_run_device([[b.ptr] for b in bufs[5:]], [[o.ptr] for o in outs[:6]])
    zs.device_synchronize()
    for k in range(6):
        got = outs[k].download(np.empty((61, 97 * 4), np.uint8))
        assert maxdiff(got, P.oracle_chain(images[5 + k])) <= LSB


@pytest.mark.parametrize("mode", [zs.Mode.Fused, zs.Mode.PerOpF32])
def test_batch_run_pool_keys_two_inputs(mode):
    """zs_batch_run over pool keys: a two-input executable (blend + bilinear resize; its per-op
    form stores intermediates, so its runs are recorded one after another) for four pairs of
    images; every run's output is a new pool image matching the oracle."""
    c, a, b, o = P.blend_resize(256, 192, 150, 100)
    exe = zs.Linker.from_included().compile(c).lower_to(zs.Capabilities(mode=mode))
    pool = zs.Pool()
    pairs, keys = [], []
    for k in range(4):
        ia = srgb_gradient_noise(256, 192, seed=31, image=2 * k)
        ib = srgb_gradient_noise(256, 192, seed=31, image=2 * k + 1)
        pairs.append((ia, ib))
        keys.append([pool.insert_srgb(ia), pool.insert_srgb(ib)])
    outs = exe.batch_run(pool, keys)
    assert len(outs) == 4 and all(len(r) == 1 for r in outs)
    for (ia, ib), (ko,) in zip(pairs, outs):
        got = pool.read(ko)
        assert maxdiff(got, P.oracle_blend_resize(ia, ib, (150, 100))) <= LSB


def test_autotune_candidates_are_byte_identical():
    """Every candidate the autotuner times computes the same bytes: the chain kernel at 1024
    and 512 threads per block, the batched thumbnails at 1..16 rows per work item.  The tuned
    choice lands in the cache, so a newly lowered executable starts from it."""
    from zosimos_gb300.synthetic import thumbnail_sizes
    img = srgb_gradient_noise(1024, 768, seed=40)
    c, _, _ = P.chain_commands(1024, 768)
    exe = zs.Linker.from_included().compile(c).lower_to()
    src, dst = zs.DeviceBuffer(img.nbytes), zs.DeviceBuffer(img.nbytes)
    src.upload(P.rgba_bytes(img))
    outs = []
    for t in (1024, 512):
        for vec in (2, 1):
            exe.set_launch(zs.Tune.ChainThreads, t)
            exe.set_launch(zs.Tune.ChainVectors, vec)
            exe.run_device([src.ptr], [dst.ptr])
            zs.device_synchronize()
            outs.append(dst.download(np.empty((768, 4096), np.uint8)))
    assert all((o == outs[0]).all() for o in outs[1:])
    chosen = exe.autotune([src.ptr], [dst.ptr], reps=5)
    assert chosen in (1024, 512) and exe.get_launch(zs.Tune.ChainVectors) in (1, 2)
    again = zs.Linker.from_included().compile(c).lower_to()
    again.run_device([src.ptr], [dst.ptr])            # first use reads the cache
    assert again.get_launch(zs.Tune.ChainThreads) == chosen
    zs.device_synchronize()
    assert (dst.download(np.empty((768, 4096), np.uint8)) == outs[0]).all()

    # 40 images at canvas 256: enough work items that the grid is full for every height, so
    # the launch shape alone cannot tell the candidates apart; each is checked on its own.
    ws, hs = thumbnail_sizes(40, seed=41, lo=48, hi=700)
    images = [srgb_gradient_noise(int(w), int(h), seed=41, image=i) for i, (w, h) in enumerate(zip(ws, hs))]
    c1, _, _ = P.chain_commands(1, 1)
    chain = zs.Linker.from_included().compile(c1).lower_to()
    bufs = []
    for im in images:
        b = zs.DeviceBuffer(im.nbytes)
        b.upload(P.rgba_bytes(im))
        bufs.append(b)
    out = zs.DeviceBuffer(40 * 256 * 256 * 4)
    args = ([b.ptr for b in bufs], [im.shape[1] for im in images], [im.shape[0] for im in images], 256, out.ptr)
    ref = P.oracle_thumbnails(images, 256)
    results = []
    for threads, rows in [(t, r) for t in (768, 640) for r in (1, 2, 4, 8, 16)] + [(768, 2)]:
        chain.set_launch(zs.Tune.BatchThreads, threads)
        chain.set_launch(zs.Tune.BatchRows, rows)
        chain.batch_thumbnails(*args)
        zs.device_synchronize()
        got = out.download(np.empty((40, 256, 1024), np.uint8))
        for k in range(40):
            assert maxdiff(got[k], ref[k]) <= LSB, (threads, rows, k)
        results.append(got)
    assert all((r == results[0]).all() for r in results[1:])
    rows = chain.autotune_batch_thumbnails(*args, reps=2)
    assert rows in (1, 2, 4, 8, 16) and chain.get_launch(zs.Tune.BatchRows) == rows
    assert chain.get_launch(zs.Tune.BatchThreads) in (768, 640)
    chain.batch_thumbnails(*args)
    zs.device_synchronize()
    assert (out.download(np.empty((40, 256, 1024), np.uint8)) == results[0]).all()
